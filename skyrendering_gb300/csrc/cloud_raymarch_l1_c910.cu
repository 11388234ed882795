// cloud_raymarch_l1_c910.cu — the cloud raymarch kernel with 1 lane(s) per ray
// (skyr_tuning::cloud_ray_lanes) at the register cuts for 9 and 10 resident
// blocks per SM (skyr_tuning::cloud_blocks_per_sm), in its own translation
// unit so that the raymarch variants compile in parallel.
#include "cloud_march.cuh"

namespace skyr {
template SKYR_CLOUD_CUT_SIGNATURE(1, 9);
template SKYR_CLOUD_CUT_SIGNATURE(1, 10);
}  // namespace skyr
