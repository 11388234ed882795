// cloud_raymarch_l1_c78.cu — the cloud raymarch kernel with 1 lane(s) per ray
// (skyr_tuning::cloud_ray_lanes) at the register cuts for 7 and 8 resident
// blocks per SM (skyr_tuning::cloud_blocks_per_sm), in its own translation
// unit so that the raymarch variants compile in parallel.
#include "cloud_march.cuh"

namespace skyr {
template SKYR_CLOUD_CUT_SIGNATURE(1, 7);
template SKYR_CLOUD_CUT_SIGNATURE(1, 8);
}  // namespace skyr
