// cloud_raymarch_l2_c56.cu — the cloud raymarch kernel with 2 lane(s) per ray
// (skyr_tuning::cloud_ray_lanes) at the register cuts for 5 and 6 resident
// blocks per SM (skyr_tuning::cloud_blocks_per_sm), in its own translation
// unit so that the raymarch variants compile in parallel.
#include "cloud_march.cuh"

namespace skyr {
template SKYR_CLOUD_CUT_SIGNATURE(2, 5);
template SKYR_CLOUD_CUT_SIGNATURE(2, 6);
}  // namespace skyr
