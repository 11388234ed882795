// cloud_lanes8.cu — the cloud raymarch kernel with 8 lanes per ray
// (skyr_tuning::cloud_ray_lanes = 8), in its own translation unit so that
// the raymarch variants compile in parallel.
#include "cloud_march.cuh"

namespace skyr {
template void launch_cloud_render<8>(bool, int, dim3, cudaStream_t, const CloudConsts&, const MaterialConsts&,
                                      const AtmoConsts&, const float4*, int, int, const void*, const void*,
                                      const float*, const float*, __half2*, float*, unsigned long long*, int, int);
}  // namespace skyr
