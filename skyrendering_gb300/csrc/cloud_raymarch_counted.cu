// cloud_raymarch_counted.cu — the instrumented cloud raymarch: one lane per
// ray, the frame's raymarch samples, density evaluations and detail-texture
// evaluations added to counters[0..2].  The production instances keep no
// counters; the frame is the same, bit for bit.
#include "cloud_march.cuh"

namespace skyr {

void launch_cloud_render_counted(bool half, dim3 grid, cudaStream_t stream, const CloudConsts& C,
                                 const MaterialConsts& M, const AtmoConsts& A, const float4* tlut, int tw, int th,
                                 const void* ap_lum, const void* ap_trans, const float* blue_noise,
                                 const float* depth, __half2* out_rgba, float* out_dist,
                                 unsigned long long* counters, int tile_w, int warps_x) {
    auto go = [&](auto tag, auto fast) {
        using S = decltype(tag);
        cloud_render_kernel<S, 5, 1, true, decltype(fast)::value><<<grid, 128, 0, stream>>>(
            C, M, A, tlut, tw, th, reinterpret_cast<const S*>(ap_lum), reinterpret_cast<const S*>(ap_trans),
            blue_noise, depth, out_rgba, out_dist, counters, tile_w, warps_x);
    };
    using Fast = std::true_type;
    using General = std::false_type;
    if (half) {
        if (M.fast_ok) go(__half2{}, Fast{});
        else go(__half2{}, General{});
    } else {
        if (M.fast_ok) go(float4{}, Fast{});
        else go(float4{}, General{});
    }
}

}  // namespace skyr
