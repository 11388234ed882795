// lut_noalloc.cu — skyr_update_lut_set_noalloc: the batched LUT set without
// any device allocation by the library.
//
// skyr_update_lut_set keeps its per-set kernel constants (one LutSetJob per
// parameter set) in a device table that the context allocates with cudaMalloc
// and grows on demand.  Some hosts cannot let a library do that: an engine
// that owns every byte of device memory through its own pool or budget, or a
// frame loop that must not take cudaMalloc/cudaFree (cudaFree synchronises the
// whole device).  For them this variant keeps the table in this module's
// static device memory instead:
//   * capacity SKYR_NOALLOC_MAX_SETS parameter sets (256 x sizeof(LutSetJob),
//     under 100 KB), held by every GPU that loads libskyr until the process
//     exits;
//   * the host learns the table's device address once per device, with that
//     device current, from cudaGetSymbolAddress (the array's name is only a
//     host-side stand-in); the first call on a device does this and should
//     come before any stream capture.  The address is kept for the life of
//     the process, so a cudaDeviceReset while the library is loaded is not
//     supported;
//   * every call validates all of its sets first, then derives their
//     constants on the host and copies them into the table with
//     cudaMemcpyAsync on the context's stream, so a rejected call leaves the
//     table as it was;
//   * every call shares the one table and overwrites the entries it uses, so
//     calls whose GPU work overlaps (two streams or contexts at once) race.
#include <mutex>

#include "atmosphere_kernels.cuh"
#include "skyr_ctx.cuh"

namespace {

constexpr int kNoAllocMaxSets = SKYR_NOALLOC_MAX_SETS;
constexpr int kMaxDevices = 64;
constexpr int kChunk = 16;  // jobs derived per host pass (stack buffer, no heap)

static __device__ __align__(256) LutSetJob g_noalloc_jobs[kNoAllocMaxSets];

std::mutex g_mu;
void* g_jobs_address[kMaxDevices] = {};

// Device address of g_noalloc_jobs on `device` (current); looked up once.
int jobs_address(int device, void** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (device < 0 || device >= kMaxDevices)
        return skyr::set_error(SKYR_ENOTSUP, "device index %d beyond %d", device, kMaxDevices);
    if (!g_jobs_address[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_jobs);
        if (e != cudaSuccess) return skyr::check_cuda(e, "cudaGetSymbolAddress(static LUT job table)");
        g_jobs_address[device] = p;
    }
    *out = g_jobs_address[device];
    return SKYR_OK;
}

template <class S>
int launch_all(skyr_ctx* ctx, const LutSetJob* jobs, int n, const skyr_lut_sizes& s, void* T, void* MS,
               void* svl, void* svt, void* apl, void* apt) {
    skyr::JobSrc<true> src{jobs};
    cudaStream_t st = ctx->stream;
    float4* t = reinterpret_cast<float4*>(T);
    S* ms = reinterpret_cast<S*>(MS);
    if (int e = skyr::check_cuda(skyr::launch_transmittance<true>(src, n, s, t, st, ctx->tuning.transmittance_lanes),
                                 "transmittance kernel"))
        return e;
    if (int e = skyr::check_cuda(skyr::launch_multiscattering<S, true>(src, n, s, t, ms, st), "multiscattering kernel"))
        return e;
    return skyr::check_cuda(skyr::launch_view_luts<S, true>(src, n, s, t, ms, reinterpret_cast<S*>(svl),
                                                            reinterpret_cast<S*>(svt), reinterpret_cast<S*>(apl),
                                                            reinterpret_cast<S*>(apt), st, ctx->tuning.view_lanes),
                            "view LUT kernel");
}

}  // namespace

extern "C" int skyr_update_lut_set_noalloc(skyr_ctx* ctx, const skyr_atmosphere_parameters* params,
                                           const skyr_atmosphere_render_parameters* render, int n_sets,
                                           const skyr_lut_sizes* sizes, void* transmittance,
                                           void* multiscattering, void* sky_view_luminance,
                                           void* sky_view_transmittance, void* aerial_perspective_luminance,
                                           void* aerial_perspective_transmittance) {
    using namespace skyr;
    if (!ctx) return set_error(SKYR_EINVAL, "null context");
    if (!params || !render) return set_error(SKYR_EINVAL, "null parameter blocks");
    if (n_sets < 1 || n_sets > kNoAllocMaxSets)
        return set_error(SKYR_EINVAL, "n_sets %d outside [1, %d], the capacity of the static scratch table", n_sets,
                         kNoAllocMaxSets);
    if (int st = validate_sizes(sizes, true)) return st;
    if (!transmittance || !multiscattering)
        return set_error(SKYR_EINVAL, "null transmittance or multi-scattering buffer");
    // the view outputs as skyr_update_lut_set takes them: each (luminance, transmittance) pair given together or
    // left out together, at least one pair given
    if ((sky_view_luminance == nullptr) != (sky_view_transmittance == nullptr) ||
        (aerial_perspective_luminance == nullptr) != (aerial_perspective_transmittance == nullptr))
        return set_error(SKYR_EINVAL, "luminance and transmittance outputs must be given together");
    if (!sky_view_luminance && !aerial_perspective_luminance) return set_error(SKYR_EINVAL, "no view LUT output given");
    // every set is checked before the first upload, so a rejected call leaves the shared table untouched
    for (int i = 0; i < n_sets; ++i) {
        if (int st = validate_atmosphere(&params[i], i)) return st;
        if (int st = validate_render(&render[i], &params[i], i)) return st;
    }
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    void* table = nullptr;
    if (int st = jobs_address(ctx->device, &table)) return st;
    LutSetJob chunk[kChunk];
    for (int i0 = 0; i0 < n_sets; i0 += kChunk) {
        int k = n_sets - i0 < kChunk ? n_sets - i0 : kChunk;
        for (int j = 0; j < k; ++j) {
            derive_atmo_consts(params[i0 + j], chunk[j].a);
            derive_view_consts(params[i0 + j], render[i0 + j], chunk[j].v);
        }
        // pageable source: the copy is staged before cudaMemcpyAsync returns
        if (int e = check_cuda(cudaMemcpyAsync(reinterpret_cast<LutSetJob*>(table) + i0, chunk,
                                               sizeof(LutSetJob) * k, cudaMemcpyHostToDevice, ctx->stream),
                               "upload of the static LUT job table"))
            return e;
    }
    skyr_lut_sizes s = *sizes;  // a missing view pair launches no texels of that LUT
    if (!sky_view_luminance) s.sky_view_width = s.sky_view_height = 0;
    if (!aerial_perspective_luminance)
        s.aerial_perspective_width = s.aerial_perspective_height = s.aerial_perspective_depth = 0;
    const LutSetJob* jobs = reinterpret_cast<const LutSetJob*>(table);
    if (s.format == SKYR_FORMAT_RGBA16F)
        return launch_all<__half2>(ctx, jobs, n_sets, s, transmittance, multiscattering, sky_view_luminance,
                                   sky_view_transmittance, aerial_perspective_luminance,
                                   aerial_perspective_transmittance);
    return launch_all<float4>(ctx, jobs, n_sets, s, transmittance, multiscattering, sky_view_luminance,
                              sky_view_transmittance, aerial_perspective_luminance, aerial_perspective_transmittance);
}
