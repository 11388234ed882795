// skyr_modules.cu — lifetime of the per-context scratch buffers.
#include <algorithm>

#include "../../include/skyr_mlp.h"
#include "../../include/skyr_surrogate.h"
#include "../../include/skyr_pathtrace.h"
#include "../../include/skyr_cloud_shadow.h"
#include "../../include/skyr_cloud_quarter.h"
#include "../../include/skyr_composite.h"
#include "skyr_ctx.cuh"

namespace skyr {

void ctx_release_resources(skyr_ctx* ctx) {
    if (ctx->cloud_scratch) cudaFree(ctx->cloud_scratch);
    if (ctx->pt_scratch) cudaFree(ctx->pt_scratch);
    if (ctx->d_status) cudaFree(ctx->d_status);
    ctx->cloud_scratch = ctx->pt_scratch = nullptr;
    ctx->d_status = nullptr;
    ctx->cloud_scratch_bytes = ctx->pt_scratch_bytes = 0;
    for (int k = 0; k < skyr_ctx::kAux; ++k) {
        if (ctx->aux[k]) cudaStreamDestroy(ctx->aux[k]);
        if (ctx->join_event[k]) cudaEventDestroy(ctx->join_event[k]);
        ctx->aux[k] = nullptr;
        ctx->join_event[k] = nullptr;
    }
    if (ctx->fork_event) cudaEventDestroy(ctx->fork_event);
    ctx->fork_event = nullptr;
}

// Grow-only per-context scratch of the path tracer (its per-frame work counters).
int ensure_pt_scratch(skyr_ctx* ctx, size_t bytes) {
    if (ctx->pt_scratch_bytes >= bytes) return SKYR_OK;
    if (ctx->pt_scratch) {
        if (int e = check_cuda(cudaStreamSynchronize(ctx->stream), "synchronize before growing scratch")) return e;
        cudaFree(ctx->pt_scratch);
        ctx->pt_scratch = nullptr;
        ctx->pt_scratch_bytes = 0;
    }
    size_t want = std::max(bytes, (size_t)4096);
    if (int e = check_cuda(cudaMalloc(&ctx->pt_scratch, want), "cudaMalloc(path tracer scratch)")) {
        ctx->pt_scratch = nullptr;
        return e;
    }
    ctx->pt_scratch_bytes = want;
    return SKYR_OK;
}

int ensure_status(skyr_ctx* ctx) {
    if (ctx->d_status) return SKYR_OK;
    cudaError_t e = cudaMalloc(&ctx->d_status, sizeof(int));
    if (e != cudaSuccess) {
        ctx->d_status = nullptr;
        return check_cuda(e, "cudaMalloc(status word)");
    }
    return check_cuda(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream), "clear status word");
}

}  // namespace skyr

extern "C" int skyr_ctx_check_status(skyr_ctx* ctx) {
    using namespace skyr;
    if (!ctx) return set_error(SKYR_EINVAL, "null context");
    if (!ctx->d_status) return SKYR_OK;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    int v = 0;
    if (int e = check_cuda(cudaMemcpyAsync(&v, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream),
                           "read status word"))
        return e;
    if (int e = check_cuda(cudaStreamSynchronize(ctx->stream), "synchronize")) return e;
    if (v == 0) return SKYR_OK;
    if (int e = check_cuda(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream), "clear status word")) return e;
    return set_error(SKYR_ETIMEOUT, "a device loop hit its iteration bound (status 0x%x)", v);
}

extern "C" int skyr_device_limits_default(skyr_device_limits* out) {
    using namespace skyr;
    if (!out) return set_error(SKYR_EINVAL, "null skyr_device_limits");
    *out = skyr_ctx{}.limits;
    return SKYR_OK;
}

extern "C" int skyr_ctx_set_limits(skyr_ctx* ctx, const skyr_device_limits* limits) {
    using namespace skyr;
    if (!ctx || !limits) return set_error(SKYR_EINVAL, "null argument");
    if (limits->tracking_steps < 1 || limits->tracking_steps > (1 << 30))
        return set_error(SKYR_EINVAL, "tracking_steps %d outside [1, 2^30]", limits->tracking_steps);
    if (limits->copy_wait_cycles < 0 || limits->copy_wait_cycles > (1ll << 40))
        return set_error(SKYR_EINVAL, "copy_wait_cycles %lld outside [0, 2^40]", (long long)limits->copy_wait_cycles);
    if (limits->reserved != 0) return set_error(SKYR_EINVAL, "reserved field must be 0");
    ctx->limits = *limits;
    return SKYR_OK;
}

extern "C" int skyr_ctx_get_limits(const skyr_ctx* ctx, skyr_device_limits* out) {
    using namespace skyr;
    if (!ctx || !out) return set_error(SKYR_EINVAL, "null argument");
    *out = ctx->limits;
    return SKYR_OK;
}

size_t skyr_struct_size_ext(int which) {
    switch (which) {
        case 3: return sizeof(skyr_noise_texture_desc);
        case 4: return sizeof(skyr_cloud_material);
        case 5: return sizeof(skyr_cloud_textures);
        case 6: return sizeof(skyr_cloud_parameters);
        case 7: return sizeof(skyr_cloud_view);
        case 8: return sizeof(skyr_density_grid);
        case 9: return sizeof(skyr_grid_generator);
        case 10: return sizeof(skyr_pathtrace_parameters);
        case 11: return sizeof(skyr_mlp_hparams);
        case 12: return sizeof(skyr_feature_volume);
        case 13: return sizeof(skyr_surrogate_parameters);
        case 14: return sizeof(skyr_tuning);
        case 15: return sizeof(skyr_cloud_shadow_sizes);
        case 16: return sizeof(skyr_cloud_light_frame);
        case 17: return sizeof(skyr_cloud_temporal_frame);
        case 18: return sizeof(skyr_cloud_quarter_buffers);
        case 19: return sizeof(skyr_composite_parameters);
        case 20: return sizeof(skyr_composite_inputs);
        case 21: return sizeof(skyr_device_limits);
        default: return 0;
    }
}
