// skyr_modules.cu — lifetime of the per-context scratch buffers.
#include "../../include/skyr_cloud.h"
#include "skyr_ctx.cuh"

namespace skyr {

void ctx_release_resources(skyr_ctx* ctx) {
    if (ctx->cloud_scratch) cudaFree(ctx->cloud_scratch);
    if (ctx->pt_scratch) cudaFree(ctx->pt_scratch);
    if (ctx->d_status) cudaFree(ctx->d_status);
    ctx->cloud_scratch = ctx->pt_scratch = nullptr;
    ctx->d_status = nullptr;
    ctx->cloud_scratch_bytes = ctx->pt_scratch_bytes = 0;
}

}  // namespace skyr

size_t skyr_struct_size_ext(int which) {
    switch (which) {
        case 3: return sizeof(skyr_noise_texture_desc);
        case 4: return sizeof(skyr_cloud_material);
        case 5: return sizeof(skyr_cloud_textures);
        case 6: return sizeof(skyr_cloud_parameters);
        case 7: return sizeof(skyr_cloud_view);
        default: return 0;
    }
}
