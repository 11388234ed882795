// skyr_ctx.cuh — the opaque context behind skyr_ctx* and internal helpers
// shared by the entry-point translation units.
#pragma once

#include <cuda_runtime.h>

#include "../../include/skyr.h"

struct skyr_ctx {
    cudaStream_t stream = nullptr;
    int device = 0;
    // device table of per-set kernel constants for batched LUT calls
    void* job_table = nullptr;
    size_t job_table_bytes = 0;
    // per-context scratch owned by the cloud / path-tracer / surrogate modules
    void* cloud_scratch = nullptr;
    size_t cloud_scratch_bytes = 0;
    void* pt_scratch = nullptr;
    size_t pt_scratch_bytes = 0;
    int* d_status = nullptr;  // device-side error flags of bounded waits
};

namespace skyr {
int set_error(int code, const char* fmt, ...);
int check_cuda(cudaError_t e, const char* what);
int ensure_job_table(skyr_ctx* ctx, size_t bytes);
// Frees the module-owned scratch of a context (defined in skyr_modules.cu).
void ctx_release_resources(skyr_ctx* ctx);
// Device status word of the context (allocated on first use, zeroed).
int ensure_status(skyr_ctx* ctx);
int ensure_pt_scratch(skyr_ctx* ctx, size_t bytes);
// Argument validation of the LUT entry points (skyr_api.cu).
int validate_atmosphere(const skyr_atmosphere_parameters* p, int i);
int validate_render(const skyr_atmosphere_render_parameters* r, const skyr_atmosphere_parameters* p, int i);
int validate_sizes(const skyr_lut_sizes* s, bool views);
}  // namespace skyr
