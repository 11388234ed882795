// skyr_ctx.cuh — the opaque context behind skyr_ctx* and internal helpers
// shared by the entry-point translation units.
#pragma once

#include <cuda_runtime.h>

#include "../../include/skyr.h"
#include "../../include/skyr_batch.h"

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
    // bounds of the device loops (skyr_ctx_set_limits)
    skyr_device_limits limits{1 << 20, 0, 1ll << 31};
    // launch shapes (skyr_batch.h)
    skyr_tuning tuning{8, 8, 8, 2, 5, 1};
    // internal streams and events that fan a call's independent launches out
    // from the context's stream and join them back (created on first use)
    static constexpr int kAux = 4;
    cudaStream_t aux[kAux] = {};
    cudaEvent_t fork_event = nullptr;
    cudaEvent_t join_event[kAux] = {};
};

struct LutSetJob;  // per-set kernel constants (skyr_internal.cuh)

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
// Validate and derive the per-set kernel constants of n LUT sets (no upload).
int derive_jobs(const skyr_atmosphere_parameters* params, const skyr_atmosphere_render_parameters* rp, int n,
                LutSetJob* jobs);
// Enqueue the LUT passes for n sets whose constants are in a device table
// (the context's tuning picks the lanes); the outputs as skyr_update_lut_set.
int launch_lut_passes(skyr_ctx* ctx, const LutSetJob* table, int n, const skyr_lut_sizes& s, bool do_view, void* T,
                      void* MS, void* svl, void* svt, void* apl, void* apt);
// Cloud raymarch of one view on `stream` (cloud.cu); the launch shape from the
// context's tuning.  `mode`: kCloudCheckOnly validates the arguments and
// derives the launch constants without launching; kCloudAfterLuts launches the
// full-resolution raymarch as a programmatic dependent of the view-LUT pass
// that the stream ran just before it (skyr_render_frame).
constexpr int kCloudCheckOnly = 1;
constexpr int kCloudAfterLuts = 2;
int cloud_render_on(skyr_ctx* ctx, cudaStream_t stream, const skyr_atmosphere_parameters* atmosphere,
                    const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                    const skyr_cloud_textures* textures, const skyr_cloud_view* view, const skyr_lut_sizes* sizes,
                    const void* transmittance, const void* aerial_perspective_luminance,
                    const void* aerial_perspective_transmittance, const float* blue_noise, const float* depth,
                    void* out_rgba, float* out_distance, unsigned long long* counters,
                    const struct CloudCheckerboard* checkerboard = nullptr, int mode = 0);
// Create the internal streams / events of a context if needed.
int ensure_aux_streams(skyr_ctx* ctx);
}  // namespace skyr
