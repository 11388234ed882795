// batch.cu — include/skyr_batch.h: launch-shape tuning and its autotuners,
// prepared LUT batches, multi-view raymarches fanned out over internal
// streams, and CUDA-graph capture of a context's calls.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/skyr_batch.h"
#include "../../include/skyr_cloud_quarter.h"
#include "skyr_ctx.cuh"
#include "skyr_internal.cuh"

struct skyr_lut_batch {
    skyr_ctx* ctx = nullptr;
    LutSetJob* table = nullptr;  // device
    int n = 0;
    skyr_lut_sizes sizes{};
    bool views = false;
};

struct skyr_graph {
    skyr_ctx* ctx = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace skyr {

int ensure_aux_streams(skyr_ctx* ctx) {
    if (ctx->fork_event) return SKYR_OK;
    for (int k = 0; k < skyr_ctx::kAux; ++k) {
        if (int e = check_cuda(cudaStreamCreateWithFlags(&ctx->aux[k], cudaStreamNonBlocking), "create stream"))
            return e;
        if (int e = check_cuda(cudaEventCreateWithFlags(&ctx->join_event[k], cudaEventDisableTiming), "create event"))
            return e;
    }
    return check_cuda(cudaEventCreateWithFlags(&ctx->fork_event, cudaEventDisableTiming), "create event");
}

}  // namespace skyr

using namespace skyr;

namespace {

constexpr int kTileCandidates[SKYR_CLOUD_TILE_CANDIDATES][2] = {
    {4, 1}, {4, 2}, {4, 4}, {8, 1}, {8, 2}, {8, 4}, {16, 1}, {16, 2}, {16, 4}, {32, 1}, {32, 2}, {32, 4}};
constexpr int kLaneCandidates[4] = {2, 4, 8, 16};
constexpr int kLanes = 4;

constexpr int kOccupancyCandidates[6] = {5, 6, 7, 8, 9, 10};
constexpr int kOccupancies = 6;
constexpr int kRayLaneCandidates[4] = {1, 2, 4, 8};

bool valid_lanes(int l) { return l == 2 || l == 4 || l == 8 || l == 16; }
bool valid_tile(int w, int bx) { return (w == 4 || w == 8 || w == 16 || w == 32) && (bx == 1 || bx == 2 || bx == 4); }

// Mean GPU time of fn() over `reps` launches after one warm-up (events on the
// context's stream); fn returns a status.
template <class F>
int time_launches(skyr_ctx* ctx, int reps, F&& fn, float* ms) {
    if (int e = fn()) return e;
    cudaEvent_t a = nullptr, b = nullptr;
    int st = check_cuda(cudaEventCreate(&a), "create event");
    if (!st) st = check_cuda(cudaEventCreate(&b), "create event");
    if (!st) st = check_cuda(cudaEventRecord(a, ctx->stream), "record event");
    for (int i = 0; !st && i < reps; ++i) st = fn();
    if (!st) st = check_cuda(cudaEventRecord(b, ctx->stream), "record event");
    if (!st) st = check_cuda(cudaEventSynchronize(b), "synchronize event");
    float t = 0.f;
    if (!st) st = check_cuda(cudaEventElapsedTime(&t, a, b), "elapsed time");
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (!st) *ms = t / (float)reps;
    return st;
}

// Times `run` for every cloud candidate (ray lanes x blocks per SM x tile
// shapes, the order of skyr_autotune_cloud's times) and keeps the fastest.
static_assert(SKYR_CLOUD_TUNE_CANDIDATES == 4 * kOccupancies * SKYR_CLOUD_TILE_CANDIDATES, "cloud candidate table");

template <class F>
int autotune_cloud_candidates(skyr_ctx* ctx, int reps, skyr_tuning* best, float* times_ms, F&& run) {
    if (!ctx || !best) return set_error(SKYR_EINVAL, "null argument");
    if (reps < 1 || reps > 1000) return set_error(SKYR_EINVAL, "reps must be in [1, 1000]");
    const skyr_tuning start = ctx->tuning;
    float tt[SKYR_CLOUD_TUNE_CANDIDATES] = {};
    int best_i = -1, st = SKYR_OK;
    auto apply = [&](int i) {
        const int* tile = kTileCandidates[i % SKYR_CLOUD_TILE_CANDIDATES];
        ctx->tuning.cloud_tile_width = tile[0];
        ctx->tuning.cloud_block_warps_x = tile[1];
        ctx->tuning.cloud_blocks_per_sm = kOccupancyCandidates[(i / SKYR_CLOUD_TILE_CANDIDATES) % kOccupancies];
        ctx->tuning.cloud_ray_lanes = kRayLaneCandidates[i / (kOccupancies * SKYR_CLOUD_TILE_CANDIDATES)];
    };
    for (int i = 0; i < SKYR_CLOUD_TUNE_CANDIDATES && !st; ++i) {
        apply(i);
        st = time_launches(ctx, reps, run, &tt[i]);
        if (!st && (best_i < 0 || tt[i] < tt[best_i])) best_i = i;
    }
    ctx->tuning = start;
    if (st) return st;
    apply(best_i);
    if (times_ms) std::memcpy(times_ms, tt, sizeof(tt));
    *best = ctx->tuning;
    return SKYR_OK;
}

}  // namespace

extern "C" {

int skyr_tuning_default(skyr_tuning* t) {
    if (!t) return set_error(SKYR_EINVAL, "null tuning");
    *t = skyr_tuning{8, 8, 8, 2, 5, 1};
    return SKYR_OK;
}

int skyr_ctx_set_tuning(skyr_ctx* ctx, const skyr_tuning* t) {
    if (!ctx || !t) return set_error(SKYR_EINVAL, "null argument");
    if (!valid_lanes(t->transmittance_lanes) || !valid_lanes(t->view_lanes))
        return set_error(SKYR_EINVAL, "lanes must be 2, 4, 8 or 16");
    if (!valid_tile(t->cloud_tile_width, t->cloud_block_warps_x))
        return set_error(SKYR_EINVAL, "cloud tile width must be 4, 8, 16 or 32 and block warps 1, 2 or 4");
    if (t->cloud_blocks_per_sm < 5 || t->cloud_blocks_per_sm > 10)
        return set_error(SKYR_EINVAL, "cloud blocks per SM must be 5 .. 10");
    if (t->cloud_ray_lanes != 1 && t->cloud_ray_lanes != 2 && t->cloud_ray_lanes != 4 && t->cloud_ray_lanes != 8)
        return set_error(SKYR_EINVAL, "cloud ray lanes must be 1, 2, 4 or 8");
    ctx->tuning = *t;
    return SKYR_OK;
}

int skyr_ctx_get_tuning(const skyr_ctx* ctx, skyr_tuning* t) {
    if (!ctx || !t) return set_error(SKYR_EINVAL, "null argument");
    *t = ctx->tuning;
    return SKYR_OK;
}

int skyr_lut_batch_create(skyr_ctx* ctx, const skyr_atmosphere_parameters* params,
                          const skyr_atmosphere_render_parameters* render, int n_sets, const skyr_lut_sizes* sizes,
                          skyr_lut_batch** out) {
    if (!ctx || !params || !sizes || !out) return set_error(SKYR_EINVAL, "null argument");
    *out = nullptr;
    if (n_sets < 1 || n_sets > (1 << 16)) return set_error(SKYR_EINVAL, "n_sets must be in [1, 65536]");
    if (int e = validate_sizes(sizes, render != nullptr)) return e;
    std::vector<LutSetJob> jobs(n_sets);
    if (int e = derive_jobs(params, render, n_sets, jobs.data())) return e;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    auto* b = new (std::nothrow) skyr_lut_batch;
    if (!b) return set_error(SKYR_ENOMEM, "out of host memory");
    b->ctx = ctx;
    b->n = n_sets;
    b->sizes = *sizes;
    b->views = render != nullptr;
    const size_t bytes = sizeof(LutSetJob) * n_sets;
    int e = check_cuda(cudaMalloc(&b->table, bytes), "cudaMalloc(LUT batch table)");
    if (!e) e = check_cuda(cudaMemcpyAsync(b->table, jobs.data(), bytes, cudaMemcpyHostToDevice, ctx->stream),
                           "upload LUT batch table");
    if (!e) e = check_cuda(cudaStreamSynchronize(ctx->stream), "synchronize");  // `jobs` goes out of scope
    if (e) {
        skyr_lut_batch_destroy(b);
        return e;
    }
    *out = b;
    return SKYR_OK;
}

int skyr_lut_batch_launch(skyr_lut_batch* b, void* transmittance, void* multiscattering, void* sky_view_luminance,
                          void* sky_view_transmittance, void* aerial_perspective_luminance,
                          void* aerial_perspective_transmittance) {
    if (!b) return set_error(SKYR_EINVAL, "null batch");
    if (!transmittance || !multiscattering) return set_error(SKYR_EINVAL, "null transmittance or multi-scattering buffer");
    bool sv = sky_view_luminance && sky_view_transmittance, ap = aerial_perspective_luminance &&
                                                               aerial_perspective_transmittance;
    if ((sky_view_luminance == nullptr) != (sky_view_transmittance == nullptr) ||
        (aerial_perspective_luminance == nullptr) != (aerial_perspective_transmittance == nullptr))
        return set_error(SKYR_EINVAL, "luminance and transmittance outputs must be given together");
    if ((sv || ap) && !b->views) return set_error(SKYR_EINVAL, "the batch was created without render parameters");
    if (int e = check_cuda(cudaSetDevice(b->ctx->device), "cudaSetDevice")) return e;
    return launch_lut_passes(b->ctx, b->table, b->n, b->sizes, sv || ap, transmittance, multiscattering,
                             sky_view_luminance, sky_view_transmittance, aerial_perspective_luminance,
                             aerial_perspective_transmittance);
}

int skyr_lut_batch_destroy(skyr_lut_batch* b) {
    if (!b) return SKYR_OK;
    if (b->table) {
        cudaSetDevice(b->ctx->device);
        cudaStreamSynchronize(b->ctx->stream);
        cudaFree(b->table);
    }
    delete b;
    return SKYR_OK;
}

int skyr_cloud_render_views(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmospheres, int n_sets,
                            const int* set_of_view, const skyr_cloud_parameters* cloud,
                            const skyr_cloud_material* material,
                            const skyr_cloud_textures* textures, const skyr_cloud_view* views, int n_views,
                            const skyr_lut_sizes* sizes, const void* transmittance,
                            const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                            const float* blue_noise, void* const* out_rgba, float* const* out_distance) {
    if (!ctx || !atmospheres || !set_of_view || !views || !sizes || !out_rgba || !out_distance)
        return set_error(SKYR_EINVAL, "null argument");
    if (n_views < 0) return set_error(SKYR_EINVAL, "negative view count");
    if (n_views == 0) return SKYR_OK;
    for (int i = 0; i < n_views; ++i)
        if (set_of_view[i] < 0 || set_of_view[i] >= n_sets)
            return set_error(SKYR_EINVAL, "view %d: LUT set index %d outside [0, %d)", i, set_of_view[i], n_sets);
    const size_t tb = skyr_lut_bytes(sizes, SKYR_LUT_TRANSMITTANCE), ab = skyr_lut_bytes(sizes, SKYR_LUT_AERIAL_PERSPECTIVE);
    if (tb == 0 || ab == 0) return set_error(SKYR_EINVAL, "bad LUT sizes");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    if (int e = ensure_aux_streams(ctx)) return e;
    if (int e = check_cuda(cudaEventRecord(ctx->fork_event, ctx->stream), "fork")) return e;
    const int k_used = std::min(n_views, (int)skyr_ctx::kAux);
    for (int k = 0; k < k_used; ++k)
        if (int e = check_cuda(cudaStreamWaitEvent(ctx->aux[k], ctx->fork_event, 0), "fork")) return e;
    int st = SKYR_OK;
    for (int i = 0; i < n_views && !st; ++i) {
        size_t s = (size_t)set_of_view[i];
        st = cloud_render_on(ctx, ctx->aux[i % k_used], &atmospheres[s], cloud, material, textures, &views[i], sizes,
                             static_cast<const char*>(transmittance) + s * tb,
                             static_cast<const char*>(aerial_perspective_luminance) + s * ab,
                             static_cast<const char*>(aerial_perspective_transmittance) + s * ab, blue_noise,
                             nullptr, out_rgba[i], out_distance[i], nullptr);
        if (st) {
            char msg[256];
            std::snprintf(msg, sizeof(msg), "%s", skyr_last_error());
            st = set_error(st, "view %d: %s", i, msg);
        }
    }
    // join every forked stream back, also after an error, so nothing is left dangling
    for (int k = 0; k < k_used; ++k) {
        int e = check_cuda(cudaEventRecord(ctx->join_event[k], ctx->aux[k]), "join");
        if (!e) e = check_cuda(cudaStreamWaitEvent(ctx->stream, ctx->join_event[k], 0), "join");
        if (!st) st = e;
    }
    return st;
}

int skyr_autotune_luts(skyr_ctx* ctx, const skyr_atmosphere_parameters* params,
                       const skyr_atmosphere_render_parameters* render, int n_sets, const skyr_lut_sizes* sizes,
                       void* transmittance, void* multiscattering, void* sky_view_luminance,
                       void* sky_view_transmittance, void* aerial_perspective_luminance,
                       void* aerial_perspective_transmittance, int reps, skyr_tuning* best, float* times_ms) {
    if (!ctx || !best) return set_error(SKYR_EINVAL, "null argument");
    if (reps < 1 || reps > 1000) return set_error(SKYR_EINVAL, "reps must be in [1, 1000]");
    skyr_lut_batch* b = nullptr;
    if (int e = skyr_lut_batch_create(ctx, params, render, n_sets, sizes, &b)) return e;
    skyr_tuning t = ctx->tuning;
    auto run = [&]() {
        return skyr_lut_batch_launch(b, transmittance, multiscattering, sky_view_luminance, sky_view_transmittance,
                                     aerial_perspective_luminance, aerial_perspective_transmittance);
    };
    int st = SKYR_OK;
    float tt[2 * kLanes] = {};
    for (int pass = 0; pass < 2 && !st; ++pass) {
        int best_i = 0;
        for (int i = 0; i < kLanes && !st; ++i) {
            (pass == 0 ? ctx->tuning.transmittance_lanes : ctx->tuning.view_lanes) = kLaneCandidates[i];
            st = time_launches(ctx, reps, run, &tt[pass * kLanes + i]);
            if (!st && tt[pass * kLanes + i] < tt[pass * kLanes + best_i]) best_i = i;
        }
        if (!st) (pass == 0 ? t.transmittance_lanes : t.view_lanes) = kLaneCandidates[best_i];
        ctx->tuning = t;
    }
    skyr_lut_batch_destroy(b);
    if (st) return st;
    if (times_ms) std::memcpy(times_ms, tt, sizeof(tt));
    *best = ctx->tuning;
    return SKYR_OK;
}

int skyr_autotune_cloud(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                        const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                        const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                        const skyr_lut_sizes* sizes, const void* transmittance,
                        const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                        const float* blue_noise, void* out_rgba, float* out_distance, int reps, skyr_tuning* best,
                        float* times_ms) {
    return autotune_cloud_candidates(ctx, reps, best, times_ms, [&]() {
        return cloud_render_on(ctx, ctx->stream, atmosphere, cloud, material, textures, view, sizes, transmittance,
                               aerial_perspective_luminance, aerial_perspective_transmittance, blue_noise, nullptr,
                               out_rgba, out_distance, nullptr);
    });
}

int skyr_autotune_cloud_quarter(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                                const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                                const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                                const skyr_lut_sizes* sizes, const void* transmittance,
                                const void* aerial_perspective_luminance,
                                const void* aerial_perspective_transmittance, const float* blue_noise,
                                const float* depth, const skyr_cloud_temporal_frame* frame,
                                const skyr_cloud_quarter_buffers* buffers, int reps, skyr_tuning* best,
                                float* times_ms) {
    return autotune_cloud_candidates(ctx, reps, best, times_ms, [&]() {
        return skyr_cloud_render_quarter(ctx, atmosphere, cloud, material, textures, view, sizes, transmittance,
                                         aerial_perspective_luminance, aerial_perspective_transmittance, blue_noise,
                                         depth, frame, buffers, nullptr);
    });
}

int skyr_graph_begin(skyr_ctx* ctx) {
    if (!ctx) return set_error(SKYR_EINVAL, "null context");
    if (!ctx->stream) return set_error(SKYR_EINVAL, "graph capture needs a context on a created (non-default) stream");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    return check_cuda(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
}

int skyr_graph_end(skyr_ctx* ctx, skyr_graph** out) {
    if (!ctx || !out) return set_error(SKYR_EINVAL, "null argument");
    *out = nullptr;
    cudaGraph_t g = nullptr;
    if (int e = check_cuda(cudaStreamEndCapture(ctx->stream, &g), "end capture")) return e;
    cudaGraphExec_t x = nullptr;
    if (int e = check_cuda(cudaGraphInstantiate(&x, g, 0), "instantiate graph")) {
        cudaGraphDestroy(g);
        return e;
    }
    auto* gr = new (std::nothrow) skyr_graph;
    if (!gr) {
        cudaGraphExecDestroy(x);
        cudaGraphDestroy(g);
        return set_error(SKYR_ENOMEM, "out of host memory");
    }
    gr->ctx = ctx;
    gr->graph = g;
    gr->exec = x;
    *out = gr;
    return SKYR_OK;
}

int skyr_graph_launch(skyr_graph* g) {
    if (!g) return set_error(SKYR_EINVAL, "null graph");
    if (int e = check_cuda(cudaSetDevice(g->ctx->device), "cudaSetDevice")) return e;
    return check_cuda(cudaGraphLaunch(g->exec, g->ctx->stream), "graph launch");
}

int skyr_graph_destroy(skyr_graph* g) {
    if (!g) return SKYR_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return SKYR_OK;
}

}  // extern "C"
