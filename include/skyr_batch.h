/*
 * skyr_batch.h — many parameter sets and views per call, launch-shape tuning,
 * an autotuner and CUDA-graph capture.  No reference counterpart: the
 * reference regenerates one parameter set per frame on one GL context and
 * picks compute local sizes by hand (src/Base/src/GLReloadableProgram.cpp:43-62).
 * Conventions as in skyr.h.
 */
#ifndef SKYR_BATCH_H_
#define SKYR_BATCH_H_

#include "skyr_cloud.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Launch shapes of the LUT passes and the cloud raymarch (struct id 14); a
 * context starts with the defaults and every later launch on it uses its
 * current values. */
typedef struct skyr_tuning {
    int transmittance_lanes; /* lanes sharing one transmittance texel: 2, 4, 8, 16 */
    int view_lanes;          /* lanes sharing one sky-view / aerial-perspective ray: 2, 4, 8, 16 */
    int cloud_tile_width;    /* pixels across one warp's tile (height 32 / width): 4, 8, 16, 32 */
    int cloud_block_warps_x; /* warps side by side in a 4-warp block: 1, 2, 4 */
    int cloud_blocks_per_sm; /* resident blocks per SM the raymarch's registers are cut for: 5 .. 10 */
    int cloud_ray_lanes;     /* lanes sharing one ray's steps: 1, 2, 4, 8 (a warp's tile is then at most
                                32 / lanes pixels wide) */
} skyr_tuning;

int skyr_tuning_default(skyr_tuning* t);
int skyr_ctx_set_tuning(skyr_ctx* ctx, const skyr_tuning* t); /* SKYR_EINVAL for values outside the lists */
int skyr_ctx_get_tuning(const skyr_ctx* ctx, skyr_tuning* t);

/* Autotuners: time every candidate on the caller's own workload (one warm-up
 * and `reps` launches each, CUDA events on the context's stream; the call
 * synchronises), keep the fastest in the context and return it in *best.
 * times_ms (may be NULL) receives the mean time per candidate:
 *   LUTs:  [0..3] transmittance lanes 2, 4, 8, 16; [4..7] view lanes 2, 4, 8, 16
 *          (the LUT set of skyr_update_lut_set; the outputs are overwritten);
 *   cloud: SKYR_CLOUD_TUNE_CANDIDATES = ray lanes {1, 2, 4, 8} x blocks per SM
 *          {5, 6, 7, 8, 9, 10} x the 12 (tile width, block warps x) pairs (4,1) (4,2) (4,4)
 *          (8,1) (8,2) (8,4) (16,1) (16,2) (16,4) (32,1) (32,2) (32,4), index =
 *          (lanes index * 6 + occupancy index) * 12 + pair index
 *          (skyr_cloud_render's outputs are overwritten). */
#define SKYR_CLOUD_TILE_CANDIDATES 12
#define SKYR_CLOUD_TUNE_CANDIDATES 288
int skyr_autotune_luts(skyr_ctx* ctx, const skyr_atmosphere_parameters* params,
                       const skyr_atmosphere_render_parameters* render, int n_sets, const skyr_lut_sizes* sizes,
                       void* transmittance, void* multiscattering, void* sky_view_luminance,
                       void* sky_view_transmittance, void* aerial_perspective_luminance,
                       void* aerial_perspective_transmittance, int reps, skyr_tuning* best, float* times_ms);
int skyr_autotune_cloud(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                        const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                        const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                        const skyr_lut_sizes* sizes, const void* transmittance,
                        const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                        const float* blue_noise, void* out_rgba, float* out_distance, int reps, skyr_tuning* best,
                        float* times_ms);

/* A prepared batch of LUT sets: the per-set constants are derived and
 * uploaded once at creation, so a launch only enqueues the three batched
 * passes (transmittance, multi-scattering, sky-view + aerial perspective) for
 * all sets -- it allocates, uploads and synchronises nothing and can be
 * captured into a CUDA graph.  Output layout as skyr_update_lut_set. */
typedef struct skyr_lut_batch skyr_lut_batch;
int skyr_lut_batch_create(skyr_ctx* ctx, const skyr_atmosphere_parameters* params,
                          const skyr_atmosphere_render_parameters* render, int n_sets, const skyr_lut_sizes* sizes,
                          skyr_lut_batch** out);
int skyr_lut_batch_launch(skyr_lut_batch* b, void* transmittance, void* multiscattering, void* sky_view_luminance,
                          void* sky_view_transmittance, void* aerial_perspective_luminance,
                          void* aerial_perspective_transmittance);
int skyr_lut_batch_destroy(skyr_lut_batch* b);

/* Cloud raymarch of n_views views (skyr_cloud_render each), view i reading LUT
 * set set_of_view[i] (< n_sets) of batched LUT buffers laid out as
 * skyr_update_lut_set (set s of a buffer starts s * skyr_lut_bytes(...) bytes
 * in) with the atmosphere atmospheres[set_of_view[i]]; outputs per view.  The views are
 * spread over the context's internal streams (forked from and joined back to
 * its stream with events), so a captured graph holds them as parallel branches.
 * Allocates nothing after the first call on a context. */
int skyr_cloud_render_views(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmospheres, int n_sets,
                            const int* set_of_view, const skyr_cloud_parameters* cloud,
                            const skyr_cloud_material* material,
                            const skyr_cloud_textures* textures, const skyr_cloud_view* views, int n_views,
                            const skyr_lut_sizes* sizes, const void* transmittance,
                            const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                            const float* blue_noise, void* const* out_rgba, float* const* out_distance);

/* CUDA graph of the calls made on a context between begin and end (stream
 * capture of the context's stream; calls that allocate, upload from the host
 * or synchronise fail while capturing -- use skyr_lut_batch for many sets). */
typedef struct skyr_graph skyr_graph;
int skyr_graph_begin(skyr_ctx* ctx);
int skyr_graph_end(skyr_ctx* ctx, skyr_graph** out);
int skyr_graph_launch(skyr_graph* g); /* on the context's stream */
int skyr_graph_destroy(skyr_graph* g);

#ifdef __cplusplus
}
#endif
#endif /* SKYR_BATCH_H_ */
