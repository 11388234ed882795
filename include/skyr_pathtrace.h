/*
 * skyr_pathtrace.h — C ABI of the volumetric-cloud path tracer
 * (shaders/SkyRendering/VolumetricCloudPathTracing.comp), its dense FP16
 * density grid and the brick majorant grid.  Conventions as in skyr.h.
 *
 * Density grid layout: nx x ny x nz half-precision values, x fastest
 * ((z * ny + y) * nx + x), z is the local "up" axis of the cloud frame; the
 * extinction at a voxel is `density * value`.  Sampling is trilinear between
 * voxel centres with a zero border (the reference's voxel sampler uses
 * CLAMP_TO_BORDER with border 0, VolumetricCloudVoxelMaterial.cpp:25-31).
 */
#ifndef SKYR_PATHTRACE_H_
#define SKYR_PATHTRACE_H_

#include "skyr_cloud.h"

#ifdef __cplusplus
extern "C" {
#endif

/* PathTracing::PRNG and ::EnvironmentLighting (src/SkyRendering/VolumetricCloud.h:92-102) */
#define SKYR_PRNG_WANG_HASH 0
#define SKYR_PRNG_PCG_HASH 1
#define SKYR_ENV_OFF 0
#define SKYR_ENV_CONST_ENVIRONMENT_MAP 1
#define SKYR_ENV_GROUND_SINGLE_BOUNCE 2
#define SKYR_ENV_GROUND_MULTI_BOUNCE 3

/* Dense density grid placed in the local cloud frame (km). */
typedef struct skyr_density_grid {
    const void* data; /* half[nx*ny*nz] */
    int nx, ny, nz;
    float origin[3];  /* local position of the grid's minimum corner */
    float voxel_size; /* edge of one voxel */
    float density;    /* extinction scale (1/km) */
    const float* majorant; /* per-brick max extinction (skyr_grid_majorants), or NULL */
    int brick;             /* brick edge in voxels (16) */
} skyr_density_grid;

/* Synthetic cloud grid: 4-octave Worley fBm (NoiseGen.comp WorleyFBM, remap
 * 1 -> 0) inside an ellipsoid with a soft edge.  value = clamp(worley *
 * envelope - threshold, 0, 1) / (1 - threshold), envelope = 1 - smoothstep(
 * inner, 1, |(p - c) / radii|), p the voxel centre in [0, 1]^3 grid units. */
typedef struct skyr_grid_generator {
    int nx, ny, nz;
    int seed;
    int base_frequency;
    int octaves;
    float center[3];
    float radii[3];
    float inner; /* envelope edge start (fraction of the radii) */
    float threshold;
} skyr_grid_generator;

/* PathTracing::InitParam (src/SkyRendering/VolumetricCloud.h:104-114) plus
 * the material's GetSigmaTMax (kSigmaTMax, VolumetricCloud.cpp:506). */
typedef struct skyr_pathtrace_parameters {
    int max_bounces;
    float region_box_half_width; /* kCloudHalfWidth: the flat AABB [-w, w]^2 x [bottom, top] */
    int importance_sampling;
    float forward_phase_g, back_phase_g, forward_scattering_ratio;
    int prng;                 /* SKYR_PRNG_* */
    int environment_lighting; /* SKYR_ENV_* */
    float sigma_t_max;        /* global majorant when the grid has no brick majorants */
    int use_brick_majorants;  /* delta / ratio tracking against the grid's brick majorants */
} skyr_pathtrace_parameters;

int skyr_pathtrace_parameters_default(skyr_pathtrace_parameters* p);

size_t skyr_grid_bytes(int nx, int ny, int nz);
/* Fill a device half grid of g->nx x g->ny x g->nz. */
int skyr_grid_generate(skyr_ctx* ctx, const skyr_grid_generator* g, void* out);
/* Number of bricks of edge `brick` covering an n-voxel axis: ceil(n / brick). */
int skyr_grid_brick_count(int n, int brick);
/* Per-brick maximum extinction (density * max value over the brick and a
 * one-voxel apron, so that it bounds the trilinear interpolant inside the
 * brick) into device floats [bz][by][bx]. */
int skyr_grid_majorants(skyr_ctx* ctx, const skyr_density_grid* grid, float* out);

/* VolumetricCloud::PathTracing::Render (src/SkyRendering/VolumetricCloud.cpp:533-569)
 * for `n_frames` progressive frames starting at frame id `frame_begin`
 * (kFrameId; the reference's first frame is 1) over the pixel region
 * [region[0], region[2]) x [region[1], region[3]) (NULL = whole view):
 * accumulates the per-frame results (rgb luminance, a = 1 when the path never
 * scattered) into `accumulation` (device float4 per pixel of the view, +=)
 * and, when `accumulation_sq` is not NULL, their squares into it (+=; for
 * variance estimates).  The frames of one call are added in no fixed order
 * (float atomics): sums agree to rounding, not bit for bit, between runs.
 * The density comes from `grid` (dense FP16, may be NULL) else from
 * `material` / `textures` (the reference's material plug-ins).  The
 * environment is the sky-view LUT lookup plus ground term of the
 * ENVIRONMENT_LUMINANCE program (AtmosphereRenderer.glsl:250-273) for the
 * atmosphere view `env_view` (its camera and sun), evaluated per direction. */
int skyr_pathtrace(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                   const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                   const skyr_cloud_textures* textures, const skyr_density_grid* grid,
                   const skyr_pathtrace_parameters* pt, const skyr_cloud_view* view,
                   const skyr_atmosphere_render_parameters* env_view, const skyr_lut_sizes* sizes,
                   const void* transmittance, const void* sky_view_luminance, const void* sky_view_transmittance,
                   const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                   unsigned frame_begin, int n_frames, const int* region, float* accumulation,
                   float* accumulation_sq);

/* skyr_pathtrace over a list of pixels (y * width + x, device ints; entries
 * outside the view are skipped) instead of a rectangle: the fallback of the
 * surrogate renderer path-traces only the pixels it flags.  No reference
 * counterpart. */
int skyr_pathtrace_pixels(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                          const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                          const skyr_cloud_textures* textures, const skyr_density_grid* grid,
                          const skyr_pathtrace_parameters* pt, const skyr_cloud_view* view,
                          const skyr_atmosphere_render_parameters* env_view, const skyr_lut_sizes* sizes,
                          const void* transmittance, const void* sky_view_luminance,
                          const void* sky_view_transmittance, const void* aerial_perspective_luminance,
                          const void* aerial_perspective_transmittance, unsigned frame_begin, int n_frames,
                          const int* pixels, int n_pixels, float* accumulation, float* accumulation_sq);

/* In-scattered radiance at points of a density grid, beyond single scattering
 * of the sun: for each point i (device float[6]: local position p, unit
 * direction w) `n_paths` paths start at p in a direction drawn from the phase
 * function about w -- as if a path travelling along w had just scattered at p,
 * that event being the first of max_bounces -- and continue as in
 * skyr_pathtrace (next-event estimation at later scattering events, the
 * environment on escape).  Their radiance is added to out[i] (device float[3],
 * +=); divided by n_paths it estimates the order >= 2 in-scattered radiance at
 * p toward -w.  Frame ids frame_begin.. seed the paths.  No reference
 * counterpart: the training targets of the multiple-scattering surrogate. */
int skyr_pathtrace_points(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                          const skyr_cloud_parameters* cloud, const skyr_density_grid* grid,
                          const skyr_pathtrace_parameters* pt, const skyr_cloud_view* view,
                          const skyr_atmosphere_render_parameters* env_view, const skyr_lut_sizes* sizes,
                          const void* transmittance, const void* sky_view_luminance,
                          const void* sky_view_transmittance, const void* aerial_perspective_luminance,
                          const void* aerial_perspective_transmittance, unsigned frame_begin, int n_paths,
                          const float* points, int n_points, float* out);

/* The display pass (VolumetricCloudPathTracing.comp:288-296): for every pixel
 * out = background * (acc.a / frames) + acc.rgb / frames, half4 output; the
 * background may be NULL (black). */
int skyr_pathtrace_resolve(skyr_ctx* ctx, const float* accumulation, int width, int height, unsigned frames,
                           const void* background_rgba16f, void* out_rgba16f);

#ifdef __cplusplus
}
#endif
#endif /* SKYR_PATHTRACE_H_ */
