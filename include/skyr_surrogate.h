/*
 * skyr_surrogate.h — C ABI of the surrogate-shaded voxel cloud: a 128-step
 * raymarch through the dense density grid in which single scattering of the
 * sun is computed and order >= 2 in-scattered radiance comes from the network
 * of skyr_mlp.h, evaluated inside the march.  No counterpart in the reference
 * (it stands in for the multiple-scattering heuristic of
 * VolumetricCloudRender.comp:125-130, and for the path tracer of
 * VolumetricCloudPathTracing.comp when an image is wanted fast).
 * Conventions as in skyr.h; positions in the local cloud frame of skyr_cloud.h.
 *
 * Network inputs (one feature record, SKYR_MLP_RECORD bf16):
 *   0       extinction at the point / sigma_ref
 *   1..32   extinction at the point + d_k * sun, d_k = span * 0.01 * 1000^(k/31)
 *   33..40  extinction at the 8 corners of a cube around the point whose
 *           corners lie 0.1 * span away, with axes (v, u, w): v the view
 *           direction, u the sun's component perpendicular to v, w = v x u;
 *           corner j is +-1/sqrt(3) along v, u, w by bits 0, 1, 2 of j
 *   41      height of the point within the grid box, 0 (bottom) .. 1 (top)
 *   42      cos(view direction, sun direction)
 *   43      transmittance from the point along the view direction to where the
 *           view ray leaves the volume (training points: a midpoint march at
 *           half-voxel steps to the grid box's exit; the raymarch: what remains
 *           of the ray's optical depth at its own samples past the point)
 *   44..78  the density stencil: mean extinction / sigma_ref from mip levels
 *           l = 2..6 of the grid (level l averages 2^l-voxel cubes), at the
 *           point and +-2^(l+1) voxels along the sun, the sun's horizontal
 *           perpendicular (sun x z; sun x x with the sun at the zenith) and
 *           their cross product; feature 44 + 7 (l - 2) + j, j = 0 the centre,
 *           j = 1, 2 +- the sun axis, 3, 4 the second axis, 5, 6 the third
 *   79..102 the view-oriented stencil: mean extinction / sigma_ref from mip
 *           levels l = 3..6 at +-2^(l+1) voxels along v, u and w (the frame of
 *           33..40); feature 79 + 6 (l - 3) + j, j = 0, 1 +-v, 2, 3 +-u, 4, 5 +-w
 *   103..111 zero
 * span = the grid's longest edge; extinctions are divided by sigma_ref.
 * Features 0..32, 41 and 44..78 depend on the position only: they are taken at
 * the nodes of a coarse lattice (every `stride` voxels, 80 bf16 per node
 * holding features 0..79, the per-sample slots zero) and interpolated
 * trilinearly; 33..40, 42, 43 and 79..102 are computed per sample.  Both are
 * done the same way for training points and for the raymarch.  Features 0..42
 * are the configured inputs; 43..102 (the view ray's far side and the two
 * stencils) cut the network's error against path-traced labels by more than
 * half.
 */
#ifndef SKYR_SURROGATE_H_
#define SKYR_SURROGATE_H_

#include "skyr_mlp.h"
#include "skyr_pathtrace.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Feature lattice of one (grid, sun direction) pair (struct id 12). */
typedef struct skyr_feature_volume {
    void* data;        /* device: node records [nodes][80] bf16, sun optical depth [nodes] f32, then
                        * the grid's mip levels 1..6 (FP16, each 256-byte aligned) */
    int stride;        /* voxels between lattice nodes */
    int nx, ny, nz;    /* nodes per axis: (grid n + stride - 1) / stride + 1 */
    float sigma_ref;   /* extinctions are divided by this */
    float sun[3];      /* local sun direction the lattice was built for */
} skyr_feature_volume;

/* Raymarch settings (struct id 13). */
typedef struct skyr_surrogate_parameters {
    int steps;              /* uniform steps through the grid box (128) */
    int use_network;        /* 0: single scattering only (the ablation) */
    float network_error;    /* relative error of the network when error_table is NULL */
    float min_transmittance;/* a ray ends below this view transmittance (1e-4) */
    /* Optional device float[SKYR_SURROGATE_ERROR_BINS^2]: relative error of the
     * network by (feature 0, mean of features 1..8) bins over [0, 1]^2, row =
     * feature-0 bin (calibrated on validation points); NULL: network_error. */
    const float* error_table;
} skyr_surrogate_parameters;

#define SKYR_SURROGATE_ERROR_BINS 8

int skyr_surrogate_parameters_default(skyr_surrogate_parameters* p);

/* Device bytes of the lattice for `grid` at `stride`; fills the node counts. */
size_t skyr_feature_volume_bytes(const skyr_density_grid* grid, int stride, skyr_feature_volume* fv);

/* Build the lattice of `grid` for the sun of `view` (angles, and the frame of
 * `atmosphere` / `cloud`): the grid's mip chain, the position features per node
 * and the optical depth to the sun (a midpoint march at half the voxel edge to
 * the grid box's exit).  Where the grid carries brick majorants
 * (skyr_grid_majorants, which must then be current) the march skips the
 * lookups in bricks whose majorant is 0: they add exactly 0.
 * fv->data (skyr_feature_volume_bytes), fv->stride and fv->sigma_ref are the
 * caller's; the node counts and fv->sun are filled in. */
int skyr_feature_volume_build(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                              const skyr_cloud_parameters* cloud, const skyr_density_grid* grid,
                              const skyr_cloud_view* view, skyr_feature_volume* fv);

/* Training points of a grid (device float[n][6]: position, unit direction):
 * half are where rays from random outside points first collide (delta tracking
 * against the grid's largest extinction `sigma_max`, direction = the ray's),
 * half uniform in the grid box where the extinction is >= sigma_min (uniform
 * direction).  Seeded. */
int skyr_surrogate_sample_points(skyr_ctx* ctx, const skyr_density_grid* grid, float sigma_max, float sigma_min,
                                 uint64_t seed, int n, float* points);

/* Feature records of points (device float[n][6]) from a lattice. */
int skyr_surrogate_records(skyr_ctx* ctx, const skyr_density_grid* grid, const skyr_feature_volume* fv,
                           const float* points, int n, uint16_t* records);

/* Bin of a feature record in the error table (row-major index), for host-side
 * calibration: device records[n] -> device int bins[n]. */
int skyr_surrogate_error_bins(skyr_ctx* ctx, const uint16_t* records, int n, int* bins);

/* The surrogate image of `view` (pixels as skyr_pathtrace): per pixel
 * out_rgba = (luminance rgb, view transmittance), aerial perspective applied at
 * the transmittance-weighted mean depth; the phase function, the sun and the
 * atmosphere as in skyr_pathtrace with `pt`.  out_error (device float per
 * pixel, may be NULL) receives an absolute error estimate: the network's
 * contribution to the luminance, each step weighted by the relative error of
 * its error-table bin (or by network_error).  `packed` is the network
 * (skyr_mlp_pack) or NULL when use_network is 0.  Where the grid carries brick
 * majorants (which must then be current) march samples in bricks whose
 * majorant is 0 take no grid lookup: their extinction is exactly 0. */
int skyr_surrogate_render(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                          const skyr_cloud_parameters* cloud, const skyr_density_grid* grid,
                          const skyr_pathtrace_parameters* pt, const skyr_cloud_view* view,
                          const skyr_lut_sizes* sizes, const void* transmittance,
                          const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                          const skyr_feature_volume* fv, const void* packed, const skyr_surrogate_parameters* sp,
                          float* out_rgba, float* out_error);

#ifdef __cplusplus
}
#endif
#endif /* SKYR_SURROGATE_H_ */
