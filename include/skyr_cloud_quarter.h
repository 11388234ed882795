/*
 * skyr_cloud_quarter.h — the reference's production cloud pass: the raymarch
 * at a quarter of the viewport's resolution on a rotating checkerboard,
 * temporally reconstructed at half resolution and upscaled into the HDR
 * target (VolumetricCloud::Render, src/SkyRendering/VolumetricCloud.cpp:327-423):
 *   1. checkerboard depth (CheckerboardGen.comp): (w/2) x (h/2) texels, the
 *      max (x, y same parity) or min of each 2x2 block of the window depth;
 *   2. index (VolumetricCloudIndexGen.comp): for each (w/4) x (h/4) texel,
 *      which of its 2x2 checkerboard texels is raymarched this frame, and its
 *      linear depth;
 *   3. raymarch (VolumetricCloudRender.comp:139-210) of those texels;
 *   4. reconstruct (VolumetricCloudReconstruct.comp): (w/2) x (h/2), the
 *      Reinhard-tonemapped neighbourhood clamp of the reprojected previous
 *      frame, blended 0.2 toward the texel raymarched this frame;
 *   5. upscale (VolumetricCloudUpscale.comp): each viewport pixel takes the
 *      depth-nearest or the mean of four reconstructed texels and is
 *      composited over the HDR target.
 * Conventions as in skyr.h.  Texel (x, y) of a w x h image is at y * w + x.
 */
#ifndef SKYR_CLOUD_QUARTER_H_
#define SKYR_CLOUD_QUARTER_H_

#include "skyr_batch.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Per-frame constants of the temporal passes (struct id 17). */
typedef struct skyr_cloud_temporal_frame {
    float reproject[16];    /* uReprojectMat: local cloud frame -> the previous frame's clip space, column-major */
    float z_near, z_far;    /* the camera planes of DepthToLinearDepth (uLinearDepthParam) */
    int base_shading_index; /* uBaseShadingIndex = frame id & 3 */
    int has_previous;       /* reproject refers to a previous frame */
} skyr_cloud_temporal_frame;

/* VolumetricCloud::Update's temporal constants (VolumetricCloud.cpp:188-239):
 * reproject = previous MVP * translate(delta.x, delta.y, 0), delta = the
 * camera's move since `previous_view` in this frame's local frame plus
 * wind_delta (additional_delta, local km; NULL: 0).  previous_view NULL: no
 * history (has_previous 0).  Host only, double, stored as float.  SKYR_EINVAL
 * for singular view-projections or planes with !(0 < z_near < z_far). */
int skyr_cloud_temporal_frame_derive(const skyr_atmosphere_parameters* atmosphere, const skyr_cloud_view* view,
                                     const skyr_cloud_view* previous_view, const float* wind_delta, float z_near,
                                     float z_far, int frame_index, skyr_cloud_temporal_frame* out);

/* Device buffers of one viewport (struct id 18; ViewportData,
 * VolumetricCloud.cpp:120-136).  With the viewport w x h: half = (w/2) x (h/2),
 * quarter = (half.w/2) x (half.h/2), integer division. */
typedef struct skyr_cloud_quarter_buffers {
    float* checkerboard_depth;        /* half, float (R32F) */
    float* index_linear_depth;        /* quarter, float2: (index 0..3, linear depth) (RG32F) */
    void* render_rgba;                /* quarter, half4 (RGBA16F): luminance, transmittance */
    float* render_distance;           /* quarter, float (R32F) */
    const void* previous_reconstruct; /* half, half4 of the previous frame; NULL: no history */
    void* reconstruct;                /* half, half4: this frame's reconstruction */
} skyr_cloud_quarter_buffers;

/* The five passes on the context's stream.  view->width / height are the
 * viewport's (the full-resolution target).  `depth`: the viewport's window
 * depth (GL [0, 1], float per pixel) or NULL for an empty depth buffer (1).
 * The raymarch reads the view's shadow froxel like skyr_cloud_render and uses
 * the context's launch shape (skyr_batch.h).  Where previous_reconstruct is
 * NULL or frame->has_previous is 0 every texel takes this frame's raymarched
 * value (blend weight 1).  `hdr`: the viewport's half4 HDR target,
 * composited in place (rgb * T + luminance, T <= 0.01 as 0); NULL stops
 * after the reconstruction.  Allocates nothing; capturable. */
int skyr_cloud_render_quarter(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                              const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                              const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                              const skyr_lut_sizes* sizes, const void* transmittance,
                              const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                              const float* blue_noise, const float* depth, const skyr_cloud_temporal_frame* frame,
                              const skyr_cloud_quarter_buffers* buffers, void* hdr);

/* The cloud autotuner of skyr_batch.h (same SKYR_CLOUD_TUNE_CANDIDATES, same
 * order of times_ms, same reps rule) timed on skyr_cloud_render_quarter's own
 * passes up to the reconstruction (hdr NULL): the checkerboard raymarch has
 * 1/16 of the viewport's rays, so it wants its own launch shape.  Keeps the
 * fastest in the context; the buffers' outputs are overwritten. */
int skyr_autotune_cloud_quarter(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                                const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                                const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                                const skyr_lut_sizes* sizes, const void* transmittance,
                                const void* aerial_perspective_luminance,
                                const void* aerial_perspective_transmittance, const float* blue_noise,
                                const float* depth, const skyr_cloud_temporal_frame* frame,
                                const skyr_cloud_quarter_buffers* buffers, int reps, skyr_tuning* best,
                                float* times_ms);

#ifdef __cplusplus
}
#endif
#endif /* SKYR_CLOUD_QUARTER_H_ */
