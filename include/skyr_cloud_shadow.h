/*
 * skyr_cloud_shadow.h — the volumetric cloud's shadow passes
 * (VolumetricCloud::RenderShadow, src/SkyRendering/VolumetricCloud.cpp:282-325):
 * a light-space shadow map of (depth, transmittance) with a temporal blend,
 * its separable blur, and the shadow froxel of mean sun visibility along the
 * view rays.  The raymarch, the path tracer and the surrogate read the froxel
 * through skyr_cloud_view.shadow_froxel.  Conventions as in skyr.h.
 *
 * Light space: the light view looks from the local camera along -sun (glm
 * lookAt, up +z, or +x when the sun is at the local zenith); the orthographic
 * projection bounds the camera frustum cut at shadow_map_max_distance plus
 * half a texel (GetLightProjection, VolumetricCloud.cpp:138-166) with depth
 * range [-1, 1].  Light NDC z is therefore the distance in km along the light
 * direction from the plane through the camera, the unit of the map's depth.
 */
#ifndef SKYR_CLOUD_SHADOW_H_
#define SKYR_CLOUD_SHADOW_H_

#include "skyr_cloud.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Map and froxel sizes (struct id 15). */
typedef struct skyr_cloud_shadow_sizes {
    int map_width, map_height;                     /* 512 x 512 (kShadowMapResolution, VolumetricCloud.cpp:52) */
    int froxel_width, froxel_height, froxel_depth; /* viewport / 12 and 128 slices (VolumetricCloud.cpp:134-135) */
} skyr_cloud_shadow_sizes;

/* The reference sizes for a viewport: 512 x 512, (w / 12) x (h / 12) x 128. */
int skyr_cloud_shadow_sizes_default(int viewport_width, int viewport_height, skyr_cloud_shadow_sizes* out);

/* The light transform of one frame (struct id 16). */
typedef struct skyr_cloud_light_frame {
    float light_view_projection[16];         /* uLightVP: local cloud frame -> light NDC, column-major */
    float inverse_light_view_projection[16]; /* uInvLightVP */
    float model[16];                         /* local cloud frame -> world (VolumetricCloud::model_) */
    float shadow_map_reproject[16];          /* uShadowMapReprojectMat: light NDC -> the previous frame's */
    int has_previous;                        /* shadow_map_reproject is valid */
} skyr_cloud_light_frame;

/* VolumetricCloud::Update's light maths (VolumetricCloud.cpp:188-235) for the
 * camera and sun of `view`: the local frame, the light view and projection
 * (cloud->shadow_map_max_distance, sizes' map resolution for the padding) and,
 * when `previous` is not NULL, the reprojection into the previous frame's map
 *   previous.light_view_projection * inverse(previous.model) * model
 *   * translate(wind_delta.x, wind_delta.y, 0) * inverse_light_view_projection,
 * wind_delta (NULL: 0) being the material's wind displacement since the
 * previous frame in local km (additional_delta, VolumetricCloudDefaultMaterial.cpp:93).
 * Host only: computed in double, stored as float.  SKYR_EINVAL for a
 * singular view_projection, a zero sun direction or a non-positive distance. */
int skyr_cloud_light_frame_derive(const skyr_atmosphere_parameters* atmosphere,
                                  const skyr_cloud_parameters* cloud, const skyr_cloud_view* view,
                                  const skyr_cloud_shadow_sizes* sizes, const skyr_cloud_light_frame* previous,
                                  const float* wind_delta, skyr_cloud_light_frame* out);

/* One frame of RenderShadow on the context's stream, three passes:
 *  1. shadow map (VolumetricCloudShadowMap.comp:37-75).  Each texel of
 *     `raw_map` is float2 (depth along the light ray of the shell's midpoint,
 *     cloud transmittance), row-major, map_height rows of map_width (the
 *     reference's RG32F).  Its light ray starts on the light's z = 0 plane and
 *     is marched in mix(12, 6, |dir.z|) jittered steps through the cloud
 *     shell with the material's SampleSigmaT.  Where `previous_raw_map` is
 *     not NULL and frame->has_previous, texels whose reprojected position
 *     lies inside the previous map keep 0.8 of it (GL LINEAR sampling).
 *  2. blur (VolumetricCloudShadowMapBlur.comp:9-42): separable 9-tap
 *     Gaussian with clamped indices, raw_map -> `shadow_map` (float2 texels).
 *  3. shadow froxel (VolumetricCloudShadowFroxel.comp:10-27): froxel_depth
 *     slices of the view rays out to cloud->shadow_froxel_max_distance.  Each
 *     texel is the running mean of the shadow-map transmittance
 *     (SampleCloudShadowTransmittance: LINEAR, CLAMP_TO_BORDER with border
 *     (1e10, 1), 0.5 km depth transition) as unorm16, [depth][height][width].
 * `shadow_map` and `froxel` may be NULL to stop after the pass before.
 * Allocates nothing; capturable into a CUDA graph. */
int skyr_cloud_shadow_render(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                             const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                             const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                             const skyr_cloud_shadow_sizes* sizes, const skyr_cloud_light_frame* frame,
                             const float* blue_noise, const float* previous_raw_map, float* raw_map,
                             float* shadow_map, uint16_t* froxel);

#ifdef __cplusplus
}
#endif
#endif /* SKYR_CLOUD_SHADOW_H_ */
