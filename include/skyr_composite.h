/*
 * skyr_composite.h — the full-screen atmosphere composite of
 * AtmosphereRenderer::Render (ATMOSPHERE_RENDER fragment shader,
 * shaders/SkyRendering/AtmosphereRenderer.glsl:345-432) as a compute pass
 * over a viewport: per pixel the in-scattered luminance and transmittance
 * along the view ray to the depth buffer's object or the atmosphere's edge
 * (the per-pixel ComputeScatteredLuminance raymarch, or the sky-view /
 * aerial-perspective LUTs), the cloud shadow froxel's visibility, and behind
 * it the object's shading, the sun disc with limb darkening or the star map.
 * Conventions as in skyr.h.
 *
 * The object term is the caller's: ComputeObjectLuminance
 * (AtmosphereRenderer.glsl:284-323) shades the G-buffer with the mesh shadow
 * map, PCSS and IBL, which belong to the raster path; the composite adds the
 * given object luminance times the transmittance.  The mesh shadow map's
 * volumetric light inside the raymarch (VOLUMETRIC_LIGHT_ENABLE) sees no
 * meshes here and is 1; the moon shadow is off, as in the reference defaults.
 */
#ifndef SKYR_COMPOSITE_H_
#define SKYR_COMPOSITE_H_

#include "skyr.h"

#ifdef __cplusplus
extern "C" {
#endif

/* AtmosphereRenderParameters and AtmosphereRenderInitParameters fields of the
 * composite (src/SkyRendering/AtmosphereRenderer.h:14-52), struct id 19. */
typedef struct skyr_composite_parameters {
    float star_luminance_scale;     /* 0.005 */
    float raymarching_steps;        /* 40 */
    int use_sky_view_lut;           /* 0: the sky is raymarched per pixel */
    int use_aerial_perspective_lut; /* 0: so is the air in front of objects */
    int dither_sample_point;        /* 1: the first sample at the blue noise's value, else at 0.5 */
} skyr_composite_parameters;

int skyr_composite_parameters_default(skyr_composite_parameters* out);

/* The per-frame buffers of one viewport (struct id 20).  Device pointers. */
typedef struct skyr_composite_inputs {
    int width, height;             /* the viewport: pixel (x, y) at y * width + x, uv = (x + 0.5, y + 0.5) / size */
    const float* depth;            /* GL window depth per pixel, or NULL: no objects (depth 1 everywhere) */
    const float* object_luminance; /* float4 per pixel (rgb used), or NULL: 0 */
    const float* blue_noise;       /* the 64 x 64 tile; needed when dither_sample_point */
    const uint8_t* star_map;       /* sRGB8 RGB texels, star_width x star_height, row 0 at v = 0; NULL: no stars */
    int star_width, star_height;
    const uint16_t* shadow_froxel; /* the cloud shadow froxel (skyr_cloud_shadow_render), or NULL: visibility 1 */
    int froxel_width, froxel_height, froxel_depth;
    float shadow_froxel_max_distance; /* km */
} skyr_composite_inputs;

/* The composite into `out_hdr` (half4 per pixel: luminance, a = 1; the
 * reference's FragColor into the RGBA16F HDR target).  LUT inputs as
 * skyr_update_lut_set's outputs for one set; the multi-scattering LUT is read
 * by the raymarch, the sky-view and aerial-perspective LUTs only when their
 * switch is on.  Allocates nothing; capturable. */
int skyr_atmosphere_composite(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                              const skyr_atmosphere_render_parameters* render,
                              const skyr_composite_parameters* parameters, const skyr_lut_sizes* sizes,
                              const void* transmittance, const void* multiscattering,
                              const void* sky_view_luminance, const void* sky_view_transmittance,
                              const void* aerial_perspective_luminance,
                              const void* aerial_perspective_transmittance, const skyr_composite_inputs* inputs,
                              void* out_hdr);

#ifdef __cplusplus
}
#endif
#endif /* SKYR_COMPOSITE_H_ */
