/*
 * skyr_environment.h — the environment luminance cube map of
 * AtmosphereRenderer::Render (ENVIRONMENT_LUMINANCE program,
 * shaders/SkyRendering/AtmosphereRenderer.glsl:248-275, dispatched at
 * src/SkyRendering/AtmosphereRenderer.cpp:234-242) and its mip chain
 * (glGenerateTextureMipmap).  Conventions as in skyr.h.
 *
 * Layout: levels 0..levels-1 consecutive; level l holds 6 faces of
 * s_l x s_l half4 texels (s_l = max(face_size >> l, 1)), face-major, rows top
 * to bottom: texel (face, x, y) of level l is at
 * level_offset(l) + (face * s_l + y) * s_l + x.  Faces in GL order
 * (+X, -X, +Y, -Y, +Z, -Z; ConvertCubUvToDir, shaders/Base/Common.glsl:13-30);
 * row y of level 0 looks along face v = 1 - (y + 0.5) / s_0 (the program's
 * flip).  rgb = luminance, a = 0.
 */
#ifndef SKYR_ENVIRONMENT_H_
#define SKYR_ENVIRONMENT_H_

#include "skyr.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Number of texels (half4) before level `level` (level == levels: the whole
 * cube); 0 for a face size that is not a power of two in [1, 512]. */
size_t skyr_environment_cube_level_offset(int face_size, int level);

/* Level 0: per texel the sky-view luminance in the texel's direction plus,
 * below the horizon, the lit ground times the sky-view transmittance, for the
 * camera and sun of `render` (kEnvironmentLuminanceTextureWidth = 128 in the
 * reference).  Levels 1..levels-1: each texel the mean of its 2x2 parent
 * texels (the box filter of glGenerateTextureMipmap, computed in FP32 from
 * the parent's stored half values).  `levels` in [1, log2(face_size) + 1].
 * Inputs as skyr_update_lut_set's outputs for one set (sky-view LUTs of
 * sizes->format).  Writes skyr_environment_cube_level_offset(face_size,
 * levels) half4 texels to device memory `out`.  Allocates nothing. */
int skyr_environment_cube(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                          const skyr_atmosphere_render_parameters* render, const skyr_lut_sizes* sizes,
                          const void* transmittance, const void* sky_view_luminance,
                          const void* sky_view_transmittance, int face_size, int levels, void* out);

/* The image-based-lighting precomputations of IBL::Precompute
 * (src/Base/src/IBL.cpp:25-45) read the cube as GL does with
 * TEXTURE_CUBE_MAP_SEAMLESS and a LINEAR / LINEAR_MIPMAP_LINEAR sampler:
 * face and (s, t) from the direction's major axis (GL 4.6 table 8.19),
 * bilinear taps past a face edge taken from the adjacent face, a tap past a
 * corner the mean of the three texels that meet there, LOD clamped to
 * [0, levels - 1].  They read it from a seamless copy: every face of every
 * level with a one-texel apron holding those edge and corner values, float4
 * texels, level l at skyr_environment_seamless_level_offset(face_size, l),
 * texel (face, i, j), i and j in [-1, s_l], at
 * offset + (face * (s_l + 2) + j + 1) * (s_l + 2) + i + 1. */
size_t skyr_environment_seamless_level_offset(int face_size, int level); /* 0 for bad sizes */

/* The seamless copy of `levels` levels of a cube (layout above) to device
 * memory `out` (skyr_environment_seamless_level_offset(face_size, levels)
 * float4 texels). */
int skyr_environment_seamless(skyr_ctx* ctx, const void* cube, int face_size, int levels, float* out);

/* EnvRadianceSH.comp: the first 9 spherical-harmonic coefficients of the
 * radiance (level 0, 32 x 32 stratified directions, 4 pi / 1024 weights)
 * written as 9 float4 (rgb, a = 0) to device memory `out`; `seamless` is the
 * cube's seamless copy. */
int skyr_environment_sh(skyr_ctx* ctx, const float* seamless, int face_size, int levels, float* out);

/* PrefilterRadiance.comp: roughness_count cube levels of the GGX-prefiltered
 * radiance (level k: side resolution >> k, roughness k / (roughness_count - 1),
 * uint(mix(1, 64, roughness^0.3)) Hammersley samples) sampled from the
 * seamless copy, half4 texels in the cube layout, to device memory `out`
 * (skyr_environment_cube_level_offset(resolution, roughness_count) texels).
 * resolution: a power of two in [1, 512]; roughness_count in
 * [2, log2(resolution) + 1] (the reference: 128, 5). */
int skyr_environment_prefilter(skyr_ctx* ctx, const float* seamless, int face_size, int levels, int resolution,
                               int roughness_count, void* out);

#ifdef __cplusplus
}
#endif
#endif /* SKYR_ENVIRONMENT_H_ */
