/*
 * skyr_cloud.h — C ABI of the procedural noise generators, the cloud material
 * plug-ins and the volumetric-cloud raymarch.  Conventions as in skyr.h.
 *
 * Noise textures live in device memory as UNORM8 bytes: mip levels 0..L-1
 * stored consecutively (level k is max(W>>k,1) x max(H>>k,1) x max(D>>k,1)),
 * each level channel-planar: byte (c, x, y, z) of a level of size w x h x d is
 * at c*w*h*d + (z*h + y)*w + x.  Sizes must be powers of two.
 */
#ifndef SKYR_CLOUD_H_
#define SKYR_CLOUD_H_

#include "skyr.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- noise generators (shaders/SkyRendering/NoiseGen.comp) -------------- */
#define SKYR_NOISE_PERLIN 0        /* PerlinFBM (NoiseGen.comp:20-35) */
#define SKYR_NOISE_WORLEY 1        /* WorleyFBM (NoiseGen.comp:36-50) */
#define SKYR_NOISE_PERLIN_WORLEY 2 /* RemapFrom01(PerlinFBM(a), WorleyFBM(b), 1) (NoiseGen.comp:95-104) */
#define SKYR_NOISE_ZERO 3          /* constant 0 */

/* NoiseCreateInfo (src/SkyRendering/VolumetricCloudDefaultMaterial.h:57-64) */
typedef struct skyr_noise_create_info {
    int seed;
    int base_frequency;
    float remap_min;
    float remap_max;
} skyr_noise_create_info;

typedef struct skyr_noise_channel {
    int kind;                 /* SKYR_NOISE_* */
    skyr_noise_create_info a; /* Perlin (or Worley) parameters */
    skyr_noise_create_info b; /* Worley parameters of SKYR_NOISE_PERLIN_WORLEY */
} skyr_noise_channel;

/* One DynamicTexture (VolumetricCloudDefaultMaterial.h:20-55): size, channel
 * generators and fBm octave count (the reference hard-codes 8,
 * NoiseGen.comp:25,41).  Texel coordinate = (index + 0.5) / size, z = 0 for
 * 2D textures (depth 1). */
typedef struct skyr_noise_texture_desc {
    int width, height, depth;
    int channels; /* 1..4 */
    int octaves;  /* 1..16 */
    skyr_noise_channel channel[4];
} skyr_noise_texture_desc;

int skyr_noise_texture_levels(const skyr_noise_texture_desc* desc);
/* Byte offset of mip level `level` (level == levels gives the total size). */
size_t skyr_noise_level_offset(const skyr_noise_texture_desc* desc, int level);

/* DynamicTexture::Generate (VolumetricCloudDefaultMaterial.h:39-49): run the
 * generator into level 0 (imageStore UNORM8 rounding) and build the mip chain
 * (box filter, 2^n sizes, round to nearest) in `out`
 * (skyr_noise_level_offset(desc, levels) bytes of device memory). */
int skyr_noise_generate(skyr_ctx* ctx, const skyr_noise_texture_desc* desc, void* out);

/* Level 0 of a texture re-laid for filtering: for each texel and each of the
 * first `channels` channels, the REPEAT-wrapped corner bytes of GL LINEAR
 * filtering at that texel, packed little-endian -- 2D: one uint32 holding
 * (x,y) (x+1,y) (x,y+1) (x+1,y+1); 3D: one uint64 holding corner
 * dx + 2 dy + 4 dz in byte dx + 2 dy + 4 dz.  Channel-planar.  The raymarch
 * reads one word per filtered sample from it instead of 4 or 8 bytes.
 * (No reference counterpart: an exact re-layout of the texture.) */
size_t skyr_noise_expanded_bytes(const skyr_noise_texture_desc* desc, int channels);
int skyr_noise_expand(skyr_ctx* ctx, const skyr_noise_texture_desc* desc, const void* tex, int channels,
                      void* out);

/* Hardware samplers of one channel of a generated texture: the bytes are
 * copied (ordered on the context's stream) into CUDA arrays that the texture
 * units sample as the GL texture of the reference is sampled -- REPEAT,
 * UNORM8.  skyr_noise_sampler_handle: level 0 with LINEAR filtering and its
 * 8-bit fixed-point weights (1/256), the precision GL drivers filter the
 * reference's textures with (magnification).  skyr_noise_sampler_nearest_handle:
 * every mip level, NEAREST at an explicit level (the NEAREST_MIPMAP_NEAREST
 * minification, the level chosen by the caller's own LOD).  The cloud raymarch
 * takes its Material1 fetches from them when skyr_cloud_textures names them.
 * The library allocates the arrays; the sampler keeps no pointer to `tex`.
 * Handles are cudaTextureObject_t as 64-bit values.  (Counterpart: the texture
 * objects the reference binds, VolumetricCloudDefaultMaterial.cpp:40-72.) */
typedef struct skyr_noise_sampler skyr_noise_sampler;
int skyr_noise_sampler_create(skyr_ctx* ctx, const skyr_noise_texture_desc* desc, const void* tex, int channel,
                              skyr_noise_sampler** out);
/* Copy a regenerated texture (same description) into the sampler; the handle stays valid. */
int skyr_noise_sampler_update(skyr_ctx* ctx, skyr_noise_sampler* sampler, const void* tex);
int skyr_noise_sampler_destroy(skyr_noise_sampler* sampler);
uint64_t skyr_noise_sampler_handle(const skyr_noise_sampler* sampler);
uint64_t skyr_noise_sampler_nearest_handle(const skyr_noise_sampler* sampler);

/* ---- material plug-ins (IVolumetricCloudMaterial) --------------------- */
#define SKYR_MATERIAL_DEFAULT0 0 /* VolumetricCloudDefaultMaterial0 (VolumetricCloudDefaultMaterial0.glsl) */
#define SKYR_MATERIAL_DEFAULT1 1 /* VolumetricCloudDefaultMaterial1 (VolumetricCloudDefaultMaterial1.glsl) */
#define SKYR_MATERIAL_MINIMAL 2  /* VolumetricCloudMinimalMaterial (VolumetricCloudMaterialMinimal.glsl) */
#define SKYR_MATERIAL_VOXEL 3    /* VolumetricCloudVoxelMaterial (VolumetricCloudMaterialVoxel.glsl), R8 grid */

/* Samplers::MipmapMin (src/Base/include/Samplers.h:20-28) */
#define SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST 0
#define SKYR_MIPMAP_LINEAR_MIPMAP_NEAREST 1
#define SKYR_MIPMAP_NEAREST_MIPMAP_LINEAR 2
#define SKYR_MIPMAP_LINEAR_MIPMAP_LINEAR 3

/* Material fields (VolumetricCloudDefaultMaterial.h:86-208,
 * VolumetricCloudMinimalMaterial.h, VolumetricCloudVoxelMaterial.h); JSON keys
 * of bin/config.json:132-174 without the trailing underscore. */
typedef struct skyr_cloud_material {
    int type; /* SKYR_MATERIAL_* */
    /* VolumetricCloudDefaultMaterialCommon */
    float density;  /* sigma_t max, 1/km */
    float lod_bias;
    float cloud_map_repeat_size, detail_repeat_size, displacement_repeat_size; /* km */
    float offset_from_first[2];        /* accumulated wind/camera offset of the local frame, km */
    float detail_offset_from_first[2]; /* extra detail offset (detail_wind_magnify_), km */
    int minfilter2d, minfilter3d, minfilter_displacement; /* SKYR_MIPMAP_* */
    /* VolumetricCloudDefaultMaterial1 */
    float base_density_threshold, base_height_hardness, base_edge_hardness;
    float detail_base, detail_scale, height_cut, edge_cut;
    /* VolumetricCloudDefaultMaterial0 */
    float detail_param[2];
    float displacement_scale;
    /* VolumetricCloudVoxelMaterial */
    float voxel_base[2];  /* km */
    float voxel_width[2]; /* km */
} skyr_cloud_material;

/* Fill `m` with the defaults of material `type`. */
int skyr_cloud_material_default(int type, skyr_cloud_material* m);

/* Device textures a material samples: cloud_map (2D, 2 channels), detail
 * (3D, channel 0 read), displacement (2D, 4 channels), voxel (3D, 1 channel);
 * unused ones may be NULL.  Each desc gives the size / channel count; only
 * width/height/depth/channels are read.  The *_expanded pointers optionally
 * give skyr_noise_expand output of the same texture (with `*_expanded_channels`
 * channels); when present the level-0 filtering reads them. */
typedef struct skyr_cloud_textures {
    const void* cloud_map;
    skyr_noise_texture_desc cloud_map_desc;
    const void* detail;
    skyr_noise_texture_desc detail_desc;
    const void* displacement;
    skyr_noise_texture_desc displacement_desc;
    const void* voxel;
    skyr_noise_texture_desc voxel_desc;
    const void* cloud_map_expanded;
    const void* detail_expanded;
    const void* displacement_expanded;
    const void* voxel_expanded;
    int cloud_map_expanded_channels, detail_expanded_channels;
    int displacement_expanded_channels, voxel_expanded_channels;
    /* optional hardware samplers of channel 0 of the cloud map and of the
     * detail texture (0 = none): skyr_noise_sampler_handle (magnified, LINEAR)
     * and skyr_noise_sampler_nearest_handle (minified, NEAREST per level) */
    uint64_t cloud_map_sampler, detail_sampler;
    uint64_t cloud_map_sampler_nearest, detail_sampler_nearest;
} skyr_cloud_textures;

/* ---- volumetric cloud (VolumetricCloud) ------------------------------ */

/* VolumetricCloud fields (src/SkyRendering/VolumetricCloud.h:20-55).  The
 * three phase constants are parameters here; the reference values 0.85, -0.15
 * and 2.16 (VolumetricCloudRender.comp:125-126) are the defaults. */
typedef struct skyr_cloud_parameters {
    float bottom_altitude; /* km */
    float thickness;       /* km */
    float max_raymarch_distance;
    float max_raymarch_steps;
    float max_visible_distance;
    float env_color[3];
    float env_color_scale;
    float sun_illuminance_scale;
    float shadow_steps;
    float shadow_distance;
    float shadow_froxel_max_distance;
    float sun_multiscattering_sigma_scale;
    float env_multiscattering_sigma_scale;
    float env_bottom_visibility;
    float env_sun_height_curve_exp;
    float phase_g_forward;
    float phase_g_back;
    float phase_back_scale;
    float shadow_map_max_distance; /* km, frustum depth the shadow map covers (VolumetricCloud.h:30) */
} skyr_cloud_parameters;

int skyr_cloud_parameters_default(skyr_cloud_parameters* c);

/* Camera and frame inputs of VolumetricCloud::Update
 * (src/SkyRendering/VolumetricCloud.cpp:168-280). */
typedef struct skyr_cloud_view {
    float camera_position[3];  /* world, y up, km */
    float view_projection[16]; /* column-major */
    float fovy;                /* degrees, for the texture LOD constant (CalKLod) */
    int viewport_width, viewport_height; /* viewport of CalKLod */
    int width, height;                   /* raymarch resolution */
    float sun_direction_theta, sun_direction_phi; /* degrees */
    float frame_id;
    float aerial_perspective_lut_max_distance;
    /* Shadow froxel of skyr_cloud_shadow_render for this view, or NULL for a
     * visibility of 1: unorm16 texels [depth][height][width], read with GL
     * LINEAR + CLAMP_TO_EDGE at the pixel's (u, v) and w = distance /
     * shadow_froxel_max_distance, and faded to 1 by clamp(1 / w, 0, 1)
     * (SampleRayScatterVisibility, VolumetricCloudShadowInterface.glsl:10-13);
     * it scales the aerial-perspective luminance of the composite. */
    const uint16_t* shadow_froxel;
    int shadow_froxel_width, shadow_froxel_height, shadow_froxel_depth;
} skyr_cloud_view;

/* The raymarch pass of VolumetricCloud::Render at full resolution
 * (shaders/SkyRendering/VolumetricCloudRender.comp:139-210), with an empty
 * depth buffer where `depth` is NULL (else one float per pixel, GL window
 * depth) and the view's shadow froxel (1 where it has none).  Inputs: the transmittance LUT and the
 * aerial-perspective LUTs of `sizes` (RGBA32F or RGBA16F per sizes->format),
 * a 64x64 float blue-noise tile.  Outputs (device): `out_rgba` half4 per pixel
 * (rgb luminance, a transmittance; reference RGBA16F), `out_distance` float per
 * pixel (transmittance-weighted mean distance; reference R32F); either may be
 * NULL. */
int skyr_cloud_render(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                      const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                      const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                      const skyr_lut_sizes* sizes, const void* transmittance,
                      const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                      const float* blue_noise, const float* depth, void* out_rgba, float* out_distance);

/* skyr_cloud_render for a caller that reads the frame on the host: the kernel
 * stores each pixel straight into `host_rgba` (half4 per pixel) and
 * `host_distance` (float per pixel), so the device-to-host transfer of the
 * frame (12 bytes per pixel) runs over the GPU's link to host memory while the
 * raymarch is still going, instead of as a copy after it.  Same inputs, pixel
 * values and layouts as skyr_cloud_render.  The reference leaves the pass's
 * images on the GPU (VolumetricCloud::Render, VolumetricCloud.cpp:327) and
 * reads frames back only as a copy after rendering (glReadPixels in
 * GLWindow::ScreenShot, src/Base/src/GLWindow.cpp:247-252).  Both outputs
 * must be page-locked host memory mapped for the context's device
 * (cudaHostAlloc / cudaMallocHost under unified addressing, or cudaHostRegister
 * with cudaHostRegisterMapped); pageable, device or misaligned pointers
 * (host_rgba 8-byte, host_distance 4-byte) return SKYR_EINVAL before any
 * launch.  Either may be NULL.  The writes are complete when the context's
 * stream reaches the end of the call. */
int skyr_cloud_render_to_host(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                              const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                              const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                              const skyr_lut_sizes* sizes, const void* transmittance,
                              const void* aerial_perspective_luminance,
                              const void* aerial_perspective_transmittance, const float* blue_noise,
                              const float* depth, void* host_rgba, float* host_distance);

/* One frame's LUT set and cloud raymarch, in the reference's per-frame order
 * (AppWindow::Render: AtmosphereRenderer::Render's LUT passes through
 * RenderViewport, src/SkyRendering/AppWindow.cpp:216, then
 * VolumetricCloud::Render, :174): skyr_update_lut_set for one parameter set
 * (atmosphere, render) into the six LUT buffers, then skyr_cloud_render (or,
 * with outputs_on_host nonzero, skyr_cloud_render_to_host) reading that set's
 * transmittance and aerial-perspective LUTs.  The results are those of the two
 * calls, bit for bit.  The raymarch is launched as a programmatic dependent of
 * the LUT set's last pass: its rays march while the LUT passes finish and wait
 * for them only before their first LUT read, so part of the raymarch overlaps
 * the LUT set.  Everything else the raymarch reads (textures, blue noise,
 * depth, the view's shadow froxel) must be complete when the call is
 * enqueued, as for the two calls.  All arguments are checked before anything
 * is enqueued; the sky-view pair may be NULL, the aerial-perspective pair not.
 * (No reference counterpart as one call.) */
int skyr_render_frame(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                      const skyr_atmosphere_render_parameters* render, const skyr_lut_sizes* sizes,
                      void* transmittance, void* multiscattering, void* sky_view_luminance,
                      void* sky_view_transmittance, void* aerial_perspective_luminance,
                      void* aerial_perspective_transmittance, const skyr_cloud_parameters* cloud,
                      const skyr_cloud_material* material, const skyr_cloud_textures* textures,
                      const skyr_cloud_view* view, const float* blue_noise, const float* depth, void* out_rgba,
                      float* out_distance, int outputs_on_host);

/* skyr_cloud_render that also accumulates work counters into device memory
 * `counters` (3 x uint64, not cleared): [0] raymarch samples taken,
 * [1] SampleSigmaT evaluations (raymarch + light march), [2] those of them
 * that sampled the detail texture (Material1: past the coverage test;
 * Material0: all).  Same outputs as skyr_cloud_render, bit for bit; the
 * instrumented kernel runs one lane per ray whatever the tuning says.
 * (No reference counterpart: instrumentation.) */
int skyr_cloud_render_counted(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                              const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                              const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                              const skyr_lut_sizes* sizes, const void* transmittance,
                              const void* aerial_perspective_luminance,
                              const void* aerial_perspective_transmittance, const float* blue_noise,
                              const float* depth, void* out_rgba, float* out_distance,
                              unsigned long long* counters);

/* Seeded 64x64 blue-noise tile (void-and-cluster ranks, value = (rank+0.5)/4096)
 * written to host memory `out` (4096 floats), for callers without the
 * reference's data/BlueNoise/64_64/HDR_L_0.png (which the caller may upload
 * instead: GL_R16 values / 65535, row y of the file = texel row y). */
int skyr_blue_noise_generate(uint32_t seed, float* out);

#ifdef __cplusplus
}
#endif
#endif /* SKYR_CLOUD_H_ */
