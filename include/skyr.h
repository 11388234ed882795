/*
 * skyr.h — C ABI of the GB300-native atmosphere-LUT / volumetric-cloud hot path.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status (SKYR_OK on success) and never throws.  Device buffers are owned by
 * the caller; their layouts are documented beside each call.  One skyr_ctx is
 * bound to one CUDA stream; calls on one context are ordered by that stream.
 * A context is not thread-safe; separate contexts are independent.
 *
 * Units follow the reference: lengths in km, extinction in 1/km, angles in
 * degrees in parameter structs.  Images are row-major with x fastest:
 * texel (x, y, z) of a W x H x D image with C channels is at
 * ((z * H + y) * W + x) * C.
 *
 * The comment on each declaration names the reference interface it replaces
 * (file:line within the c52e/SkyRendering project).
 */
#ifndef SKYR_H_
#define SKYR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SKYR_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define SKYR_OK 0
#define SKYR_EINVAL 1   /* bad argument (null pointer, size out of range, NaN parameter) */
#define SKYR_ENOMEM 2   /* device or host allocation failed */
#define SKYR_ECUDA 3    /* a CUDA runtime call failed */
#define SKYR_ETIMEOUT 4 /* a bounded device-side wait gave up */
#define SKYR_ENOTSUP 5  /* combination not supported */

/* ---- storage formats of LUT outputs ----------------------------------- */
#define SKYR_FORMAT_RGBA32F 0 /* float4 per texel (reference GL_RGBA32F) */
#define SKYR_FORMAT_RGBA16F 1 /* half4 per texel */

typedef struct skyr_ctx skyr_ctx;

/* Version of this ABI (SKYR_ABI_VERSION of the built library). */
int skyr_abi_version(void);

/* Human-readable name of a status code; static storage. */
const char* skyr_status_string(int status);

/* Message of the last failed call on this host thread; static thread-local storage. */
const char* skyr_last_error(void);

/* sizeof() of the public structs, for binding layout checks:
 * 0 skyr_atmosphere_parameters, 1 skyr_atmosphere_render_parameters,
 * 2 skyr_lut_sizes, 3 skyr_noise_texture_desc, 4 skyr_cloud_material,
 * 5 skyr_cloud_textures, 6 skyr_cloud_parameters, 7 skyr_cloud_view,
 * 8 skyr_density_grid, 9 skyr_grid_generator, 10 skyr_pathtrace_parameters;
 * further ids are listed beside later structs.
 * Returns 0 for an unknown id.  (No reference counterpart: ABI hygiene.) */
size_t skyr_struct_size(int which);

/* Create a context bound to `cuda_stream` (a cudaStream_t; NULL = legacy default
 * stream) on the current CUDA device.
 * Replaces the GL-context ownership of Atmosphere/AtmosphereRenderer/VolumetricCloud
 * (src/SkyRendering/Atmosphere.cpp:43-70, src/SkyRendering/VolumetricCloud.cpp:54-113). */
int skyr_ctx_create(void* cuda_stream, skyr_ctx** out_ctx);
int skyr_ctx_destroy(skyr_ctx* ctx);
/* Block the host until all work queued on the context's stream is done. */
int skyr_ctx_synchronize(skyr_ctx* ctx);
/* Synchronise and report the context's device status word: SKYR_ETIMEOUT
 * when a device loop stopped at its iteration bound since the last check
 * (the word is then cleared), else SKYR_OK.  (No reference counterpart: the
 * reference has no device-side error reporting.) */
int skyr_ctx_check_status(skyr_ctx* ctx);

/* Bounds of the device loops that could otherwise run long on bad input or a
 * broken device.  A loop that reaches its bound stops, sets the context's
 * status word, and skyr_ctx_check_status reports SKYR_ETIMEOUT; nothing waits
 * without a bound.  Each context starts with skyr_device_limits_default.
 * (No reference counterpart: the reference has no device-side bounds.)
 * struct id 21 of skyr_struct_size. */
typedef struct skyr_device_limits {
    /* samples of one free-flight or ratio-tracking walk of the path tracer
     * (a valid scene needs ~ sigma_max x chord, tens to hundreds); default
     * 2^20, range [1, 2^30] */
    int32_t tracking_steps;
    int32_t reserved; /* 0 */
    /* SM clock cycles a block waits for an asynchronous unit of its own
     * before it gives up: the bulk copy of the network into the shared memory
     * of a surrogate-raymarch block, and the tensor-core products of the
     * network's inference and training kernels.  A block that gives up
     * waits for the work in flight with the default bound, frees its tensor
     * memory and leaves without writing its outputs.  Default 2^31 (about a
     * second), range [0, 2^40] (0: no block waits, every block gives up at
     * once) */
    int64_t copy_wait_cycles;
} skyr_device_limits;
int skyr_device_limits_default(skyr_device_limits* out);
int skyr_ctx_set_limits(skyr_ctx* ctx, const skyr_device_limits* limits); /* SKYR_EINVAL outside the ranges */
int skyr_ctx_get_limits(const skyr_ctx* ctx, skyr_device_limits* out);

/* ======================================================================== */
/* Atmosphere                                                                */
/* ======================================================================== */

/* User-unit atmosphere description; same fields, units and defaults as
 * AtmosphereParameters (src/SkyRendering/Atmosphere.h:10-38) and the
 * "earth_.parameters" block of bin/config.json:62-108. */
typedef struct skyr_atmosphere_parameters {
    float solar_illuminance[3];
    float sun_angular_radius; /* degrees */
    float bottom_radius;      /* km */
    float thickness;          /* km; top radius = bottom_radius + thickness */
    float ground_albedo[3];
    float rayleigh_exponential_distribution; /* km */
    float rayleigh_scattering_scale;         /* 1/km */
    float rayleigh_scattering[3];
    float mie_exponential_distribution; /* km */
    float mie_phase_g;
    float mie_scattering_scale; /* 1/km */
    float mie_scattering[3];
    float mie_absorption_scale; /* 1/km */
    float mie_absorption[3];
    float ozone_center_altitude; /* km */
    float ozone_width;           /* km */
    float ozone_absorption_scale; /* 1/km */
    float ozone_absorption[3];
    float transmittance_steps;
    float multiscattering_steps;
    float multiscattering_mask; /* 0..1 */
} skyr_atmosphere_parameters;

/* Fill `p` with the reference defaults (src/SkyRendering/Atmosphere.h:13-38). */
int skyr_atmosphere_parameters_default(skyr_atmosphere_parameters* p);

/* View-dependent part of AtmosphereRenderParameters
 * (src/SkyRendering/AtmosphereRenderer.h:12-35) plus the camera inputs that
 * AtmosphereRenderer::Render derives its frame from
 * (src/SkyRendering/AtmosphereRenderer.cpp:52-83). */
typedef struct skyr_atmosphere_render_parameters {
    float sun_direction_theta; /* zenith angle, degrees */
    float sun_direction_phi;   /* azimuth, degrees */
    float sky_view_lut_steps;
    float aerial_perspective_lut_steps;
    float aerial_perspective_lut_max_distance; /* km */
    float camera_position[3];  /* world space, y up, km; Earth centre at (0, -bottom_radius, 0) */
    float view_projection[16]; /* column-major (glm::mat4 memory order) */
} skyr_atmosphere_render_parameters;

/* Sizes of every LUT.  Reference sizes: transmittance 256x64
 * (src/SkyRendering/Atmosphere.cpp:9-15), multi-scattering 32x32 (:17-19),
 * sky-view 128x128 (src/SkyRendering/AtmosphereRenderer.cpp:15-17),
 * aerial perspective 32x32xdepth (:19-21, depth from
 * AtmosphereRenderInitParameters::aerial_perspective_lut_depth). */
typedef struct skyr_lut_sizes {
    int transmittance_width, transmittance_height;
    int multiscattering_width, multiscattering_height;
    int sky_view_width, sky_view_height;
    int aerial_perspective_width, aerial_perspective_height, aerial_perspective_depth;
    int format; /* SKYR_FORMAT_* of the multi-scattering, sky-view and AP outputs;
                   the transmittance LUT is always RGBA32F (grazing-ray
                   transmittance falls below the FP16 normal range). */
} skyr_lut_sizes;

/* Bytes of one LUT of `kind` (SKYR_LUT_*) for one parameter set. */
#define SKYR_LUT_TRANSMITTANCE 0
#define SKYR_LUT_MULTISCATTERING 1
#define SKYR_LUT_SKY_VIEW 2
#define SKYR_LUT_AERIAL_PERSPECTIVE 3
size_t skyr_lut_bytes(const skyr_lut_sizes* sizes, int kind);

/* Atmosphere::UpdateLuts (src/SkyRendering/Atmosphere.cpp:101-124):
 * regenerate the transmittance and multi-scattering LUTs of `n_sets`
 * parameter sets.  Outputs are device buffers holding n_sets consecutive LUTs:
 *   transmittance   : RGBA32F, rgb = T to the top boundary, a = 1
 *   multiscattering : `sizes->format`, rgb = Psi_ms, a = 1              */
int skyr_update_luts(skyr_ctx* ctx, const skyr_atmosphere_parameters* params, int n_sets,
                     const skyr_lut_sizes* sizes, void* transmittance, void* multiscattering);

/* The SKY_VIEW and AERIAL_PERSPECTIVE passes of AtmosphereRenderer::Render
 * (src/SkyRendering/AtmosphereRenderer.cpp:221-233,
 *  shaders/SkyRendering/AtmosphereRenderer.glsl:147-245) for `n_sets` views;
 * view i uses params[i], render[i] and the i-th transmittance /
 * multi-scattering LUT.  Outputs (device, n_sets consecutive images):
 *   sky_view_luminance, sky_view_transmittance        : W x H, a = 0
 *   aerial_perspective_luminance, ..._transmittance   : W x H x D, a = 0  */
int skyr_render_view_luts(skyr_ctx* ctx, const skyr_atmosphere_parameters* params,
                          const skyr_atmosphere_render_parameters* render, int n_sets,
                          const skyr_lut_sizes* sizes, const void* transmittance,
                          const void* multiscattering, void* sky_view_luminance,
                          void* sky_view_transmittance, void* aerial_perspective_luminance,
                          void* aerial_perspective_transmittance);

/* The whole LUT set of Earth::Update + the LUT passes of AtmosphereRenderer::Render
 * for `n_sets` (parameter set, view) pairs in one stream-ordered launch sequence:
 * transmittance -> multi-scattering -> {sky-view, aerial perspective}.
 * Same buffers and layouts as the two calls above. */
int skyr_update_lut_set(skyr_ctx* ctx, const skyr_atmosphere_parameters* params,
                        const skyr_atmosphere_render_parameters* render, int n_sets,
                        const skyr_lut_sizes* sizes, void* transmittance, void* multiscattering,
                        void* sky_view_luminance, void* sky_view_transmittance,
                        void* aerial_perspective_luminance, void* aerial_perspective_transmittance);

/* Allocation-free form of skyr_update_lut_set, for callers that cannot let the
 * library allocate device memory: hosts that own every device allocation
 * through their own pool or budget, or frame loops that must not take
 * cudaMalloc / cudaFree (cudaFree synchronises the device).  Same arguments,
 * outputs and results as skyr_update_lut_set (a sky-view or aerial-perspective
 * output pair may be left out, as there); the caller still allocates the
 * outputs.  The per-set kernel constants go to a static device table of this
 * library (SKYR_NOALLOC_MAX_SETS sets, under 100 KB, held by every GPU that
 * loads the library until exit) instead of a cudaMalloc'ed one:
 *   - n_sets above SKYR_NOALLOC_MAX_SETS is rejected with SKYR_EINVAL;
 *   - every set is validated before anything is copied, so a rejected call
 *     leaves the table as it was;
 *   - each call derives the constants on the host and copies them into the
 *     table with cudaMemcpyAsync on the context's stream;
 *   - the first call on a device looks up the table's device address
 *     (cudaGetSymbolAddress) and should come before any stream capture; the
 *     address is kept until exit, so cudaDeviceReset is not supported while
 *     the library is loaded;
 *   - every call shares the one table, so calls whose GPU work overlaps
 *     (two streams or contexts at once) race.
 * No counterpart in the reference. */
#define SKYR_NOALLOC_MAX_SETS 256
int skyr_update_lut_set_noalloc(skyr_ctx* ctx, const skyr_atmosphere_parameters* params,
                                const skyr_atmosphere_render_parameters* render, int n_sets,
                                const skyr_lut_sizes* sizes, void* transmittance, void* multiscattering,
                                void* sky_view_luminance, void* sky_view_transmittance,
                                void* aerial_perspective_luminance, void* aerial_perspective_transmittance);

#ifdef __cplusplus
}
#endif
#endif /* SKYR_H_ */
