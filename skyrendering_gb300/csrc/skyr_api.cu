// skyr_api.cu — C ABI entry points: context, status reporting, validation,
// host-side derivation of kernel constants and the LUT dispatch.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "atmosphere_kernels.cuh"
#include "skyr_ctx.cuh"

namespace {
thread_local char g_last_error[512] = "";
}

size_t skyr_struct_size_ext(int which);  // later modules (skyr_modules.cu)

namespace skyr {

int set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

int check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return SKYR_OK;
    if (e == cudaErrorMemoryAllocation)
        return set_error(SKYR_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
    return set_error(SKYR_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

int ensure_job_table(skyr_ctx* ctx, size_t bytes) {
    if (ctx->job_table_bytes >= bytes) return SKYR_OK;
    if (ctx->job_table) {
        cudaError_t e = cudaFree(ctx->job_table);
        ctx->job_table = nullptr;
        ctx->job_table_bytes = 0;
        if (e != cudaSuccess) return check_cuda(e, "cudaFree(job table)");
    }
    size_t cap = bytes < 4096 ? 4096 : bytes;
    cudaError_t e = cudaMalloc(&ctx->job_table, cap);
    if (e != cudaSuccess) return check_cuda(e, "cudaMalloc(job table)");
    ctx->job_table_bytes = cap;
    return SKYR_OK;
}

}  // namespace skyr

using namespace skyr;

// ---------------------------------------------------------------------------
// Host derivations (double precision, cast once)
// ---------------------------------------------------------------------------
namespace {

struct D3 {
    double x, y, z;
};
D3 d3(const float* f) { return {f[0], f[1], f[2]}; }
D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
D3 scale(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
double dlen(D3 a) { return std::sqrt(ddot(a, a)); }
D3 dcross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float3 tof(D3 a) { return make_float3((float)a.x, (float)a.y, (float)a.z); }

// FromThetaPhiToDirection (src/Base/src/Utils.cpp:23-31)
D3 theta_phi(double theta, double phi) {
    return {std::cos(phi) * std::sin(theta), std::cos(theta), std::sin(phi) * std::sin(theta)};
}

bool invert4(const double* m, double* out) {  // column-major, Gauss-Jordan
    double w[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            w[r][c] = m[c * 4 + r];
            w[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(w[r][c]) > std::fabs(w[p][c])) p = r;
        if (w[p][c] == 0.0) return false;
        if (p != c)
            for (int k = 0; k < 8; ++k) std::swap(w[c][k], w[p][k]);
        double inv = 1.0 / w[c][c];
        for (int k = 0; k < 8; ++k) w[c][k] *= inv;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            double f = w[r][c];
            for (int k = 0; k < 8; ++k) w[r][k] -= f * w[c][k];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = w[r][c + 4];
    return true;
}

bool finite_all(const float* f, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(f[i])) return false;
    return true;
}

}  // namespace

namespace skyr {

// AssignBufferData (src/SkyRendering/Atmosphere.cpp:49-70)
void derive_atmo_consts(const skyr_atmosphere_parameters& p, AtmoConsts& a) {
    std::memset(&a, 0, sizeof(a));
    a.solar_illuminance = make_float3(p.solar_illuminance[0], p.solar_illuminance[1], p.solar_illuminance[2]);
    a.sun_angular_radius = (float)((double)p.sun_angular_radius * M_PI / 180.0);
    a.rayleigh_scattering = tof(scale(d3(p.rayleigh_scattering), p.rayleigh_scattering_scale));
    a.mie_scattering = tof(scale(d3(p.mie_scattering), p.mie_scattering_scale));
    D3 mie_abs = scale(d3(p.mie_absorption), p.mie_absorption_scale);
    D3 mie_sca = scale(d3(p.mie_scattering), p.mie_scattering_scale);
    a.mie_extinction = tof({mie_sca.x + mie_abs.x, mie_sca.y + mie_abs.y, mie_sca.z + mie_abs.z});
    a.ozone_absorption = tof(scale(d3(p.ozone_absorption), p.ozone_absorption_scale));
    a.inv_rayleigh_h = (float)(1.0 / p.rayleigh_exponential_distribution);
    a.inv_mie_h = (float)(1.0 / p.mie_exponential_distribution);
    a.ozone_center = p.ozone_center_altitude;
    a.inv_ozone_width = (float)(1.0 / p.ozone_width);
    a.ground_albedo = make_float3(p.ground_albedo[0], p.ground_albedo[1], p.ground_albedo[2]);
    a.mie_g = p.mie_phase_g;
    a.ms_mask = p.multiscattering_mask;
    double R = p.bottom_radius, th = p.thickness, top = R + th;
    a.R = (float)R;
    a.top = (float)top;
    a.thickness = (float)th;
    a.R2 = (float)(R * R);
    a.top2_minus_R2 = (float)(th * (2.0 * R + th));
    a.Hh = (float)std::sqrt(th * (2.0 * R + th));
    a.transmittance_steps = p.transmittance_steps;
    a.multiscattering_steps = p.multiscattering_steps;
    double g = p.mie_phase_g;
    a.mie_phase_k = (float)(3.0 / (8.0 * M_PI) * (1.0 - g * g) / (2.0 + g * g));
    a.inv_Hh = (float)(1.0 / std::sqrt(th * (2.0 * R + th)));
    a.inv_thickness = (float)(1.0 / th);
    double alpha = (double)p.sun_angular_radius * M_PI / 180.0;
    a.inv_2R_alpha = alpha > 0.0 ? (float)(1.0 / (2.0 * R * alpha)) : 3.0e38f;
}

// AssignBufferData (src/SkyRendering/AtmosphereRenderer.cpp:52-83)
void derive_view_consts(const skyr_atmosphere_parameters& p, const skyr_atmosphere_render_parameters& r,
                        ViewConsts& v) {
    std::memset(&v, 0, sizeof(v));
    const double deg = M_PI / 180.0;
    D3 sun = theta_phi(r.sun_direction_theta * deg, r.sun_direction_phi * deg);
    double R = p.bottom_radius, top = R + (double)p.thickness;
    D3 center{0.0, -R, 0.0};
    D3 cam = d3(r.camera_position);
    D3 rel = sub(cam, center);
    double cam_r = dlen(rel);
    D3 up = scale(rel, 1.0 / cam_r);
    D3 right = dcross(sun, up);
    double rl = dlen(right);
    if (rl != 0.0) {
        right = scale(right, 1.0 / rl);
    } else {
        D3 biased = theta_phi((r.sun_direction_theta + 90.0) * deg, r.sun_direction_phi * deg);
        right = dcross(biased, up);
        right = scale(right, 1.0 / dlen(right));
    }
    D3 front = dcross(up, right);
    // cam_r - R without cancellation: |rel|^2 - R^2 = x^2 + z^2 + (y+R)^2 - R^2
    double y = (double)r.camera_position[1];
    double rho2 = cam.x * cam.x + cam.z * cam.z + y * (y + 2.0 * R);
    v.sun = tof(sun);
    v.up = tof(up);
    v.right = tof(right);
    v.front = tof(front);
    v.cam_r = (float)cam_r;
    v.cam_rho2 = (float)rho2;
    v.cam_h = (float)(rho2 / (cam_r + R));
    v.sky_view_steps = r.sky_view_lut_steps;
    v.ap_steps = r.aerial_perspective_lut_steps;
    v.ap_max_distance = r.aerial_perspective_lut_max_distance;
    v.in_space = cam_r > top ? 1.f : 0.f;
    double vp[16], ivp[16];
    for (int i = 0; i < 16; ++i) vp[i] = r.view_projection[i];
    if (!invert4(vp, ivp))
        for (int i = 0; i < 16; ++i) ivp[i] = (i % 5 == 0) ? 1.0 : 0.0;
    auto col = [&](int c) { return D3{ivp[c * 4 + 0], ivp[c * 4 + 1], ivp[c * 4 + 2]}; };
    auto colw = [&](int c) { return ivp[c * 4 + 3]; };
    v.ap_a0 = tof(sub(col(0), scale(cam, colw(0))));
    v.ap_a1 = tof(sub(col(1), scale(cam, colw(1))));
    v.ap_a3 = tof(sub(col(3), scale(cam, colw(3))));
    v.ap_w0 = (float)colw(0);
    v.ap_w1 = (float)colw(1);
    v.ap_w3 = (float)colw(3);
}

int validate_atmosphere(const skyr_atmosphere_parameters* p, int i) {
    if (!finite_all(reinterpret_cast<const float*>(p), sizeof(*p) / sizeof(float)))
        return set_error(SKYR_EINVAL, "atmosphere parameters[%d]: non-finite value", i);
    if (!(p->bottom_radius > 0.f) || !(p->thickness > 0.f))
        return set_error(SKYR_EINVAL, "atmosphere parameters[%d]: bottom_radius and thickness must be > 0", i);
    if (!(p->rayleigh_exponential_distribution > 0.f) || !(p->mie_exponential_distribution > 0.f) ||
        !(p->ozone_width > 0.f))
        return set_error(SKYR_EINVAL, "atmosphere parameters[%d]: scale heights and ozone width must be > 0", i);
    if (!(p->transmittance_steps > 0.f) || !(p->multiscattering_steps > 0.f) || p->transmittance_steps > 4096.f ||
        p->multiscattering_steps > 4096.f)
        return set_error(SKYR_EINVAL, "atmosphere parameters[%d]: step counts must be in (0, 4096]", i);
    if (!(std::fabs(p->mie_phase_g) < 1.f))
        return set_error(SKYR_EINVAL, "atmosphere parameters[%d]: |mie_phase_g| must be < 1", i);
    return SKYR_OK;
}

int validate_render(const skyr_atmosphere_render_parameters* r, const skyr_atmosphere_parameters* p, int i) {
    if (!finite_all(reinterpret_cast<const float*>(r), sizeof(*r) / sizeof(float)))
        return set_error(SKYR_EINVAL, "render parameters[%d]: non-finite value", i);
    if (!(r->sky_view_lut_steps > 0.f) || !(r->aerial_perspective_lut_steps > 0.f) ||
        r->sky_view_lut_steps > 4096.f || r->aerial_perspective_lut_steps > 4096.f)
        return set_error(SKYR_EINVAL, "render parameters[%d]: step counts must be in (0, 4096]", i);
    if (!(r->aerial_perspective_lut_max_distance > 0.f))
        return set_error(SKYR_EINVAL, "render parameters[%d]: aerial_perspective_lut_max_distance must be > 0", i);
    double x = r->camera_position[0], y = r->camera_position[1], z = r->camera_position[2];
    double R = p->bottom_radius;
    if (x * x + z * z + y * (y + 2.0 * R) < 0.0)
        return set_error(SKYR_EINVAL, "render parameters[%d]: camera below the ground sphere", i);
    return SKYR_OK;
}

int validate_sizes(const skyr_lut_sizes* s, bool views) {
    if (!s) return set_error(SKYR_EINVAL, "null skyr_lut_sizes");
    auto ok = [](int v) { return v >= 2 && v <= 8192; };
    if (!ok(s->transmittance_width) || !ok(s->transmittance_height) || !ok(s->multiscattering_width) ||
        !ok(s->multiscattering_height))
        return set_error(SKYR_EINVAL, "LUT sizes must be in [2, 8192]");
    if (views && (!ok(s->sky_view_width) || !ok(s->sky_view_height) || !ok(s->aerial_perspective_width) ||
                  !ok(s->aerial_perspective_height) || !ok(s->aerial_perspective_depth)))
        return set_error(SKYR_EINVAL, "view LUT sizes must be in [2, 8192]");
    if (s->format != SKYR_FORMAT_RGBA32F && s->format != SKYR_FORMAT_RGBA16F)
        return set_error(SKYR_EINVAL, "unknown LUT format %d", s->format);
    return SKYR_OK;
}

}  // namespace skyr

// ---------------------------------------------------------------------------
// LUT dispatch
// ---------------------------------------------------------------------------
namespace {

constexpr int kMaxSets = 1 << 16;

int build_jobs(skyr_ctx* ctx, const skyr_atmosphere_parameters* params, const skyr_atmosphere_render_parameters* rp,
               int n, std::vector<LutSetJob>& jobs) {
    jobs.resize(n);
    if (int st = skyr::derive_jobs(params, rp, n, jobs.data())) return st;
    if (n > 1) {
        int st = ensure_job_table(ctx, sizeof(LutSetJob) * n);
        if (st) return st;
        st = check_cuda(cudaMemcpyAsync(ctx->job_table, jobs.data(), sizeof(LutSetJob) * n, cudaMemcpyHostToDevice,
                                        ctx->stream),
                        "upload job table");
        if (st) return st;
    }
    return SKYR_OK;
}

template <class S, bool TABLE>
int run(skyr_ctx* ctx, JobSrc<TABLE> src, int n, const skyr_lut_sizes& s, bool do_base, bool do_view, float4* T,
        S* MS, S* svl, S* svt, S* apl, S* apt) {
    cudaStream_t st = ctx->stream;
    if (do_base) {
        int e = check_cuda(launch_transmittance<TABLE>(src, n, s, T, st, ctx->tuning.transmittance_lanes),
                           "transmittance kernel");
        if (e) return e;
        e = check_cuda(launch_multiscattering<S, TABLE>(src, n, s, T, MS, st), "multiscattering kernel");
        if (e) return e;
    }
    if (do_view) {
        skyr_lut_sizes v = s;
        if (!svl) v.sky_view_width = v.sky_view_height = 0;
        if (!apl) v.aerial_perspective_width = v.aerial_perspective_height = v.aerial_perspective_depth = 0;
        return check_cuda(launch_view_luts<S, TABLE>(src, n, v, T, MS, svl, svt, apl, apt, st, ctx->tuning.view_lanes),
                          "view LUT kernel");
    }
    return SKYR_OK;
}

template <class S>
int dispatch_fmt(skyr_ctx* ctx, const std::vector<LutSetJob>& jobs, int n, const skyr_lut_sizes& s, bool do_base,
                 bool do_view, void* T, void* MS, void* svl, void* svt, void* apl, void* apt) {
    auto c = [](void* p) { return reinterpret_cast<S*>(p); };
    if (n == 1) {
        JobSrc<false> src{jobs[0]};
        return run<S, false>(ctx, src, n, s, do_base, do_view, reinterpret_cast<float4*>(T), c(MS), c(svl), c(svt),
                             c(apl), c(apt));
    }
    JobSrc<true> src{reinterpret_cast<const LutSetJob*>(ctx->job_table)};
    return run<S, true>(ctx, src, n, s, do_base, do_view, reinterpret_cast<float4*>(T), c(MS), c(svl), c(svt),
                        c(apl), c(apt));
}

int lut_entry(skyr_ctx* ctx, const skyr_atmosphere_parameters* params, const skyr_atmosphere_render_parameters* rp,
              int n, const skyr_lut_sizes* sizes, bool do_base, bool do_view, void* T, void* MS, void* svl, void* svt,
              void* apl, void* apt) {
    if (!ctx) return set_error(SKYR_EINVAL, "null context");
    if (!params) return set_error(SKYR_EINVAL, "null atmosphere parameters");
    if (n <= 0 || n > kMaxSets) return set_error(SKYR_EINVAL, "n_sets must be in [1, %d]", kMaxSets);
    int st = validate_sizes(sizes, do_view);
    if (st) return st;
    if (!T || !MS) return set_error(SKYR_EINVAL, "null transmittance or multi-scattering buffer");
    if (do_view) {
        if (!rp) return set_error(SKYR_EINVAL, "null render parameters");
        if ((svl == nullptr) != (svt == nullptr) || (apl == nullptr) != (apt == nullptr))
            return set_error(SKYR_EINVAL, "luminance and transmittance outputs must be given together");
        if (!svl && !apl) return set_error(SKYR_EINVAL, "no view LUT output given");
    }
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    std::vector<LutSetJob> jobs;
    st = build_jobs(ctx, params, do_view ? rp : nullptr, n, jobs);
    if (st) return st;
    if (sizes->format == SKYR_FORMAT_RGBA16F)
        return dispatch_fmt<__half2>(ctx, jobs, n, *sizes, do_base, do_view, T, MS, svl, svt, apl, apt);
    return dispatch_fmt<float4>(ctx, jobs, n, *sizes, do_base, do_view, T, MS, svl, svt, apl, apt);
}

}  // namespace

namespace skyr {

int derive_jobs(const skyr_atmosphere_parameters* params, const skyr_atmosphere_render_parameters* rp, int n,
                LutSetJob* jobs) {
    for (int i = 0; i < n; ++i) {
        int st = validate_atmosphere(&params[i], i);
        if (st) return st;
        derive_atmo_consts(params[i], jobs[i].a);
        if (rp) {
            st = validate_render(&rp[i], &params[i], i);
            if (st) return st;
            derive_view_consts(params[i], rp[i], jobs[i].v);
        } else {
            std::memset(&jobs[i].v, 0, sizeof(ViewConsts));
        }
    }
    return SKYR_OK;
}

int launch_lut_passes(skyr_ctx* ctx, const LutSetJob* table, int n, const skyr_lut_sizes& s, bool do_view, void* T,
                      void* MS, void* svl, void* svt, void* apl, void* apt) {
    JobSrc<true> src{table};
    if (s.format == SKYR_FORMAT_RGBA16F)
        return run<__half2, true>(ctx, src, n, s, true, do_view, reinterpret_cast<float4*>(T),
                                  reinterpret_cast<__half2*>(MS), reinterpret_cast<__half2*>(svl),
                                  reinterpret_cast<__half2*>(svt), reinterpret_cast<__half2*>(apl),
                                  reinterpret_cast<__half2*>(apt));
    return run<float4, true>(ctx, src, n, s, true, do_view, reinterpret_cast<float4*>(T),
                             reinterpret_cast<float4*>(MS), reinterpret_cast<float4*>(svl),
                             reinterpret_cast<float4*>(svt), reinterpret_cast<float4*>(apl),
                             reinterpret_cast<float4*>(apt));
}

}  // namespace skyr

extern "C" {

int skyr_abi_version(void) { return SKYR_ABI_VERSION; }

size_t skyr_struct_size(int which) {
    switch (which) {
        case 0: return sizeof(skyr_atmosphere_parameters);
        case 1: return sizeof(skyr_atmosphere_render_parameters);
        case 2: return sizeof(skyr_lut_sizes);
        default: return skyr_struct_size_ext(which);
    }
}

const char* skyr_status_string(int status) {
    switch (status) {
        case SKYR_OK: return "SKYR_OK";
        case SKYR_EINVAL: return "SKYR_EINVAL";
        case SKYR_ENOMEM: return "SKYR_ENOMEM";
        case SKYR_ECUDA: return "SKYR_ECUDA";
        case SKYR_ETIMEOUT: return "SKYR_ETIMEOUT";
        case SKYR_ENOTSUP: return "SKYR_ENOTSUP";
        default: return "SKYR_UNKNOWN";
    }
}

const char* skyr_last_error(void) { return g_last_error; }

int skyr_ctx_create(void* cuda_stream, skyr_ctx** out_ctx) {
    if (!out_ctx) return set_error(SKYR_EINVAL, "null out_ctx");
    *out_ctx = nullptr;
    int dev = 0;
    if (int e = check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return e;
    skyr_ctx* c = new (std::nothrow) skyr_ctx();
    if (!c) return set_error(SKYR_ENOMEM, "host allocation of skyr_ctx failed");
    c->stream = reinterpret_cast<cudaStream_t>(cuda_stream);
    c->device = dev;
    *out_ctx = c;
    return SKYR_OK;
}

int skyr_ctx_destroy(skyr_ctx* ctx) {
    if (!ctx) return SKYR_OK;
    int st = SKYR_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream); else cudaDeviceSynchronize();
    ctx_release_resources(ctx);
    if (ctx->job_table) st = check_cuda(cudaFree(ctx->job_table), "cudaFree(job table)");
    delete ctx;
    return st;
}

int skyr_ctx_synchronize(skyr_ctx* ctx) {
    if (!ctx) return set_error(SKYR_EINVAL, "null context");
    cudaSetDevice(ctx->device);
    return check_cuda(ctx->stream ? cudaStreamSynchronize(ctx->stream) : cudaDeviceSynchronize(), "synchronize");
}

int skyr_atmosphere_parameters_default(skyr_atmosphere_parameters* p) {
    if (!p) return set_error(SKYR_EINVAL, "null parameters");
    // AtmosphereParameters defaults (src/SkyRendering/Atmosphere.h:13-38)
    *p = skyr_atmosphere_parameters{};
    p->solar_illuminance[0] = p->solar_illuminance[1] = p->solar_illuminance[2] = 1.f;
    p->sun_angular_radius = 0.5334f * 0.5f;
    p->bottom_radius = 6360.f;
    p->thickness = 6420.f - 6360.f;
    p->ground_albedo[0] = p->ground_albedo[1] = p->ground_albedo[2] = 0.4f;
    p->rayleigh_exponential_distribution = 8.f;
    p->rayleigh_scattering_scale = 0.0331f;
    p->rayleigh_scattering[0] = 0.175287f;
    p->rayleigh_scattering[1] = 0.409607f;
    p->rayleigh_scattering[2] = 1.f;
    p->mie_exponential_distribution = 1.2f;
    p->mie_phase_g = 0.8f;
    p->mie_scattering_scale = 0.003996f;
    p->mie_scattering[0] = p->mie_scattering[1] = p->mie_scattering[2] = 1.f;
    p->mie_absorption_scale = 0.000444f;
    p->mie_absorption[0] = p->mie_absorption[1] = p->mie_absorption[2] = 1.f;
    p->ozone_center_altitude = 25.f;
    p->ozone_width = 15.f;
    p->ozone_absorption_scale = 0.001881f;
    p->ozone_absorption[0] = 0.345561f;
    p->ozone_absorption[1] = 1.f;
    p->ozone_absorption[2] = 0.045189f;
    p->transmittance_steps = 40.f;
    p->multiscattering_steps = 30.f;
    p->multiscattering_mask = 1.f;
    return SKYR_OK;
}

size_t skyr_lut_bytes(const skyr_lut_sizes* s, int kind) {
    if (!s) return 0;
    size_t texel = s->format == SKYR_FORMAT_RGBA16F ? 8 : 16;
    switch (kind) {
        case SKYR_LUT_TRANSMITTANCE: return (size_t)s->transmittance_width * s->transmittance_height * 16;
        case SKYR_LUT_MULTISCATTERING: return (size_t)s->multiscattering_width * s->multiscattering_height * texel;
        case SKYR_LUT_SKY_VIEW: return (size_t)s->sky_view_width * s->sky_view_height * texel;
        case SKYR_LUT_AERIAL_PERSPECTIVE:
            return (size_t)s->aerial_perspective_width * s->aerial_perspective_height * s->aerial_perspective_depth *
                   texel;
        default: return 0;
    }
}

int skyr_update_luts(skyr_ctx* ctx, const skyr_atmosphere_parameters* params, int n_sets, const skyr_lut_sizes* sizes,
                     void* transmittance, void* multiscattering) {
    return lut_entry(ctx, params, nullptr, n_sets, sizes, true, false, transmittance, multiscattering, nullptr,
                     nullptr, nullptr, nullptr);
}

int skyr_render_view_luts(skyr_ctx* ctx, const skyr_atmosphere_parameters* params,
                          const skyr_atmosphere_render_parameters* render, int n_sets, const skyr_lut_sizes* sizes,
                          const void* transmittance, const void* multiscattering, void* sky_view_luminance,
                          void* sky_view_transmittance, void* aerial_perspective_luminance,
                          void* aerial_perspective_transmittance) {
    return lut_entry(ctx, params, render, n_sets, sizes, false, true, const_cast<void*>(transmittance),
                     const_cast<void*>(multiscattering), sky_view_luminance, sky_view_transmittance,
                     aerial_perspective_luminance, aerial_perspective_transmittance);
}

int skyr_update_lut_set(skyr_ctx* ctx, const skyr_atmosphere_parameters* params,
                        const skyr_atmosphere_render_parameters* render, int n_sets, const skyr_lut_sizes* sizes,
                        void* transmittance, void* multiscattering, void* sky_view_luminance,
                        void* sky_view_transmittance, void* aerial_perspective_luminance,
                        void* aerial_perspective_transmittance) {
    return lut_entry(ctx, params, render, n_sets, sizes, true, true, transmittance, multiscattering,
                     sky_view_luminance, sky_view_transmittance, aerial_perspective_luminance,
                     aerial_perspective_transmittance);
}

}  // extern "C"
