// cloud.cu — the volumetric-cloud raymarch (VolumetricCloudRender.comp) with
// the material plug-ins (SampleSigmaT) for sm_103a.
//
// One thread per pixel, each warp an 8x4 pixel tile so that the rays of a warp
// stay coherent through the cloud layer (their texture reads share cache lines).
// Texture filtering is done in software in FP32 with GL's exact rules (hardware
// texture units interpolate with 8-bit weights).  The shell intersections use
// cancellation-free FP32 forms; all frame derivations are done on the host in
// double.
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <cstring>

#include "atmosphere_kernels.cuh"
#include "cloud_internal.cuh"
#include "cloud_material.cuh"
#include "cloud_march.cuh"
#include "lut_access.cuh"
#include "skyr_ctx.cuh"

namespace skyr {

// ---------------------------------------------------------------------------
// Host derivation
// ---------------------------------------------------------------------------
namespace {
struct D3 {
    double x, y, z;
};
D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
D3 add(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
D3 mul(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
double dotd(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
D3 crossd(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
D3 normd(D3 a) { return mul(a, 1.0 / std::sqrt(dotd(a, a))); }
float3 tof(D3 a) { return make_float3((float)a.x, (float)a.y, (float)a.z); }
}  // namespace

bool invert4d(const double* m, double* out) {
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
        double iv = 1.0 / w[c][c];
        for (int k = 0; k < 8; ++k) w[c][k] *= iv;
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

void matmul4d(const double* a, const double* b, double* c) {  // column-major c = a b
    for (int r = 0; r < 4; ++r)
        for (int col = 0; col < 4; ++col) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + r] * b[col * 4 + k];
            c[col * 4 + r] = s;
        }
}

// The local z-up frame of VolumetricCloud::Update (VolumetricCloud.cpp:188-201):
// columns front, right, up and the surface point below the camera.
void cloud_local_frame(double R, const float cam_world[3], double model[16]) {
    D3 center{0.0, -R, 0.0};
    D3 cam{cam_world[0], cam_world[1], cam_world[2]};
    D3 up = normd(sub(cam, center));
    D3 origin = add(center, mul(up, R));
    D3 front = normd(crossd(up, D3{1.0, 0.0, 0.0}));
    D3 right = normd(crossd(up, front));
    const double m[16] = {front.x, front.y, front.z, 0, right.x, right.y, right.z, 0,
                          up.x,    up.y,    up.z,    0, origin.x, origin.y, origin.z, 1};
    for (int i = 0; i < 16; ++i) model[i] = m[i];
}

namespace {

int fill_tex(DTex& t, const void* p, const skyr_noise_texture_desc& d, bool border, bool required,
             const char* what, const void* ex, int ex_channels) {
    std::memset(&t, 0, sizeof(t));
    if (!p) {
        if (required) return set_error(SKYR_EINVAL, "material needs the %s texture", what);
        t.w = t.h = t.d = t.levels = 1;
        return SKYR_OK;
    }
    if (int st = validate_noise_desc(&d, false)) return st;
    t.base = reinterpret_cast<const uint8_t*>(p);
    t.w = d.width;
    t.h = d.height;
    t.d = d.depth;
    t.levels = noise_levels(&d);
    if (t.levels > kMaxLevels) return set_error(SKYR_EINVAL, "%s texture has too many mip levels", what);
    t.border = border ? 1 : 0;
    t.channels = d.channels;
    if (ex) {
        if (ex_channels < 1 || ex_channels > d.channels)
            return set_error(SKYR_EINVAL, "%s expanded texture: bad channel count %d", what, ex_channels);
        if (d.depth > 1 && (d.width < 2 || d.height < 2))
            return set_error(SKYR_EINVAL, "%s expanded texture: 3D needs width, height >= 2", what);
        t.ex = ex;
        t.ex_channels = ex_channels;
    }
    return SKYR_OK;
}
}  // namespace

// The constants of the specialised density evaluation (cloud_fast.cuh), and
// whether it applies: Material1, NEAREST_MIPMAP_NEAREST minification on both
// textures, REPEAT, for each texture a hardware sampler or the expanded level 0,
// a square cloud map and a cubic detail texture.
static void derive_fast_consts(const skyr_cloud_material& m, const skyr_cloud_textures& tex,
                               const skyr_cloud_parameters& cp, double R, MaterialConsts& mc, double tan_half,
                               double vmin) {
    mc.fast_ok = 0;
    // the height series holds while |rho2| / R^2 <= 0.02 for every sample: the primary samples lie in the
    // layer, the light-march samples within shadow_distance of it
    const double h_hi = (double)cp.bottom_altitude + cp.thickness + cp.shadow_distance,
                 h_lo = (double)cp.bottom_altitude - cp.shadow_distance;
    const double x_max = std::max(std::fabs(h_hi * (2.0 * R + h_hi)), std::fabs(h_lo * (2.0 * R + h_lo))) / (R * R);
    if (!(x_max <= 0.02)) return;
    const skyr_noise_texture_desc &cd = tex.cloud_map_desc, &dd = tex.detail_desc;
    if (m.type != SKYR_MATERIAL_DEFAULT1 || m.minfilter2d != SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST ||
        m.minfilter3d != SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST || !(mc.cloud_map_tex.ex || tex.cloud_map_sampler) ||
        !(mc.detail_tex.ex || tex.detail_sampler) || mc.cloud_map_tex.border || mc.detail_tex.border ||
        cd.width != cd.height || cd.depth != 1 || dd.width != dd.height || dd.width != dd.depth || dd.depth < 2)
        return;
    auto fill = [&](FastTex& t, const DTex& d, const skyr_noise_texture_desc& desc, double repeat,
                    uint64_t sampler, uint64_t sampler_nearest) {
        t.base = d.base;
        t.ex = d.ex;
        t.tex = sampler;
        t.tex_near = sampler_nearest;
        t.w = desc.width;
        t.h = desc.height;
        t.d = desc.depth;
        t.last = d.levels - 1;
        t.fw = (float)desc.width;
        t.fh = (float)desc.height;
        t.fd = (float)desc.depth;
        // CalKLod (VolumetricCloudDefaultMaterial.cpp:24-28) in double
        double maxw = std::max(desc.width, std::max(desc.height, desc.depth));
        double lod_k = std::log2(maxw * tan_half / (repeat * vmin)) + (double)m.lod_bias;
        t.lod_k = (float)lod_k;
        // lambda = 0.5 log2 d2 + lod_k <= 1/2  <=>  d2 <= 2^(1 - 2 lod_k)
        t.mag_d2 = (float)std::exp2(1.0 - 2.0 * lod_k);
        for (int l = 0; l < kMaxLevels; ++l)
            t.off[l] = l < d.levels ? (unsigned)noise_level_offset(&desc, l) : 0u;
    };
    FastConsts& f = mc.fast;
    fill(f.cm, mc.cloud_map_tex, cd, m.cloud_map_repeat_size, tex.cloud_map_sampler, tex.cloud_map_sampler_nearest);
    fill(f.dt, mc.detail_tex, dd, m.detail_repeat_size, tex.detail_sampler, tex.detail_sampler_nearest);
    // Material1's terms in 0..255 texel units (VolumetricCloudDefaultMaterial1.glsl:18-28)
    const double e = m.base_edge_hardness, hh = m.base_height_hardness;
    f.cov_a = (float)(e / 255.0);
    f.cov_b = (float)(-(double)m.base_density_threshold * e);
    f.hh_a = (float)-hh;
    f.hh_b = (float)hh;
    f.det_a = (float)((double)m.detail_scale / 255.0);
    f.det_b = (float)((double)m.detail_base * m.detail_scale);
    f.height_cut = mc.m1_height_cut;
    f.ec_a = (float)(-1.0 / 255.0);
    f.ec_b = m.edge_cut;
    f.density = m.density;
    const double inv_layer = 1.0 / cp.thickness;
    f.h_ir2 = (float)(1.0 / (R * R));
    f.h_k1 = (float)(inv_layer / (2.0 * R));
    f.h_k0 = (float)(-(double)cp.bottom_altitude * inv_layer);
    mc.fast_ok = 1;
}

// VolumetricCloud::Update (VolumetricCloud.cpp:168-280), the material Update
// (VolumetricCloudDefaultMaterial.cpp:84-101,451-463; VolumetricCloudVoxelMaterial.cpp:93-105)
// and CalKLod (VolumetricCloudDefaultMaterial.cpp:24-28).
int derive_cloud_consts(const skyr_atmosphere_parameters& atmo, const skyr_cloud_parameters& cp,
                        const skyr_cloud_material& m, const skyr_cloud_textures& tex, const skyr_cloud_view& v,
                        const skyr_lut_sizes& sizes, CloudConsts& c, MaterialConsts& mc) {
    std::memset(&c, 0, sizeof(c));
    std::memset(&mc, 0, sizeof(mc));
    const double deg = M_PI / 180.0;
    double R = atmo.bottom_radius;
    D3 center{0.0, -R, 0.0};
    D3 cam{v.camera_position[0], v.camera_position[1], v.camera_position[2]};
    D3 up = normd(sub(cam, center));
    D3 origin = add(center, mul(up, R));
    D3 front = normd(crossd(up, D3{1.0, 0.0, 0.0}));
    D3 right = normd(crossd(up, front));
    double model[16] = {front.x, front.y, front.z, 0, right.x, right.y, right.z, 0,
                        up.x,    up.y,    up.z,    0, origin.x, origin.y, origin.z, 1};
    double vp[16], mvp[16], imvp[16];
    for (int i = 0; i < 16; ++i) vp[i] = v.view_projection[i];
    matmul4d(vp, model, mvp);
    if (!invert4d(mvp, imvp)) return set_error(SKYR_EINVAL, "view_projection is singular");
    // local camera: the model is a rotation + translation, inverse = transpose
    D3 rel = sub(cam, origin);
    D3 cam_l{dotd(front, rel), dotd(right, rel), dotd(up, rel)};
    D3 sun_w{std::cos(v.sun_direction_phi * deg) * std::sin(v.sun_direction_theta * deg),
             std::cos(v.sun_direction_theta * deg),
             std::sin(v.sun_direction_phi * deg) * std::sin(v.sun_direction_theta * deg)};
    D3 sun_l = normd(D3{dotd(front, sun_w), dotd(right, sun_w), dotd(up, sun_w)});
    auto col = [&](int k) { return D3{imvp[k * 4 + 0], imvp[k * 4 + 1], imvp[k * 4 + 2]}; };
    auto colw = [&](int k) { return imvp[k * 4 + 3]; };
    c.a0 = tof(sub(col(0), mul(cam_l, colw(0))));
    c.a1 = tof(sub(col(1), mul(cam_l, colw(1))));
    c.a2 = tof(sub(col(2), mul(cam_l, colw(2))));
    c.af = tof(add(sub(col(2), mul(cam_l, colw(2))), sub(col(3), mul(cam_l, colw(3)))));
    c.w0 = (float)colw(0);
    c.w1 = (float)colw(1);
    c.w2 = (float)colw(2);
    c.wf = (float)(colw(2) + colw(3));
    c.a3 = tof(sub(col(3), mul(cam_l, colw(3))));
    c.w3 = (float)colw(3);
    c.cam = tof(cam_l);
    c.sun = tof(sun_l);
    c.R = (float)R;
    c.bottom = cp.bottom_altitude;
    c.top = (float)((double)cp.bottom_altitude + cp.thickness);
    c.rb = (float)(R + cp.bottom_altitude);
    c.rt = (float)(R + (double)cp.bottom_altitude + cp.thickness);
    c.inv_layer = (float)(1.0 / cp.thickness);
    {
        double b = cp.bottom_altitude, tp = (double)cp.bottom_altitude + cp.thickness, h = cam_l.z;
        c.rho2_bottom = (float)(b * (2.0 * R + b));
        c.rho2_top = (float)(tp * (2.0 * R + tp));
        c.cam_rho2 = (float)(h * (2.0 * R + h));
    }
    c.jitter_offset = (float)v.frame_id * 0.61803398875f;
    c.row_pivot = 0;  // march order: the identity until the launch sets it (march_order)
    c.row_dir = 1;
    c.sun_illuminance_scale = cp.sun_illuminance_scale;
    c.max_raymarch_distance = cp.max_raymarch_distance;
    c.max_raymarch_steps = cp.max_raymarch_steps;
    c.max_visible_distance = cp.max_visible_distance;
    c.env_color_scale = make_float3(cp.env_color[0] * cp.env_color_scale, cp.env_color[1] * cp.env_color_scale,
                                    cp.env_color[2] * cp.env_color_scale);
    c.shadow_steps = cp.shadow_steps;
    c.sun_ms_sigma_scale = cp.sun_multiscattering_sigma_scale;
    c.env_ms_sigma_scale = cp.env_multiscattering_sigma_scale;
    c.shadow_distance = cp.shadow_distance;
    c.env_bottom_visibility = cp.env_bottom_visibility;
    c.env_sun_height_curve_exp = cp.env_sun_height_curve_exp;
    c.g_fwd = cp.phase_g_forward;
    c.g_back = cp.phase_g_back;
    c.back_scale = cp.phase_back_scale;
    c.ap_max_distance = v.aerial_perspective_lut_max_distance;
    c.inv_ap_max_distance = (float)(1.0 / v.aerial_perspective_lut_max_distance);
    double cam_r = R + cam_l.z;
    c.atmo_in_space = cam_r > R + (double)atmo.thickness ? 1.f : 0.f;
    c.width = v.width;
    c.height = v.height;
    c.ap_w = sizes.aerial_perspective_width;
    c.ap_h = sizes.aerial_perspective_height;
    c.ap_d = sizes.aerial_perspective_depth;
    if (v.shadow_froxel) {
        if (v.shadow_froxel_width < 1 || v.shadow_froxel_height < 1 || v.shadow_froxel_depth < 1 ||
            v.shadow_froxel_width > 16384 || v.shadow_froxel_height > 16384 || v.shadow_froxel_depth > 4096)
            return set_error(SKYR_EINVAL, "shadow froxel size out of range");
        if (!(cp.shadow_froxel_max_distance > 0.f)) return set_error(SKYR_EINVAL, "bad shadow froxel max distance");
        c.froxel = v.shadow_froxel;
        c.fx_w = v.shadow_froxel_width;
        c.fx_h = v.shadow_froxel_height;
        c.fx_d = v.shadow_froxel_depth;
        c.inv_froxel_max_distance = (float)(1.0 / cp.shadow_froxel_max_distance);
    }

    mc.type = m.type;
    mc.min2d = m.minfilter2d;
    mc.min3d = m.minfilter3d;
    mc.mindisp = m.minfilter_displacement;
    double tan_half = std::tan(v.fovy * deg * 0.5);
    double vmin = std::min(v.viewport_width, v.viewport_height);
    auto info = [&](const skyr_noise_texture_desc& d, double repeat, double ox, double oy) {
        SampleInfoD s;
        s.frequency = (float)(1.0 / repeat);
        s.bias_x = (float)(ox / repeat - std::floor(ox / repeat));
        s.bias_y = (float)(oy / repeat - std::floor(oy / repeat));
        double maxw = std::max(d.width, std::max(d.height, d.depth));
        s.k_lod = (float)(maxw * tan_half / (repeat * vmin));
        return s;
    };
    double ox = m.offset_from_first[0], oy = m.offset_from_first[1];
    mc.cloud_map = info(tex.cloud_map_desc, m.cloud_map_repeat_size, ox, oy);
    mc.detail = info(tex.detail_desc, m.detail_repeat_size, ox + m.detail_offset_from_first[0],
                     oy + m.detail_offset_from_first[1]);
    mc.displacement = info(tex.displacement_desc, m.displacement_repeat_size, ox, oy);
    mc.lod_bias = m.lod_bias;
    mc.density = m.density;
    mc.m1_threshold = m.base_density_threshold;
    mc.m1_height_hardness = m.base_height_hardness;
    mc.m1_edge_hardness = m.base_edge_hardness;
    mc.m1_detail_base = m.detail_base;
    mc.m1_detail_scale = m.detail_scale;
    mc.m1_height_cut = 1.f - m.height_cut;
    mc.m1_edge_cut = m.edge_cut;
    mc.m0_detail_x = m.detail_param[0];
    mc.m0_detail_y = m.detail_param[1];
    mc.m0_disp_scale = m.displacement_scale;
    mc.vx_freq_x = (float)(1.0 / m.voxel_width[0]);
    mc.vx_freq_y = (float)(1.0 / m.voxel_width[1]);
    mc.vx_bias_x = (float)((ox + m.voxel_base[0]) / m.voxel_width[0]);
    mc.vx_bias_y = (float)((oy + m.voxel_base[1]) / m.voxel_width[1]);
    {
        const skyr_noise_texture_desc& d = tex.voxel_desc;
        double maxw = std::max(d.width, std::max(d.height, d.depth));
        mc.vx_k_lod = (float)(maxw * tan_half / (std::min(m.voxel_width[0], m.voxel_width[1]) * vmin));
    }
    bool d0 = m.type == SKYR_MATERIAL_DEFAULT0, d1 = m.type == SKYR_MATERIAL_DEFAULT1;
    if (int st = fill_tex(mc.cloud_map_tex, tex.cloud_map, tex.cloud_map_desc, false, d0 || d1, "cloud map",
                          tex.cloud_map_expanded, tex.cloud_map_expanded_channels))
        return st;
    if (int st = fill_tex(mc.detail_tex, tex.detail, tex.detail_desc, false, d0 || d1, "detail", tex.detail_expanded,
                          tex.detail_expanded_channels))
        return st;
    if (int st = fill_tex(mc.displacement_tex, tex.displacement, tex.displacement_desc, false, d0, "displacement",
                          tex.displacement_expanded, tex.displacement_expanded_channels))
        return st;
    if (int st = fill_tex(mc.voxel_tex, tex.voxel, tex.voxel_desc, true, m.type == SKYR_MATERIAL_VOXEL, "voxel",
                          nullptr, 0))
        return st;
    if (d0 && tex.displacement_desc.channels < 4) return set_error(SKYR_EINVAL, "displacement texture needs 4 channels");
    if ((d0 || d1) && tex.cloud_map_desc.channels < 2) return set_error(SKYR_EINVAL, "cloud map needs 2 channels");
    derive_fast_consts(m, tex, cp, R, mc, tan_half, vmin);
    return SKYR_OK;
}

// Length of the view ray with cos(view, up) = mu from the camera's altitude h
// inside the cloud layer [bottom, top] above a sphere of radius R, up to the
// distance `end` or the ground, in double precision.
static double layer_path(double R, double h, double bottom, double top, double mu, double end) {
    const double r = R + h, rm = r * mu;
    auto inside = [&](double s, double& t0, double& t1) {  // the ray's stretch inside the sphere of radius s
        const double disc = rm * rm - (r - s) * (r + s);
        if (disc < 0.0) return false;
        const double q = std::sqrt(disc);
        t0 = -rm - q;
        t1 = -rm + q;
        return true;
    };
    double g0, g1, o0, o1, i0, i1;
    if (r > R && inside(R, g0, g1) && g0 > 0.0) end = std::min(end, g0);
    if (!inside(R + top, o0, o1)) return 0.0;
    const double a = std::max(0.0, o0), b = std::min(end, o1);
    if (!(b > a)) return 0.0;
    double len = b - a;
    if (inside(R + bottom, i0, i1)) {
        const double lo = std::max(a, i0), hi = std::min(b, i1);
        if (hi > lo) len -= hi - lo;
    }
    return len;
}

// The raymarch's block-row order (march_row): outward from the block row whose
// centre ray runs the longest way through the cloud layer within the visible
// distance, towards the longer-running neighbour first.  The rays that graze
// the layer are the costliest, so they start first and the launch ends on
// cheap rows; with no row in the layer the order stays the identity.  Every
// pixel's result is the same in any order.
static void march_order(CloudConsts& C, int rows_per_block, int block_rows) {
    auto path = [&](int by) -> double {
        if (by < 0 || by >= block_rows) return -1.0;
        const int py = std::min(by * rows_per_block + rows_per_block / 2, C.height - 1);
        const double y = 2.0 * ((py + 0.5) / C.height) - 1.0;  // centre column, no depth
        const double dx = (double)C.a1.x * y + C.af.x, dy = (double)C.a1.y * y + C.af.y,
                     dz = (double)C.a1.z * y + C.af.z, wv = (double)C.w1 * y + C.wf;
        const double len = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (!(len > 0.0) || wv == 0.0) return 0.0;
        const double mu = dz / len * (wv < 0.0 ? -1.0 : 1.0);
        const double vis = std::min(len / std::fabs(wv), (double)C.max_visible_distance);
        return layer_path(C.R, C.cam.z, C.bottom, C.top, mu, vis);
    };
    int p = 0;
    double best = 0.0;
    for (int by = 0; by < block_rows; ++by) {
        const double l = path(by);
        if (l > best) best = l, p = by;
    }
    C.row_pivot = p;
    C.row_dir = path(p + 1) >= path(p - 1) ? 1 : -1;
}

int cloud_render_on(skyr_ctx* ctx, cudaStream_t stream, const skyr_atmosphere_parameters* atmosphere,
                    const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                    const skyr_cloud_textures* textures, const skyr_cloud_view* view, const skyr_lut_sizes* sizes,
                    const void* transmittance, const void* aerial_perspective_luminance,
                    const void* aerial_perspective_transmittance, const float* blue_noise, const float* depth,
                    void* out_rgba, float* out_distance, unsigned long long* counters,
                    const CloudCheckerboard* checkerboard, int mode) {
    if (!ctx) return set_error(SKYR_EINVAL, "null context");
    if (!atmosphere || !cloud || !material || !textures || !view || !sizes)
        return set_error(SKYR_EINVAL, "null parameter block");
    if (!transmittance || !aerial_perspective_luminance || !aerial_perspective_transmittance || !blue_noise)
        return set_error(SKYR_EINVAL, "null LUT or blue-noise input");
    if (view->width < 1 || view->height < 1 || view->width > 16384 || view->height > 16384)
        return set_error(SKYR_EINVAL, "render size must be in [1, 16384]");
    if (view->viewport_width < 1 || view->viewport_height < 1) return set_error(SKYR_EINVAL, "bad viewport size");
    if (material->type < SKYR_MATERIAL_DEFAULT0 || material->type > SKYR_MATERIAL_VOXEL)
        return set_error(SKYR_EINVAL, "unknown material type %d", material->type);
    if (!(cloud->thickness > 0.f) || !(cloud->max_raymarch_distance > 0.f) || !(cloud->max_raymarch_steps >= 1.f) ||
        cloud->max_raymarch_steps > 4096.f || !(cloud->shadow_steps > 0.f) || cloud->shadow_steps > 256.f)
        return set_error(SKYR_EINVAL, "cloud parameters out of range");
    if (sizes->aerial_perspective_width < 2 || sizes->aerial_perspective_height < 2 ||
        sizes->aerial_perspective_depth < 2 || sizes->transmittance_width < 2 || sizes->transmittance_height < 2)
        return set_error(SKYR_EINVAL, "LUT sizes must be >= 2");
    if (!(view->aerial_perspective_lut_max_distance > 0.f)) return set_error(SKYR_EINVAL, "bad AP max distance");
    CloudConsts C;
    MaterialConsts M;
    if (int st = derive_cloud_consts(*atmosphere, *cloud, *material, *textures, *view, *sizes, C, M)) return st;
    if (checkerboard) {
        C.width = checkerboard->quarter_w;
        C.height = checkerboard->quarter_h;
        C.cb_index = checkerboard->index;
        C.cb_depth = checkerboard->depth;
        C.cb_w = checkerboard->half_w;
        C.cb_h = checkerboard->half_h;
        depth = nullptr;
    }
    if (mode & kCloudCheckOnly) return SKYR_OK;
    AtmoConsts A;
    derive_atmo_consts(*atmosphere, A);
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    const bool pdl = (mode & kCloudAfterLuts) && !checkerboard;
    const int tile_w = ctx->tuning.cloud_tile_width, warps_x = ctx->tuning.cloud_block_warps_x;
    const int G = ctx->tuning.cloud_ray_lanes, tw = std::min(tile_w, 32 / G);
    const int bw = tw * warps_x, bh = (32 / G / tw) * (4 / warps_x);
    dim3 grid((C.width + bw - 1) / bw, (C.height + bh - 1) / bh);
    march_order(C, bh, (int)grid.y);
    const float4* T = reinterpret_cast<const float4*>(transmittance);
    const bool half = sizes->format == SKYR_FORMAT_RGBA16F;
    const int occ = ctx->tuning.cloud_blocks_per_sm;
    auto* out = reinterpret_cast<__half2*>(out_rgba);
    const int tlw = sizes->transmittance_width, tlh = sizes->transmittance_height;
    if (counters) {  // the instrumented launch: one lane per ray (the frame does not depend on it)
        const int tw1 = std::min(tile_w, 32);
        dim3 grid1((C.width + tw1 * warps_x - 1) / (tw1 * warps_x),
                   (C.height + (32 / tw1) * (4 / warps_x) - 1) / ((32 / tw1) * (4 / warps_x)));
        march_order(C, (32 / tw1) * (4 / warps_x), (int)grid1.y);
        launch_cloud_render_counted(half, grid1, stream, C, M, A, T, tlw, tlh, aerial_perspective_luminance,
                                    aerial_perspective_transmittance, blue_noise, depth, out, out_distance, counters,
                                    tile_w, warps_x);
        return check_cuda(cudaGetLastError(), "cloud raymarch kernel (counted)");
    }
    if (G == 8)
        launch_cloud_render<8>(half, occ, grid, stream, C, M, A, T, tlw, tlh, aerial_perspective_luminance,
                               aerial_perspective_transmittance, blue_noise, depth, out, out_distance, counters,
                               tile_w, warps_x, pdl);
    else if (G == 4)
        launch_cloud_render<4>(half, occ, grid, stream, C, M, A, T, tlw, tlh, aerial_perspective_luminance,
                               aerial_perspective_transmittance, blue_noise, depth, out, out_distance, counters,
                               tile_w, warps_x, pdl);
    else if (G == 2)
        launch_cloud_render<2>(half, occ, grid, stream, C, M, A, T, tlw, tlh, aerial_perspective_luminance,
                               aerial_perspective_transmittance, blue_noise, depth, out, out_distance, counters,
                               tile_w, warps_x, pdl);
    else
        launch_cloud_render<1>(half, occ, grid, stream, C, M, A, T, tlw, tlh, aerial_perspective_luminance,
                               aerial_perspective_transmittance, blue_noise, depth, out, out_distance, counters,
                               tile_w, warps_x, pdl);
    return check_cuda(cudaGetLastError(), "cloud raymarch kernel");
}

// The device aliases of the raymarch's host outputs: both must be page-locked
// host memory mapped into this device's address space, and the kernel then
// stores through the mapped alias.  Anything else (pageable or device memory)
// is refused, before any launch.
static int map_host_outputs(void* host_rgba, float* host_distance, void* alias[2]) {
    void* host[2] = {host_rgba, host_distance};
    const size_t align[2] = {8, 4};
    const char* name[2] = {"host_rgba", "host_distance"};
    for (int k = 0; k < 2; ++k) {
        alias[k] = nullptr;
        if (!host[k]) continue;
        cudaPointerAttributes a{};
        cudaError_t e = cudaPointerGetAttributes(&a, host[k]);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(SKYR_EINVAL, "%s: not page-locked host memory (%s)", name[k], cudaGetErrorString(e));
        }
        if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr)
            return set_error(SKYR_EINVAL, "%s: not page-locked host memory mapped for the device", name[k]);
        if (reinterpret_cast<uintptr_t>(a.devicePointer) % align[k] != 0)
            return set_error(SKYR_EINVAL, "%s: not %zu-byte aligned", name[k], align[k]);
        alias[k] = a.devicePointer;
    }
    return SKYR_OK;
}

}  // namespace skyr

using namespace skyr;

extern "C" {

int skyr_cloud_render(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                      const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                      const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                      const skyr_lut_sizes* sizes, const void* transmittance,
                      const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                      const float* blue_noise, const float* depth, void* out_rgba, float* out_distance) {
    return cloud_render_on(ctx, ctx ? ctx->stream : nullptr, atmosphere, cloud, material, textures, view, sizes,
                           transmittance, aerial_perspective_luminance, aerial_perspective_transmittance, blue_noise,
                           depth, out_rgba, out_distance, nullptr);
}

int skyr_cloud_render_to_host(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                              const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                              const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                              const skyr_lut_sizes* sizes, const void* transmittance,
                              const void* aerial_perspective_luminance,
                              const void* aerial_perspective_transmittance, const float* blue_noise,
                              const float* depth, void* host_rgba, float* host_distance) {
    if (!ctx) return set_error(SKYR_EINVAL, "null context");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    void* alias[2] = {nullptr, nullptr};
    if (int st = map_host_outputs(host_rgba, host_distance, alias)) return st;
    return cloud_render_on(ctx, ctx->stream, atmosphere, cloud, material, textures, view, sizes, transmittance,
                           aerial_perspective_luminance, aerial_perspective_transmittance, blue_noise, depth,
                           alias[0], static_cast<float*>(alias[1]), nullptr);
}

int skyr_render_frame(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                      const skyr_atmosphere_render_parameters* render, const skyr_lut_sizes* sizes,
                      void* transmittance, void* multiscattering, void* sky_view_luminance,
                      void* sky_view_transmittance, void* aerial_perspective_luminance,
                      void* aerial_perspective_transmittance, const skyr_cloud_parameters* cloud,
                      const skyr_cloud_material* material, const skyr_cloud_textures* textures,
                      const skyr_cloud_view* view, const float* blue_noise, const float* depth, void* out_rgba,
                      float* out_distance, int outputs_on_host) {
    if (!ctx) return set_error(SKYR_EINVAL, "null context");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    void* out[2] = {out_rgba, out_distance};
    if (outputs_on_host)
        if (int st = map_host_outputs(out_rgba, out_distance, out)) return st;
    // the raymarch's arguments are checked before the LUT set is enqueued, so a
    // rejected call enqueues nothing
    if (int st = cloud_render_on(ctx, ctx->stream, atmosphere, cloud, material, textures, view, sizes, transmittance,
                                 aerial_perspective_luminance, aerial_perspective_transmittance, blue_noise, depth,
                                 out[0], static_cast<float*>(out[1]), nullptr, nullptr, kCloudCheckOnly))
        return st;
    if (!render) return set_error(SKYR_EINVAL, "null render parameters");
    if (int st = skyr_update_lut_set(ctx, atmosphere, render, 1, sizes, transmittance, multiscattering,
                                     sky_view_luminance, sky_view_transmittance, aerial_perspective_luminance,
                                     aerial_perspective_transmittance))
        return st;
    return cloud_render_on(ctx, ctx->stream, atmosphere, cloud, material, textures, view, sizes, transmittance,
                           aerial_perspective_luminance, aerial_perspective_transmittance, blue_noise, depth, out[0],
                           static_cast<float*>(out[1]), nullptr, nullptr, kCloudAfterLuts);
}

int skyr_cloud_render_counted(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                              const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                              const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                              const skyr_lut_sizes* sizes, const void* transmittance,
                              const void* aerial_perspective_luminance,
                              const void* aerial_perspective_transmittance, const float* blue_noise,
                              const float* depth, void* out_rgba, float* out_distance,
                              unsigned long long* counters) {
    if (!counters) return set_error(SKYR_EINVAL, "null counters");
    return cloud_render_on(ctx, ctx ? ctx->stream : nullptr, atmosphere, cloud, material, textures, view, sizes,
                           transmittance, aerial_perspective_luminance, aerial_perspective_transmittance, blue_noise,
                           depth, out_rgba, out_distance, counters);
}



int skyr_cloud_parameters_default(skyr_cloud_parameters* c) {
    if (!c) return set_error(SKYR_EINVAL, "null parameters");
    // VolumetricCloud defaults (src/SkyRendering/VolumetricCloud.h:20-35)
    *c = skyr_cloud_parameters{};
    c->bottom_altitude = 2.f;
    c->thickness = 2.f;
    c->max_raymarch_distance = 30.f;
    c->max_raymarch_steps = 128.f;
    c->max_visible_distance = 120.f;
    c->env_color[0] = c->env_color[1] = c->env_color[2] = 1.f;
    c->env_color_scale = 0.1f;
    c->sun_illuminance_scale = 1.f;
    c->shadow_steps = 5.f;
    c->shadow_distance = 2.f;
    c->shadow_froxel_max_distance = 20.f;
    c->sun_multiscattering_sigma_scale = 0.3f;
    c->env_multiscattering_sigma_scale = 0.5f;
    c->env_bottom_visibility = 0.4f;
    c->env_sun_height_curve_exp = 1.f;
    c->phase_g_forward = 0.85f;
    c->phase_g_back = -0.15f;
    c->phase_back_scale = 2.16f;
    c->shadow_map_max_distance = 20.f;
    return SKYR_OK;
}

int skyr_cloud_material_default(int type, skyr_cloud_material* m) {
    if (!m) return set_error(SKYR_EINVAL, "null material");
    if (type < SKYR_MATERIAL_DEFAULT0 || type > SKYR_MATERIAL_VOXEL)
        return set_error(SKYR_EINVAL, "unknown material type %d", type);
    *m = skyr_cloud_material{};
    m->type = type;
    // VolumetricCloudDefaultMaterialCommon (VolumetricCloudDefaultMaterial.h:126-133, .cpp:37-64)
    m->lod_bias = 2.75f;
    m->density = 15.f;
    m->cloud_map_repeat_size = 18.99f;
    m->detail_repeat_size = 5.33f;
    m->displacement_repeat_size = 3.51f;
    m->minfilter2d = m->minfilter3d = m->minfilter_displacement = SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST;
    // VolumetricCloudDefaultMaterial1 (VolumetricCloudDefaultMaterial.h:199-205)
    m->detail_base = 0.67f;
    m->detail_scale = 1.86f;
    m->base_density_threshold = 0.4f;
    m->base_height_hardness = 6.f;
    m->base_edge_hardness = 6.f;
    m->height_cut = 0.9f;
    m->edge_cut = 0.8f;
    // VolumetricCloudDefaultMaterial0 (VolumetricCloudDefaultMaterial.h:165-166)
    m->detail_param[0] = 0.4f;
    m->detail_param[1] = 0.f;
    m->displacement_scale = 1.f;
    // VolumetricCloudVoxelMaterial (VolumetricCloudVoxelMaterial.h:32-35)
    m->voxel_width[0] = m->voxel_width[1] = 2.f;
    if (type == SKYR_MATERIAL_VOXEL) m->density = 20.f;
    if (type == SKYR_MATERIAL_MINIMAL) m->density = 0.5f;  // VolumetricCloudMinimalMaterial.h:26
    return SKYR_OK;
}

}  // extern "C"
