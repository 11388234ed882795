// oracle_cloud.hpp — TEST INFRASTRUCTURE ONLY.
//
// Restatement of the cloud material plug-ins and the volumetric-cloud raymarch
// of c52e/SkyRendering:
//   shaders/SkyRendering/VolumetricCloudCommon.glsl:36-98
//   shaders/SkyRendering/VolumetricCloudDefaultMaterialCommon.glsl:20-24
//   shaders/SkyRendering/VolumetricCloudDefaultMaterial0.glsl:9-32
//   shaders/SkyRendering/VolumetricCloudDefaultMaterial1.glsl:14-29
//   shaders/SkyRendering/VolumetricCloudMaterialMinimal.glsl:6-8
//   shaders/SkyRendering/VolumetricCloudMaterialVoxel.glsl:12-16
//   shaders/SkyRendering/VolumetricCloudRender.comp:39-210
//   host src/SkyRendering/VolumetricCloud.cpp:168-280 and
//   src/SkyRendering/VolumetricCloudDefaultMaterial.cpp:24-28,84-101.
// GL texture sampling (textureLod with LINEAR magnification and the
// *_MIPMAP_* minification filters, REPEAT / CLAMP_TO_BORDER wrapping, UNORM8
// texels) is emulated in the scalar type T.  Loop counters that the reference
// keeps in FP32 (the light-march `t += 1/steps`) stay FP32 here too, because
// they decide the number of samples.
// Parity status: unpinned (see oracle_math.hpp).
#pragma once

#include "../include/skyr_cloud.h"
#include "oracle_atmosphere.hpp"

namespace orc {

// A UNORM8 texture in the device layout of skyr_cloud.h (levels consecutive,
// channel-planar) viewed on the host.
struct Tex8 {
    const uint8_t* data = nullptr;
    int w = 1, h = 1, d = 1, channels = 1, levels = 1;
    std::vector<size_t> off;
    bool border = false;  // CLAMP_TO_BORDER (border 0) instead of REPEAT
    void init() {
        levels = 1;
        int m = std::max(w, std::max(h, d));
        while ((m >> levels) > 0) ++levels;
        off.assign(levels + 1, 0);
        for (int l = 0; l < levels; ++l) {
            size_t lw = std::max(w >> l, 1), lh = std::max(h >> l, 1), ld = std::max(d >> l, 1);
            off[l + 1] = off[l] + lw * lh * ld * channels;
        }
    }
    int lw(int l) const { return std::max(w >> l, 1); }
    int lh(int l) const { return std::max(h >> l, 1); }
    int ld(int l) const { return std::max(d >> l, 1); }
    // texel with wrapping; returns value/255
    template <class T>
    T texel(int l, int c, int x, int y, int z) const {
        int W = lw(l), H = lh(l), D = ld(l);
        if (border) {
            if (x < 0 || y < 0 || z < 0 || x >= W || y >= H || z >= D) return T(0);
        } else {
            x = ((x % W) + W) % W;
            y = ((y % H) + H) % H;
            z = ((z % D) + D) % D;
        }
        return T(data[off[l] + (size_t)c * W * H * D + ((size_t)z * H + y) * W + x]) / T(255);
    }
    template <class T>
    T nearest(int l, int c, T u, T v, T s) const {
        return texel<T>(l, c, (int)std::floor(u * T(lw(l))), (int)std::floor(v * T(lh(l))),
                        d > 1 ? (int)std::floor(s * T(ld(l))) : 0);
    }
    template <class T>
    T linear(int l, int c, T u, T v, T s) const {
        T x = u * T(lw(l)) - T(0.5), y = v * T(lh(l)) - T(0.5);
        T fx = std::floor(x), fy = std::floor(y);
        T a = x - fx, b = y - fy;
        int x0 = (int)fx, y0 = (int)fy;
        if (d <= 1) {
            T t00 = texel<T>(l, c, x0, y0, 0), t10 = texel<T>(l, c, x0 + 1, y0, 0);
            T t01 = texel<T>(l, c, x0, y0 + 1, 0), t11 = texel<T>(l, c, x0 + 1, y0 + 1, 0);
            return (T(1) - b) * ((T(1) - a) * t00 + a * t10) + b * ((T(1) - a) * t01 + a * t11);
        }
        T z = s * T(ld(l)) - T(0.5);
        T fz = std::floor(z);
        T g = z - fz;
        int z0 = (int)fz;
        T r = 0;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx)
                    r += (dx ? a : T(1) - a) * (dy ? b : T(1) - b) * (dz ? g : T(1) - g) *
                         texel<T>(l, c, x0 + dx, y0 + dy, z0 + dz);
        return r;
    }
    // textureLod with mag = LINEAR and minification `minf` (GL 4.6 8.14-8.15)
    template <class T>
    T sample(int c, T u, T v, T s, T lod, int minf) const {
        T lambda = clampg(lod, T(-1000), T(1000));
        T cswitch = (minf == SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST || minf == SKYR_MIPMAP_NEAREST_MIPMAP_LINEAR)
                        ? T(0.5)
                        : T(0);
        if (!(lambda > cswitch)) return linear<T>(0, c, u, v, s);
        int q = levels - 1;
        bool lin_in = minf == SKYR_MIPMAP_LINEAR_MIPMAP_NEAREST || minf == SKYR_MIPMAP_LINEAR_MIPMAP_LINEAR;
        auto at = [&](int l) { return lin_in ? linear<T>(l, c, u, v, s) : nearest<T>(l, c, u, v, s); };
        if (minf == SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST || minf == SKYR_MIPMAP_LINEAR_MIPMAP_NEAREST) {
            int dl = lambda <= T(0.5) ? 0 : (int)std::ceil(lambda + T(0.5)) - 1;
            return at(std::min(dl, q));
        }
        if (lambda >= T(q)) return at(q);
        int d1 = (int)std::floor(lambda);
        T f = lambda - T(d1);
        return (T(1) - f) * at(d1) + f * at(std::min(d1 + 1, q));
    }
};

// SampleInfo (VolumetricCloudDefaultMaterialCommon.glsl:4-8)
template <class T>
struct SampleInfo {
    T bias_x, bias_y, frequency, k_lod;
};

// Everything VolumetricCloud::Update and the material's Update upload.
template <class T>
struct CloudFrame {
    M4<T> inv_mvp;
    V3<T> cam, sun;  // local z-up frame
    T R, bottom, top;
    T frame_id, ap_max_distance;
    // VolumetricCloudBufferData
    T sun_illuminance_scale, max_raymarch_distance, max_raymarch_steps, max_visible_distance;
    V3<T> env_color_scale;
    float shadow_steps;  // the light-march loop runs in FP32, see header
    T sun_ms_sigma_scale, env_ms_sigma_scale, shadow_distance, env_bottom_visibility, env_sun_height_curve_exp;
    T g_fwd, g_back, back_scale;
    // material
    int type;
    SampleInfo<T> cloud_map, detail, displacement;
    T lod_bias, density;
    int min2d, min3d, mindisp;
    T m1_threshold, m1_height_hardness, m1_edge_hardness, m1_detail_base, m1_detail_scale, m1_height_cut, m1_edge_cut;
    T m0_detail_x, m0_detail_y, m0_disp_scale;
    T vx_freq_x, vx_freq_y, vx_bias_x, vx_bias_y, vx_k_lod;
    // shadow froxel of the view (skyr_cloud_view.shadow_froxel), null: visibility 1
    const uint16_t* froxel = nullptr;
    int fx_w = 0, fx_h = 0, fx_d = 0;
    T inv_froxel_max = T(0);
};

template <class T>
T fract_d(double x) {
    return T(x - std::floor(x));
}

// VolumetricCloud::Update (VolumetricCloud.cpp:168-280), the material Update
// (VolumetricCloudDefaultMaterial.cpp:84-101, VolumetricCloudVoxelMaterial.cpp:93-105)
// and CalKLod (VolumetricCloudDefaultMaterial.cpp:24-28).
template <class T>
CloudFrame<T> derive_cloud_frame(const skyr_atmosphere_parameters& atmo, const skyr_cloud_parameters& cp,
                                 const skyr_cloud_material& m, const skyr_cloud_textures& tex,
                                 const skyr_cloud_view& v) {
    CloudFrame<T> f;
    T R = T(atmo.bottom_radius);
    V3<T> center(T(0), -R, T(0));
    V3<T> cam = v3f<T>(v.camera_position);
    V3<T> up = normalize(cam - center);
    V3<T> origin = center + up * R;
    V3<T> front = normalize(cross(up, V3<T>(T(1), T(0), T(0))));
    V3<T> right = normalize(cross(up, front));
    M4<T> model;
    for (int i = 0; i < 16; ++i) model.m[i] = T(0);
    for (int r = 0; r < 3; ++r) {
        model(r, 0) = front[r];
        model(r, 1) = right[r];
        model(r, 2) = up[r];
        model(r, 3) = origin[r];
    }
    model(3, 3) = T(1);
    M4<T> inv_model = inverse(model);
    M4<T> mvp = matmul(mat_from_floats<T>(v.view_projection), model);
    f.inv_mvp = inverse(mvp);
    f.cam = mul_point(inv_model, cam);
    T deg = T(kPi) / T(180);
    V3<T> sun_world = from_theta_phi<T>(T(v.sun_direction_theta) * deg, T(v.sun_direction_phi) * deg);
    f.sun = normalize(mul_dir(inv_model, sun_world));
    f.R = R;
    f.bottom = T(cp.bottom_altitude);
    f.top = T(cp.bottom_altitude) + T(cp.thickness);
    f.frame_id = T(v.frame_id);
    f.ap_max_distance = T(v.aerial_perspective_lut_max_distance);
    f.sun_illuminance_scale = T(cp.sun_illuminance_scale);
    f.max_raymarch_distance = T(cp.max_raymarch_distance);
    f.max_raymarch_steps = T(cp.max_raymarch_steps);
    f.max_visible_distance = T(cp.max_visible_distance);
    f.env_color_scale = v3f<T>(cp.env_color) * T(cp.env_color_scale);
    f.shadow_steps = cp.shadow_steps;
    f.sun_ms_sigma_scale = T(cp.sun_multiscattering_sigma_scale);
    f.env_ms_sigma_scale = T(cp.env_multiscattering_sigma_scale);
    f.shadow_distance = T(cp.shadow_distance);
    f.env_bottom_visibility = T(cp.env_bottom_visibility);
    f.env_sun_height_curve_exp = T(cp.env_sun_height_curve_exp);
    f.g_fwd = T(cp.phase_g_forward);
    f.g_back = T(cp.phase_g_back);
    f.back_scale = T(cp.phase_back_scale);

    f.type = m.type;
    T tan_half = std::tan(T(v.fovy) * deg * T(0.5));
    T vmin = T(std::min(v.viewport_width, v.viewport_height));
    auto info = [&](const skyr_noise_texture_desc& d, float repeat, double ox, double oy) {
        SampleInfo<T> s;
        s.frequency = T(1) / T(repeat);
        s.bias_x = fract_d<T>(ox / (double)repeat);
        s.bias_y = fract_d<T>(oy / (double)repeat);
        T maxw = T(std::max(d.width, std::max(d.height, d.depth)));
        s.k_lod = maxw * tan_half / (T(repeat) * vmin);
        return s;
    };
    double ox = m.offset_from_first[0], oy = m.offset_from_first[1];
    f.cloud_map = info(tex.cloud_map_desc, m.cloud_map_repeat_size, ox, oy);
    f.detail = info(tex.detail_desc, m.detail_repeat_size, ox + m.detail_offset_from_first[0],
                    oy + m.detail_offset_from_first[1]);
    f.displacement = info(tex.displacement_desc, m.displacement_repeat_size, ox, oy);
    f.lod_bias = T(m.lod_bias);
    f.density = T(m.density);
    f.min2d = m.minfilter2d;
    f.min3d = m.minfilter3d;
    f.mindisp = m.minfilter_displacement;
    f.m1_threshold = T(m.base_density_threshold);
    f.m1_height_hardness = T(m.base_height_hardness);
    f.m1_edge_hardness = T(m.base_edge_hardness);
    f.m1_detail_base = T(m.detail_base);
    f.m1_detail_scale = T(m.detail_scale);
    f.m1_height_cut = T(1) - T(m.height_cut);  // uHeightCut = 1 - height_cut_ (cpp:461)
    f.m1_edge_cut = T(m.edge_cut);
    f.m0_detail_x = T(m.detail_param[0]);
    f.m0_detail_y = T(m.detail_param[1]);
    f.m0_disp_scale = T(m.displacement_scale);
    // VolumetricCloudVoxelMaterial::Update (VolumetricCloudVoxelMaterial.cpp:93-105)
    f.vx_freq_x = T(1) / T(m.voxel_width[0]);
    f.vx_freq_y = T(1) / T(m.voxel_width[1]);
    f.vx_bias_x = T((ox + m.voxel_base[0]) / (double)m.voxel_width[0]);
    f.vx_bias_y = T((oy + m.voxel_base[1]) / (double)m.voxel_width[1]);
    {
        const skyr_noise_texture_desc& d = tex.voxel_desc;
        T maxw = T(std::max(d.width, std::max(d.height, d.depth)));
        f.vx_k_lod = maxw * tan_half / (T(std::min(m.voxel_width[0], m.voxel_width[1])) * vmin);
    }
    if (v.shadow_froxel) {
        f.froxel = v.shadow_froxel;
        f.fx_w = v.shadow_froxel_width;
        f.fx_h = v.shadow_froxel_height;
        f.fx_d = v.shadow_froxel_depth;
        f.inv_froxel_max = T(1) / T(cp.shadow_froxel_max_distance);  // GetShadowFroxel (VolumetricCloud.h:72)
    }
    return f;
}

template <class T>
struct CloudOracle {
    const AtmosphereOracle<T>& O;
    CloudFrame<T> F;
    Tex8 cloud_map, detail, displacement, voxel;
    const Image<T>* tlut;
    const Image<T>* ap_lum;
    const Image<T>* ap_trans;
    const float* blue_noise;

    // CalHeight01 (VolumetricCloudCommon.glsl:36-39)
    T CalHeight01(V3<T> p) const {
        T alt = length(V3<T>(p.x, p.y, p.z + F.R)) - F.R;
        return clampg((alt - F.bottom) / (F.top - F.bottom), T(0), T(1));
    }

    // GetUVWLod (VolumetricCloudDefaultMaterialCommon.glsl:20-24)
    void uvw_lod(V3<T> p, const SampleInfo<T>& s, T& u, T& v, T& w, T& lod) const {
        u = p.x * s.frequency + s.bias_x;
        v = p.y * s.frequency + s.bias_y;
        w = p.z * s.frequency;
        lod = std::log2(s.k_lod * length(p - F.cam)) + F.lod_bias;
    }

    // SampleSigmaT of the four materials
    T SampleSigmaT(V3<T> p, T h01) const {
        switch (F.type) {
            case SKYR_MATERIAL_DEFAULT1: {
                T u, v, w, lod;
                uvw_lod(p, F.cloud_map, u, v, w, lod);
                T cr = cloud_map.sample<T>(0, u, v, T(0), lod, F.min2d);
                T density = clampg((cr - F.m1_threshold) * F.m1_edge_hardness, T(0), T(1));
                density *= clampg((T(1) - h01) * F.m1_height_hardness, T(0), T(1));
                if (density == T(0)) return T(0);
                uvw_lod(p, F.detail, u, v, w, lod);
                T dt = detail.sample<T>(0, u, v, w, lod, F.min3d);
                dt = (dt + F.m1_detail_base) * F.m1_detail_scale;
                dt *= std::max(clampg(h01 - F.m1_height_cut, T(0), T(1)), clampg(F.m1_edge_cut - cr, T(0), T(1)));
                return clampg(density - dt, T(0), T(1)) * F.density * h01;
            }
            case SKYR_MATERIAL_DEFAULT0: {
                T u, v, w, lod;
                uvw_lod(p, F.cloud_map, u, v, w, lod);
                T cr = cloud_map.sample<T>(0, u, v, T(0), lod, F.min2d);
                T cg = cloud_map.sample<T>(1, u, v, T(0), lod, F.min2d);
                uvw_lod(p, F.displacement, u, v, w, lod);
                V3<T> disp;
                disp.x = displacement.sample<T>(0, u, v, T(0), lod, F.mindisp);
                disp.y = displacement.sample<T>(1, u, v, T(0), lod, F.mindisp);
                disp.x += displacement.sample<T>(2, u, w, T(0), lod, F.mindisp);
                disp.z = displacement.sample<T>(3, u, w, T(0), lod, F.mindisp);
                p = p + disp * F.m0_disp_scale;
                uvw_lod(p, F.detail, u, v, w, lod);
                T dt = detail.sample<T>(0, u, v, w, lod, F.min3d) * F.m0_detail_x + F.m0_detail_y;
                // CalHeightMask (VolumetricCloudDefaultMaterial0.glsl:9-12)
                T hit = clampg(h01 / cg, T(0), T(1));
                T mask = clampg(hit * (hit - T(1)) * T(-4), T(0), T(1));
                T x = cr * mask;
                return clampg((x - dt) / (T(1) - dt), T(0), T(1)) * h01 * F.density;
            }
            case SKYR_MATERIAL_MINIMAL: return F.density;
            case SKYR_MATERIAL_VOXEL: {
                T u = p.x * F.vx_freq_x + F.vx_bias_x;
                T v = p.y * F.vx_freq_y + F.vx_bias_y;
                T lod = std::log2(F.vx_k_lod * length(p - F.cam)) + F.lod_bias;
                return voxel.sample<T>(0, u, v, h01, lod, SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST) * F.density;
            }
        }
        return T(0);
    }

    // SampleRayScatterVisibility (VolumetricCloudShadowInterface.glsl:10-13): the
    // R16 froxel through a LINEAR + CLAMP_TO_EDGE sampler
    // (Samplers::GetLinearNoMipmapClampToEdge, VolumetricCloud.h:72)
    T RayScatterVisibility(T u, T v, T dist) const {
        if (!F.froxel) return T(1);
        T w = dist * F.inv_froxel_max;
        T c[3] = {u * T(F.fx_w) - T(0.5), v * T(F.fx_h) - T(0.5), w * T(F.fx_d) - T(0.5)};
        const int n[3] = {F.fx_w, F.fx_h, F.fx_d};
        int i0[3], i1[3];
        T f[3];
        for (int k = 0; k < 3; ++k) {
            T fl = std::floor(c[k]);
            f[k] = c[k] - fl;
            i0[k] = std::min(std::max(int(fl), 0), n[k] - 1);
            i1[k] = std::min(std::max(int(fl) + 1, 0), n[k] - 1);
        }
        T s = T(0);
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    int x = dx ? i1[0] : i0[0], y = dy ? i1[1] : i0[1], z = dz ? i1[2] : i0[2];
                    T wgt = (dx ? f[0] : T(1) - f[0]) * (dy ? f[1] : T(1) - f[1]) * (dz ? f[2] : T(1) - f[2]);
                    s += wgt * T(F.froxel[(size_t(z) * F.fx_h + y) * F.fx_w + x]) / T(65535);
                }
        return mixg(T(1), s, clampg(T(1) / w, T(0), T(1)));
    }

    // RayShellIntersect (VolumetricCloudRender.comp:39-71)
    void RayShellIntersect(T r, T mu, T t[2][2]) const {
        t[0][0] = t[0][1] = t[1][0] = t[1][1] = T(0);
        T rb = F.R + F.bottom, rt = F.R + F.top;
        T db = r * r * (mu * mu - T(1)) + rb * rb;
        T dt = r * r * (mu * mu - T(1)) + rt * rt;
        T sb = std::sqrt(db), st = std::sqrt(dt);
        if (F.cam.z < F.bottom) {
            t[0][0] = -r * mu + sb;
            t[0][1] = -r * mu + st;
        } else if (F.cam.z < F.top) {
            if (db >= T(0) && mu < T(0)) {
                t[0][1] = -r * mu - sb;
                t[1][0] = -r * mu + sb;
                t[1][1] = -r * mu + st;
            } else {
                t[0][1] = -r * mu + st;
            }
        } else {
            if (db >= T(0) && mu < T(0)) {
                t[0][0] = -r * mu - st;
                t[0][1] = -r * mu - sb;
                t[1][0] = -r * mu + sb;
                t[1][1] = -r * mu + st;
            } else if (dt >= T(0) && mu < T(0)) {
                t[0][0] = -r * mu - st;
                t[0][1] = -r * mu + st;
            }
        }
    }

    T HG(T c, T g) const {  // VolumetricCloudCommon.glsl:58-63
        T a = T(1) - g * g;
        T b = T(1) + g * g - T(2) * g * c;
        b *= std::sqrt(b);
        return (T(0.25) / T(kPi)) * a / b;
    }

    // SampleShadow (VolumetricCloudRender.comp:98-114)
    T SampleShadow(V3<T> pos) const {
        T od = 0;
        float inv = 1.0f / F.shadow_steps;
        V3<T> sv = F.sun * F.shadow_distance;
        T prev = 0;
        for (float tf = inv; tf <= 1.0f; tf += inv) {
            T cur = T(tf) * T(tf);
            T dt = cur - prev;
            V3<T> sp = pos + sv * (prev + T(0.5) * dt);
            od += SampleSigmaT(sp, CalHeight01(sp)) * F.shadow_distance * dt;
            prev = cur;
        }
        return std::exp(-od);
    }

    struct Ctx {
        T t, height01, step, trans, trans_sum, wsum, cos_sun_view;
        V3<T> pos;
        T sun, env;
    };

    // RayMarchStep (VolumetricCloudRender.comp:116-137)
    void RayMarchStep(Ctx& c) const {
        T sigma = SampleSigmaT(c.pos, c.height01);
        if (sigma < T(1e-5)) return;
        T tr = std::exp(-c.step * sigma);
        T tsun = SampleShadow(c.pos);
        T phase = mixg(HG(c.cos_sun_view, F.g_back) * F.back_scale, HG(c.cos_sun_view, F.g_fwd),
                       std::exp(-F.sun_ms_sigma_scale * sigma));
        T s = tsun * phase;
        T e = mixg(F.env_bottom_visibility, T(1), c.height01);
        e = e - e * std::exp(-F.env_ms_sigma_scale * sigma);
        s = s - s * tr;
        e = e - e * tr;
        c.sun += c.trans * s;
        c.env += c.trans * e;
        c.trans_sum += c.trans;
        c.wsum += c.t * c.trans;
        c.trans *= tr;
    }

    // GetSunVisibility(transmittance_texture, pos) (VolumetricCloudCommon.glsl:75-80)
    V3<T> SunVisibilityAt(V3<T> pos) const {
        V3<T> up(pos.x, pos.y, pos.z + F.R);
        T r = length(up);
        up = up / r;
        return O.GetSunVisibility(*tlut, r, dot(F.sun, up));
    }

    // main (VolumetricCloudRender.comp:139-210) at full resolution: pixel
    // (px, py) of a w x h image with window depth `depth`.
    void Pixel(int px, int py, int w, int h, float depth, T out_rgba[4], T& out_dist) const {
        PixelAt((T(px) + T(0.5)) / T(w), (T(py) + T(0.5)) / T(h), depth, px, py, out_rgba, out_dist);
    }

    // The same for the ray through screen (u, v) at window depth `depth`, its
    // blue noise taken at pixel (nx, ny): the quarter-resolution pass
    // raymarches checkerboard texels and indexes the noise by its own pixel
    // (VolumetricCloudRender.comp:140-166).
    void PixelAt(T u, T v, float depth, int nx, int ny, T out_rgba[4], T& out_dist) const {
        V3<T> frag = projective_mul(F.inv_mvp, V3<T>(u * T(2) - T(1), v * T(2) - T(1), T(depth) * T(2) - T(1)));
        V3<T> view = normalize(frag - F.cam);
        T r = F.cam.z + F.R;
        T mu = view.z;
        T it[2][2];
        RayShellIntersect(r, mu, it);
        T frag_dist = length(frag - F.cam);
        for (int i = 0; i < 2; ++i) it[i][1] = clampg(std::min(frag_dist, F.max_visible_distance), it[i][0], it[i][1]);
        Ctx c;
        c.cos_sun_view = dot(F.sun, view);
        T dist = it[0][1] - it[0][0];
        dist = std::min(dist, F.max_raymarch_distance);
        unsigned n = (unsigned)std::max(F.max_raymarch_steps * (dist / F.max_raymarch_distance), T(1));
        c.step = dist / T(n);
        c.trans = T(1);
        c.trans_sum = c.wsum = T(0);
        c.sun = c.env = T(0);
        T noise = T(blue_noise[(ny & 63) * 64 + (nx & 63)]);
        T jitter = fractg(noise + F.frame_id * T(0.61803398875));
        c.t = it[0][0] + c.step * jitter;
        for (unsigned k = n; k != 0; --k, c.t += c.step) {
            c.pos = F.cam + view * c.t;
            c.height01 = CalHeight01(c.pos);
            RayMarchStep(c);
            if (c.trans < T(0.01)) break;
        }
        T dist1 = it[1][1] - it[1][0];
        if (dist1 > T(0)) {
            dist1 = std::min(dist1, F.max_raymarch_distance);
            unsigned n1 = (unsigned)std::max(F.max_raymarch_steps * (dist1 / F.max_raymarch_distance), T(1));
            c.step = dist1 / T(n1);
            c.t = it[1][0] + c.step * jitter;
            for (unsigned k = n1; k != 0; --k, c.t += c.step) {
                c.pos = F.cam + view * c.t;
                c.height01 = CalHeight01(c.pos);
                RayMarchStep(c);
                if (c.trans < T(0.01)) break;
            }
        }
        T avg_t = c.wsum == T(0) ? frag_dist : c.wsum / c.trans_sum;
        out_dist = avg_t;
        V3<T> avg_pos = F.cam + view * avg_t;
        V3<T> upp = normalize(V3<T>(avg_pos.x, avg_pos.y, avg_pos.z + F.R));
        T sun_cos = clampg(dot(upp, F.sun), T(0), T(1));
        V3<T> lum = SunVisibilityAt(avg_pos) * (c.sun * F.sun_illuminance_scale) * O.A.solar_illuminance +
                    F.env_color_scale * (c.env * std::pow(sun_cos, F.env_sun_height_curve_exp));
        // GetAerialPerspective (VolumetricCloudCommon.glsl:81-98)
        T ta = avg_t;
        if (r > O.A.top_radius) {
            T disc = r * r * (mu * mu - T(1)) + O.A.top_radius * O.A.top_radius;
            if (mu < T(0) && disc >= T(0)) ta -= std::max(-r * mu - std::sqrt(std::max(disc, T(0))), T(0));
            else ta = T(0);
        }
        T wz = std::sqrt(ta / F.ap_max_distance);
        T uu = T(0.5) / T(ap_lum->w) + u * (T(1) - T(1) / T(ap_lum->w));
        T vv = T(0.5) / T(ap_lum->h) + v * (T(1) - T(1) / T(ap_lum->h));
        T ww = T(0.5) / T(ap_lum->d) + wz * (T(1) - T(1) / T(ap_lum->d));
        V3<T> at = sample_linear_clamp3(*ap_trans, uu, vv, ww);
        V3<T> al = sample_linear_clamp3(*ap_lum, uu, vv, ww);
        al = al * RayScatterVisibility(u, v, avg_t);  // VolumetricCloudRender.comp:198
        lum = lum * at + al * (T(1) - c.trans);
        lum = lum / std::max(T(1e-5), T(1) - c.trans);
        T fade = smoothstepg(F.max_visible_distance * T(0.75), F.max_visible_distance, it[0][0]);
        T trans = mixg(c.trans, T(1), fade);
        lum = lum * (T(1) - trans);
        out_rgba[0] = lum.x;
        out_rgba[1] = lum.y;
        out_rgba[2] = lum.z;
        out_rgba[3] = trans;
    }
};

}  // namespace orc
