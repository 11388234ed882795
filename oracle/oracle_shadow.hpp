// oracle_shadow.hpp — TEST INFRASTRUCTURE ONLY: FP64 restatement of the
// volumetric cloud's shadow passes (VolumetricCloud::RenderShadow,
// src/SkyRendering/VolumetricCloud.cpp:282-325) and of the light transform of
// VolumetricCloud::Update (VolumetricCloud.cpp:138-166,188-235).  It is the
// reference the CUDA shadow passes are checked against; nothing in the
// library calls it.
//
// The light transform is rebuilt the way the reference builds it: the Camera
// (position, front, up, right, fovy, aspect; src/Base/src/Camera.cpp:14-36) is
// recovered from the view-projection matrix, and the frustum section is
// formed from those vectors (GetLightProjection), not from NDC corners.
#pragma once

#include <cmath>
#include <cstdint>

#include "oracle_cloud.hpp"

namespace orc {

struct LightFrameD {
    M4<double> light_vp, inv_light_vp, model, reproject;
    bool has_previous = false;
};

inline M4<double> identity_m4() {
    M4<double> m;
    for (int i = 0; i < 16; ++i) m.m[i] = (i % 5) == 0 ? 1.0 : 0.0;
    return m;
}

// glm::lookAt, right-handed
inline M4<double> look_at(V3<double> eye, V3<double> center, V3<double> up) {
    V3<double> f = normalize(center - eye);
    V3<double> s = normalize(cross(f, up));
    V3<double> u = cross(s, f);
    M4<double> m = identity_m4();
    for (int c = 0; c < 3; ++c) {
        m(0, c) = s[c];
        m(1, c) = u[c];
        m(2, c) = -f[c];
    }
    m(0, 3) = -dot(s, eye);
    m(1, 3) = -dot(u, eye);
    m(2, 3) = dot(f, eye);
    return m;
}

// glm::ortho, right-handed, clip depth [-1, 1]
inline M4<double> ortho(double l, double r, double b, double t, double n, double f) {
    M4<double> m = identity_m4();
    m(0, 0) = 2.0 / (r - l);
    m(1, 1) = 2.0 / (t - b);
    m(2, 2) = -2.0 / (f - n);
    m(0, 3) = -(r + l) / (r - l);
    m(1, 3) = -(t + b) / (t - b);
    m(2, 3) = -(f + n) / (f - n);
    return m;
}

// The Camera behind a view: ViewProjection = perspective(fovy, aspect) *
// lookAt(position, position + front, up) (Camera.cpp:14-18).
struct CameraD {
    V3<double> position, front, up, right;
    double tan_half_fovy, aspect;
};

inline CameraD camera_of(const skyr_cloud_view& v) {
    M4<double> ivp = inverse(mat_from_floats<double>(v.view_projection));
    CameraD c;
    c.position = v3f<double>(v.camera_position);
    V3<double> mid = projective_mul(ivp, V3<double>(0, 0, 0));
    V3<double> xr = projective_mul(ivp, V3<double>(1, 0, 0));
    V3<double> yt = projective_mul(ivp, V3<double>(0, 1, 0));
    c.front = normalize(mid - c.position);
    c.right = normalize(xr - mid);
    c.up = normalize(yt - mid);
    double depth = dot(mid - c.position, c.front);
    c.tan_half_fovy = length(yt - mid) / depth;
    c.aspect = length(xr - mid) / length(yt - mid);
    return c;
}

// VolumetricCloud::Update's light maths.  `previous` carries the previous
// frame's light_vp and model; `wind` is additional_delta (local km) or null.
inline LightFrameD derive_light_frame(const skyr_atmosphere_parameters& atmo, const skyr_cloud_parameters& cp,
                                      const skyr_cloud_view& v, int map_w, int map_h, const LightFrameD* previous,
                                      const float* wind) {
    const double R = atmo.bottom_radius;
    V3<double> center(0.0, -R, 0.0);
    V3<double> cam = v3f<double>(v.camera_position);
    V3<double> up = normalize(cam - center);
    V3<double> origin = center + up * R;
    V3<double> front = normalize(cross(up, V3<double>(1, 0, 0)));
    V3<double> right = normalize(cross(up, front));
    M4<double> model = identity_m4();
    for (int r = 0; r < 3; ++r) {
        model(r, 0) = front[r];
        model(r, 1) = right[r];
        model(r, 2) = up[r];
        model(r, 3) = origin[r];
    }
    M4<double> inv_model = inverse(model);
    V3<double> local_cam = mul_point(inv_model, cam);
    const double deg = kPi / 180.0;
    V3<double> sun_world = from_theta_phi<double>(double(v.sun_direction_theta) * deg,
                                                  double(v.sun_direction_phi) * deg);
    V3<double> local_sun = normalize(mul_dir(inv_model, sun_world));
    V3<double> lup = (local_sun.x == 0.0 && local_sun.y == 0.0) ? V3<double>(1, 0, 0) : V3<double>(0, 0, 1);
    M4<double> light_view = look_at(local_cam, local_cam - local_sun, lup);
    // GetLightProjection (VolumetricCloud.cpp:138-166)
    CameraD c = camera_of(v);
    const double dmax = cp.shadow_map_max_distance;
    V3<double> far_center = c.position + c.front * dmax;
    V3<double> vu = c.up * (c.tan_half_fovy * dmax);
    V3<double> vr = c.right * (c.aspect * c.tan_half_fovy * dmax);
    V3<double> verts[5] = {c.position, far_center + vu + vr, far_center + vu - vr, far_center - vu + vr,
                           far_center - vu - vr};
    double mn[2] = {1e10, 1e10}, mx[2] = {-1e10, -1e10};
    for (const auto& w : verts) {
        V3<double> vl = mul_point(light_view, mul_point(inv_model, w));
        for (int i = 0; i < 2; ++i) {
            mn[i] = std::min(mn[i], vl[i]);
            mx[i] = std::max(mx[i], vl[i]);
        }
    }
    const double res[2] = {double(map_w), double(map_h)};
    for (int i = 0; i < 2; ++i) {
        double pad = 0.5 * (mx[i] - mn[i]) / res[i];
        mn[i] -= pad;
        mx[i] += pad;
    }
    LightFrameD out;
    out.light_vp = matmul(ortho(mn[0], mx[0], mn[1], mx[1], -1.0, 1.0), light_view);
    out.inv_light_vp = inverse(out.light_vp);
    out.model = model;
    out.reproject = identity_m4();
    if (previous) {
        M4<double> add = identity_m4();
        if (wind) {
            add(0, 3) = wind[0];
            add(1, 3) = wind[1];
        }
        out.reproject = matmul(matmul(matmul(previous->light_vp, matmul(inverse(previous->model), model)), add),
                               out.inv_light_vp);
        out.has_previous = true;
    }
    return out;
}

// GL LINEAR fetch of a two-channel float texture with CLAMP_TO_BORDER and
// border (1e10, 1) (shadow_map_sampler_, VolumetricCloud.cpp:106-112).
inline void sample_map_border(const double* map, int w, int h, double u, double v, double out[2]) {
    double x = u * w - 0.5, y = v * h - 0.5;
    double fx = std::floor(x), fy = std::floor(y);
    double a = x - fx, b = y - fy;
    int x0 = int(fx), y0 = int(fy);
    for (int ch = 0; ch < 2; ++ch) {
        double s = 0.0;
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                int xi = x0 + dx, yi = y0 + dy;
                double t = (xi >= 0 && xi < w && yi >= 0 && yi < h) ? map[(size_t(yi) * w + xi) * 2 + ch]
                                                                    : (ch == 0 ? 1e10 : 1.0);
                s += (dx ? a : 1 - a) * (dy ? b : 1 - b) * t;
            }
        out[ch] = s;
    }
}

// VolumetricCloudShadowMap.comp:37-75
struct ShadowMapOracle {
    const CloudOracle<double>& C;
    LightFrameD L;
    int w, h;
    const float* blue_noise;
    const double* previous;  // raw map of the previous frame (2 per texel) or null

    // LineShellFirstIntersect (VolumetricCloudShadowMap.comp:18-35)
    void LineShellFirstIntersect(double r, double mu, double& t1, double& t2) const {
        t1 = t2 = 0.0;
        double rb = C.F.R + C.F.bottom, rt = C.F.R + C.F.top;
        double dt = r * r * (mu * mu - 1.0) + rt * rt;
        if (dt > 0) {
            double db = r * r * (mu * mu - 1.0) + rb * rb;
            double st = std::sqrt(dt);
            t1 = -r * mu - st;
            t2 = -r * mu + (db >= 0 ? -std::sqrt(db) : st);
        }
    }

    void Texel(int x, int y, double out[2]) const {
        const auto& F = C.F;
        double u = (x + 0.5) / w, v = (y + 0.5) / h;
        V3<double> origin = projective_mul(L.inv_light_vp, V3<double>(u * 2 - 1, v * 2 - 1, 0.0));
        V3<double> dir = -F.sun;
        V3<double> up(origin.x, origin.y, origin.z + F.R);
        double r = length(up);
        up = up / r;
        double mu = dot(up, dir);
        double t1, t2;
        LineShellFirstIntersect(r, mu, t1, t2);
        double dist = std::max(t2 - t1, 0.0);
        dist = std::min(dist, 1.0 / std::cos(85.0 * kPi / 180.0) * (F.top - F.bottom));
        double od = 0.0;
        if (dist > 0.0) {
            // the step count is a GLSL float: mix(12, 6, |dir.z|), truncated by uint()
            float steps_f = 12.0f + (6.0f - 12.0f) * std::fabs(float(dir.z));
            double step = dist / double(steps_f);
            double noise = blue_noise[(y & 63) * 64 + (x & 63)];
            double t = t1 + step * fractg(noise + F.frame_id * 0.61803398875);
            for (unsigned cnt = unsigned(steps_f); cnt != 0; cnt--, t += step) {
                V3<double> pos = origin + dir * t;
                od += C.SampleSigmaT(pos, C.CalHeight01(pos)) * step;
            }
        }
        double res[2] = {mixg(t1, t2, 0.5), std::exp(-od)};
        if (previous && L.has_previous) {
            V3<double> p = projective_mul(L.reproject, V3<double>(u * 2 - 1, v * 2 - 1, 0.0));
            double pu = p.x * 0.5 + 0.5, pv = p.y * 0.5 + 0.5;
            if (pu >= 0.5 / w && pu <= (w - 0.5) / w && pv >= 0.5 / h && pv <= (h - 0.5) / h) {
                double pre[2];
                sample_map_border(previous, w, h, pu, pv, pre);
                for (int k = 0; k < 2; ++k) res[k] = mixg(pre[k], res[k], 0.2);
            }
        }
        out[0] = res[0];
        out[1] = res[1];
    }
};

// VolumetricCloudShadowMapBlur.comp:9-42, both passes
inline void shadow_blur(int w, int h, const double* in, double* out) {
    static const double wgt[5] = {0.227027, 0.1945946, 0.1216216, 0.054054, 0.016216};
    std::vector<double> tmp(size_t(w) * h * 2);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
            for (int c = 0; c < 2; ++c) {
                double s = in[(size_t(y) * w + x) * 2 + c] * wgt[0];
                for (int i = 1; i < 5; ++i) {
                    s += in[(size_t(y) * w + std::max(x - i, 0)) * 2 + c] * wgt[i];
                    s += in[(size_t(y) * w + std::min(x + i, w - 1)) * 2 + c] * wgt[i];
                }
                tmp[(size_t(y) * w + x) * 2 + c] = s;
            }
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
            for (int c = 0; c < 2; ++c) {
                double s = tmp[(size_t(y) * w + x) * 2 + c] * wgt[0];
                for (int i = 1; i < 5; ++i) {
                    s += tmp[(size_t(std::max(y - i, 0)) * w + x) * 2 + c] * wgt[i];
                    s += tmp[(size_t(std::min(y + i, h - 1)) * w + x) * 2 + c] * wgt[i];
                }
                out[(size_t(y) * w + x) * 2 + c] = s;
            }
}

// SampleCloudShadowTransmittance (VolumetricCloudShadowInterface.glsl:4-8)
inline double shadow_transmittance(const double* map, int w, int h, V3<double> light_ndc) {
    double dt[2];
    sample_map_border(map, w, h, light_ndc.x * 0.5 + 0.5, light_ndc.y * 0.5 + 0.5, dt);
    return mixg(dt[1], 1.0, clampg((dt[0] - light_ndc.z) * (1.0 / 0.5), 0.0, 1.0));
}

// VolumetricCloudShadowFroxel.comp:10-27 for column (x, y) of a fw x fh x fd
// froxel: the running mean per slice before the R16 store.
inline void froxel_column(const CloudFrame<double>& F, const LightFrameD& L, const double* map, int mw, int mh,
                          int fw, int fh, int fd, double max_distance, int x, int y, double* out) {
    double u = (x + 0.5) / fw, v = (y + 0.5) / fh;
    V3<double> frag = projective_mul(F.inv_mvp, V3<double>(u * 2 - 1, v * 2 - 1, 0.0));
    double step = max_distance / fd;
    V3<double> dir = normalize(frag - F.cam);
    double t = 0.5 * step, sum = 0.0;
    for (int z = 0; z < fd; ++z, t += step) {
        V3<double> pos = F.cam + dir * t;
        sum += shadow_transmittance(map, mw, mh, projective_mul(L.light_vp, pos));
        out[z] = sum / double(z + 1);
    }
}

// imageStore into an R16 texel: round(clamp(v, 0, 1) * 65535)
inline uint16_t unorm16(double v) {
    return uint16_t(std::lround(clampg(v, 0.0, 1.0) * 65535.0));
}

}  // namespace orc
