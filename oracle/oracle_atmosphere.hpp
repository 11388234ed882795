// oracle_atmosphere.hpp — TEST INFRASTRUCTURE ONLY.
//
// Line-by-line restatement, templated on the scalar type, of the atmosphere LUT
// math of c52e/SkyRendering:
//   shaders/SkyRendering/Atmosphere.glsl:37-178,220-438
//   shaders/SkyRendering/AtmosphereInterface.glsl:6-23
//   shaders/SkyRendering/AtmosphereRenderer.glsl:56-245
//   host derivations src/SkyRendering/Atmosphere.cpp:49-70 and
//   src/SkyRendering/AtmosphereRenderer.cpp:52-83.
// The formulas are kept in the reference's form (no reformulation): in double
// they are the FP64 oracle, in float they mirror the reference's FP32 GL path.
// Parity status: unpinned (see oracle_math.hpp).
#pragma once

#include "../include/skyr.h"
#include "oracle_math.hpp"

namespace orc {

// AtmosphereBufferData (shaders/SkyRendering/Atmosphere.glsl:6-32)
template <class T>
struct Atmo {
    V3<T> solar_illuminance;
    T sun_angular_radius;
    V3<T> rayleigh_scattering;
    T inv_rayleigh_exponential_distribution;
    V3<T> mie_scattering;
    T inv_mie_exponential_distribution;
    V3<T> mie_absorption;
    T ozone_center_altitude;
    V3<T> ozone_absorption;
    T inv_ozone_width;
    V3<T> ground_albedo;
    T mie_phase_g;
    T multiscattering_mask;
    T bottom_radius, top_radius, transmittance_steps, multiscattering_steps;
};

template <class T>
V3<T> v3f(const float* f) {
    return {T(f[0]), T(f[1]), T(f[2])};
}

// AssignBufferData (src/SkyRendering/Atmosphere.cpp:49-70)
template <class T>
Atmo<T> derive_atmosphere(const skyr_atmosphere_parameters& p) {
    Atmo<T> a;
    a.solar_illuminance = v3f<T>(p.solar_illuminance);
    a.sun_angular_radius = T(p.sun_angular_radius) * T(kPi) / T(180);
    a.rayleigh_scattering = v3f<T>(p.rayleigh_scattering) * T(p.rayleigh_scattering_scale);
    a.mie_scattering = v3f<T>(p.mie_scattering) * T(p.mie_scattering_scale);
    a.mie_absorption = v3f<T>(p.mie_absorption) * T(p.mie_absorption_scale);
    a.ozone_absorption = v3f<T>(p.ozone_absorption) * T(p.ozone_absorption_scale);
    a.inv_rayleigh_exponential_distribution = T(1) / T(p.rayleigh_exponential_distribution);
    a.inv_mie_exponential_distribution = T(1) / T(p.mie_exponential_distribution);
    a.ozone_center_altitude = T(p.ozone_center_altitude);
    a.inv_ozone_width = T(1) / T(p.ozone_width);
    a.ground_albedo = v3f<T>(p.ground_albedo);
    a.bottom_radius = T(p.bottom_radius);
    a.top_radius = T(p.bottom_radius) + T(p.thickness);
    a.mie_phase_g = T(p.mie_phase_g);
    a.transmittance_steps = T(p.transmittance_steps);
    a.multiscattering_steps = T(p.multiscattering_steps);
    a.multiscattering_mask = T(p.multiscattering_mask);
    return a;
}

template <class T>
struct AtmosphereOracle {
    Atmo<T> A;

    T ClampCosine(T mu) const { return clampg(mu, T(-1), T(1)); }
    T ClampDistance(T d) const { return std::max(d, T(0)); }
    T SafeSqrt(T a) const { return std::sqrt(std::max(a, T(0))); }

    // Atmosphere.glsl:57-69
    bool RayIntersectsGround(T r, T mu) const {
        return mu < T(0) && r * r * (mu * mu - T(1)) + A.bottom_radius * A.bottom_radius >= T(0);
    }
    T DistanceToTopAtmosphereBoundary(T r, T mu) const {
        T disc = r * r * (mu * mu - T(1)) + A.top_radius * A.top_radius;
        return ClampDistance(-r * mu + SafeSqrt(disc));
    }
    T DistanceToBottomAtmosphereBoundary(T r, T mu) const {
        T disc = r * r * (mu * mu - T(1)) + A.bottom_radius * A.bottom_radius;
        return ClampDistance(-r * mu - SafeSqrt(disc));
    }

    // Atmosphere.glsl:71-88
    void GetRMuFromTransmittanceTextureIndex(int ix, int iy, int w, int h, T& r, T& mu) const {
        T x_mu = T(ix) / T(w - 1);
        T x_r = T(iy) / T(h - 1);
        T H = std::sqrt(A.top_radius * A.top_radius - A.bottom_radius * A.bottom_radius);
        T rho = H * x_r;
        r = std::sqrt(rho * rho + A.bottom_radius * A.bottom_radius);
        T d_min = A.top_radius - r;
        T d_max = rho + H;
        T d = d_min + x_mu * (d_max - d_min);
        mu = d == T(0) ? T(1) : (H * H - rho * rho - d * d) / (T(2) * r * d);
        mu = ClampCosine(mu);
    }

    // Atmosphere.glsl:53-55,90-103
    V2<T> GetTransmittanceTextureUvFromRMu(int w, int h, T r, T mu) const {
        T H = std::sqrt(A.top_radius * A.top_radius - A.bottom_radius * A.bottom_radius);
        T rho = SafeSqrt(r * r - A.bottom_radius * A.bottom_radius);
        T d = DistanceToTopAtmosphereBoundary(r, mu);
        T d_min = A.top_radius - r;
        T d_max = rho + H;
        T x_mu = (d - d_min) / (d_max - d_min);
        T x_r = rho / H;
        return {T(0.5) / T(w) + x_mu * (T(1) - T(1) / T(w)), T(0.5) / T(h) + x_r * (T(1) - T(1) / T(h))};
    }

    // Atmosphere.glsl:105-117
    V3<T> GetSunVisibility(const Image<T>& tlut, T r, T mu_s) const {
        T sin_theta_h = A.bottom_radius / r;
        T cos_theta_h = -std::sqrt(std::max(T(1) - sin_theta_h * sin_theta_h, T(0)));
        V2<T> uv = GetTransmittanceTextureUvFromRMu(tlut.w, tlut.h, r, mu_s);
        V3<T> t = sample_linear_clamp(tlut, uv.x, uv.y);
        return t * smoothstepg(-sin_theta_h * A.sun_angular_radius, sin_theta_h * A.sun_angular_radius,
                               mu_s - cos_theta_h);
    }

    // Atmosphere.glsl:119-132
    V3<T> GetExtinction(T altitude) const {
        V3<T> rayleigh = A.rayleigh_scattering *
                         clampg(std::exp(-altitude * A.inv_rayleigh_exponential_distribution), T(0), T(1));
        V3<T> mie = (A.mie_scattering + A.mie_absorption) *
                    clampg(std::exp(-altitude * A.inv_mie_exponential_distribution), T(0), T(1));
        T oz = altitude < A.ozone_center_altitude
                   ? T(1) + (altitude - A.ozone_center_altitude) * A.inv_ozone_width
                   : T(1) - (altitude - A.ozone_center_altitude) * A.inv_ozone_width;
        V3<T> ozone = A.ozone_absorption * std::max(T(0), oz);
        return rayleigh + mie + ozone;
    }

    // Atmosphere.glsl:134-159
    T RayleighPhase(T c) const { return T(3) / (T(16) * T(kPi)) * (T(1) + c * c); }
    T MiePhase(T g, T c) const {
        T k = T(3) / (T(8) * T(kPi)) * (T(1) - g * g) / (T(2) + g * g);
        return k * (T(1) + c * c) / std::pow(T(1) + g * g - T(2) * g * c, T(1.5));
    }
    void GetScattering(T altitude, V3<T>& rayleigh, V3<T>& mie) const {
        rayleigh = A.rayleigh_scattering *
                   clampg(std::exp(-altitude * A.inv_rayleigh_exponential_distribution), T(0), T(1));
        mie = A.mie_scattering * clampg(std::exp(-altitude * A.inv_mie_exponential_distribution), T(0), T(1));
    }

    // Atmosphere.glsl:161-178
    V3<T> GetMultiscatteringContribution(const Image<T>& mslut, T r, T mu_s) const {
        T x_mu_s = mu_s * T(0.5) + T(0.5);
        T x_r = (r - A.bottom_radius) / (A.top_radius - A.bottom_radius);
        T u = T(0.5) / T(mslut.w) + x_mu_s * (T(1) - T(1) / T(mslut.w));
        T v = T(0.5) / T(mslut.h) + x_r * (T(1) - T(1) / T(mslut.h));
        return sample_linear_clamp(mslut, u, v);
    }

    // ComputeTransmittanceToTopAtmosphereBoundary (Atmosphere.glsl:311-327)
    V3<T> ComputeTransmittance(T r, T mu) const {
        T steps = A.transmittance_steps;
        T dx = DistanceToTopAtmosphereBoundary(r, mu) / steps;
        V3<T> optical(T(0));
        for (T i = T(0.5); i < steps; i += T(1)) {
            T d_i = i * dx;
            T r_i = std::sqrt(d_i * d_i + T(2) * r * mu * d_i + r * r);
            T alt = r_i - A.bottom_radius;
            optical += GetExtinction(alt) * dx;
        }
        return vexp(-optical);
    }

    // ComputeScatteredLuminance (Atmosphere.glsl:220-295).  `ms` selects the
    // MULTISCATTERING_COMPUTE_PROGRAM variant (isotropic phases, no MS term, no
    // solar illuminance, L_f accumulated, start_i = 0.5).
    V3<T> ComputeScatteredLuminance(const Image<T>& tlut, const Image<T>* mslut, bool ms, T start_i,
                                    V3<T> earth_center, V3<T> start_position, V3<T> view_direction,
                                    V3<T> sun_direction, T marching_distance, T steps, V3<T>& transmittance,
                                    V3<T>* L_f) const {
        T r = length(start_position - earth_center);
        V3<T> up_direction = normalize(start_position - earth_center);
        T mu = dot(view_direction, up_direction);
        T cos_sun_view = dot(view_direction, sun_direction);
        T dx = marching_distance / steps;
        transmittance = V3<T>(T(1));
        V3<T> luminance(T(0));
        if (ms) {
            *L_f = V3<T>(T(0));
            start_i = T(0.5);
        }
        T rayleigh_phase = ms ? T(1) / (T(4) * T(kPi)) : RayleighPhase(cos_sun_view);
        T mie_phase = ms ? T(1) / (T(4) * T(kPi)) : MiePhase(A.mie_phase_g, cos_sun_view);
        for (T i = start_i; i < steps; i += T(1)) {
            T d_i = i * dx;
            T r_i = std::sqrt(d_i * d_i + T(2) * r * mu * d_i + r * r);
            V3<T> position_i = start_position + view_direction * d_i;
            T altitude_i = r_i - A.bottom_radius;
            V3<T> rs, mss;
            GetScattering(altitude_i, rs, mss);
            V3<T> scattering_i = rs + mss;
            V3<T> scattering_with_phase_i = rs * rayleigh_phase + mss * mie_phase;
            V3<T> extinction_i = GetExtinction(altitude_i);
            V3<T> transmittance_i = vexp(-extinction_i * dx);
            V3<T> up_i = normalize(position_i - earth_center);
            T mu_s_i = dot(sun_direction, up_i);
            V3<T> luminance_i = scattering_with_phase_i * GetSunVisibility(tlut, r_i, mu_s_i);
            if (!ms) {
                V3<T> msc = GetMultiscatteringContribution(*mslut, r_i, mu_s_i);
                luminance_i += msc * scattering_i * A.multiscattering_mask;
                luminance_i *= A.solar_illuminance;
            }
            luminance += transmittance * (luminance_i - luminance_i * transmittance_i) / extinction_i;
            if (ms) *L_f += transmittance * (scattering_i - scattering_i * transmittance_i) / extinction_i;
            transmittance *= transmittance_i;
        }
        return luminance;
    }

    // ComputeGroundLuminance (Atmosphere.glsl:297-306)
    V3<T> ComputeGroundLuminance(const Image<T>& tlut, bool ms, V3<T> earth_center, V3<T> position,
                                 V3<T> sun_direction) const {
        V3<T> up = normalize(position - earth_center);
        T mu_s = dot(sun_direction, up);
        V3<T> sun_at_ground = GetSunVisibility(tlut, A.bottom_radius, mu_s);
        if (!ms) sun_at_ground *= A.solar_illuminance;
        V3<T> normal = normalize(position - earth_center);
        return A.ground_albedo * sun_at_ground *
               (T(1) / T(kPi) * clampg(dot(normal, sun_direction), T(0), T(1)));
    }

    // TRANSMITTANCE program (Atmosphere.glsl:329-337)
    void TransmittanceLut(Image<T>& out) const {
        for (int y = 0; y < out.h; ++y)
            for (int x = 0; x < out.w; ++x) TransmittanceTexel(out, x, y);
    }
    void TransmittanceTexel(Image<T>& out, int x, int y) const {
        T r, mu;
        GetRMuFromTransmittanceTextureIndex(x, y, out.w, out.h, r, mu);
        V3<T> t = ComputeTransmittance(r, mu);
        T* p = out.at(x, y);
        p[0] = t.x; p[1] = t.y; p[2] = t.z; p[3] = T(1);
    }

    // GetDirectionFromLocalIndex (Atmosphere.glsl:344-355)
    static V3<T> DirectionFromLocalIndex(int index) {
        T unit_theta = (T(0.5) + T(index / 8)) / T(8);
        T unit_phi = (T(0.5) + T(index % 8)) / T(8);
        T cos_theta = T(1) - T(2) * unit_theta;
        T sin_theta = std::sqrt(clampg(T(1) - cos_theta * cos_theta, T(0), T(1)));
        T phi = T(2) * T(kPi) * unit_phi;
        return {std::cos(phi) * sin_theta, cos_theta, std::sin(phi) * sin_theta};
    }

    // MULTISCATTERING program (Atmosphere.glsl:357-438); the 64-lane tree sum
    // is a plain sum here.
    void MultiscatteringTexel(const Image<T>& tlut, Image<T>& out, int x, int y) const {
        T x_mu_s = T(x) / T(out.w - 1), x_alt = T(y) / T(out.h - 1);
        T altitude = x_alt * (A.top_radius - A.bottom_radius);
        T mu_s = x_mu_s * T(2) - T(1);
        V3<T> earth_center(T(0), -A.bottom_radius, T(0));
        V3<T> start_position(T(0), altitude, T(0));
        V3<T> sun_direction(T(0), mu_s, std::sqrt(T(1) - mu_s * mu_s));
        V3<T> L2(T(0)), fms(T(0));
        for (int k = 0; k < 64; ++k) {
            V3<T> view = DirectionFromLocalIndex(k);
            T r = altitude + A.bottom_radius;
            T mu = view.y;
            bool ground = RayIntersectsGround(r, mu);
            T dist = ground ? DistanceToBottomAtmosphereBoundary(r, mu) : DistanceToTopAtmosphereBoundary(r, mu);
            V3<T> trans, lf;
            V3<T> lum = ComputeScatteredLuminance(tlut, nullptr, true, T(0.5), earth_center, start_position, view,
                                                  sun_direction, dist, A.multiscattering_steps, trans, &lf);
            if (ground) {
                V3<T> gp = start_position + view * dist;
                lum += trans * ComputeGroundLuminance(tlut, true, earth_center, gp, sun_direction);
            }
            L2 += lum;
            fms += lf;
        }
        L2 = L2 / T(64);
        fms = fms / T(64);
        V3<T> F = V3<T>(T(1)) / (V3<T>(T(1)) - fms);
        V3<T> c = L2 * F;
        T* p = out.at(x, y);
        p[0] = c.x; p[1] = c.y; p[2] = c.z; p[3] = T(1);
    }
};

// AtmosphereRenderBufferData fields derived by AssignBufferData
// (src/SkyRendering/AtmosphereRenderer.cpp:52-83) and Earth::center
// (src/SkyRendering/Earth.h:37).
template <class T>
struct RenderFrame {
    V3<T> sun_direction, earth_center, camera_position, up, right, front;
    T camera_earth_center_distance;
    M4<T> inv_view_projection;
    T sky_view_lut_steps, aerial_perspective_lut_steps, aerial_perspective_lut_max_distance;
};

// FromThetaPhiToDirection (src/Base/src/Utils.cpp:23-31)
template <class T>
V3<T> from_theta_phi(T theta, T phi) {
    return {std::cos(phi) * std::sin(theta), std::cos(theta), std::sin(phi) * std::sin(theta)};
}

template <class T>
RenderFrame<T> derive_render_frame(const skyr_atmosphere_parameters& p, const skyr_atmosphere_render_parameters& r) {
    RenderFrame<T> f;
    T deg = T(kPi) / T(180);
    f.sun_direction = from_theta_phi<T>(T(r.sun_direction_theta) * deg, T(r.sun_direction_phi) * deg);
    f.camera_position = v3f<T>(r.camera_position);
    f.inv_view_projection = inverse(mat_from_floats<T>(r.view_projection));
    f.sky_view_lut_steps = T(r.sky_view_lut_steps);
    f.aerial_perspective_lut_steps = T(r.aerial_perspective_lut_steps);
    f.aerial_perspective_lut_max_distance = T(r.aerial_perspective_lut_max_distance);
    f.earth_center = V3<T>(T(0), -T(p.bottom_radius), T(0));
    f.camera_earth_center_distance = length(f.camera_position - f.earth_center);
    f.up = normalize(f.camera_position - f.earth_center);
    f.right = cross(f.sun_direction, f.up);
    T len = length(f.right);
    if (len != T(0)) {
        f.right = f.right / len;
    } else {
        V3<T> biased = from_theta_phi<T>((T(r.sun_direction_theta) + T(90)) * deg, T(r.sun_direction_phi) * deg);
        f.right = normalize(cross(biased, f.up));
    }
    f.front = cross(f.up, f.right);
    return f;
}

template <class T>
struct ViewLutOracle {
    const AtmosphereOracle<T>& O;
    RenderFrame<T> F;

    // FromSpaceIntersectTopAtmosphereBoundary (AtmosphereInterface.glsl:6-13)
    bool FromSpaceIntersectTop(T r, T mu, T& near_distance) const {
        T disc = r * r * (mu * mu - T(1)) + O.A.top_radius * O.A.top_radius;
        if (mu < T(0) && disc >= T(0)) {
            near_distance = O.ClampDistance(-r * mu - O.SafeSqrt(disc));
            return true;
        }
        return false;
    }

    // ComputeRaymarchingStartPositionAndChangeDistance (AtmosphereRenderer.glsl:56-72)
    V3<T> StartPosition(V3<T> view, T& marching_distance) const {
        V3<T> start = F.camera_position;
        if (F.camera_earth_center_distance > O.A.top_radius) {
            T r = F.camera_earth_center_distance;
            T mu = dot(view, F.up);
            T nd;
            if (FromSpaceIntersectTop(r, mu, nd)) {
                start = start + view * nd;
                marching_distance -= nd;
            } else {
                marching_distance = T(0);
            }
        }
        return start;
    }

    // GetHorizonDownAngleFromR / GetCosLatLonFromSkyViewTextureIndex /
    // GetViewDirectionFromCosLatLon (AtmosphereRenderer.glsl:74-111)
    V3<T> SkyViewDirection(int ix, int iy, int w, int h, T r, T& cos_lat) const {
        T x_cos_lon = T(ix) / T(w - 1);
        T x_cos_lat = T(iy) / T(h - 1);
        T tpd = std::sqrt(r * r - O.A.bottom_radius * O.A.bottom_radius);
        T horizon_down = std::acos(tpd / r);
        T horizon_up = T(kPi) - horizon_down;
        T lat;
        if (x_cos_lat < T(0.5)) {
            T c = T(1) - T(2) * x_cos_lat;
            c = T(1) - c * c;
            lat = horizon_up * c;
        } else {
            T c = x_cos_lat * T(2) - T(1);
            c *= c;
            lat = horizon_up + horizon_down * c;
        }
        cos_lat = std::cos(lat);
        T cos_lon = -(x_cos_lon * x_cos_lon * T(2) - T(1));
        T sin_lat = clampg(std::sqrt(T(1) - cos_lat * cos_lat), T(0), T(1));
        T sin_lon = clampg(std::sqrt(T(1) - cos_lon * cos_lon), T(0), T(1));
        return F.up * cos_lat + F.front * (sin_lat * cos_lon) + F.right * (sin_lat * sin_lon);
    }

    // SKY_VIEW program (AtmosphereRenderer.glsl:153-186), start_i = 0.5
    void SkyViewTexel(const Image<T>& tlut, const Image<T>& mslut, Image<T>& lum_out, Image<T>& trans_out, int ix,
                      int iy) const {
        T r = F.camera_earth_center_distance;
        T cos_lat;
        V3<T> view = SkyViewDirection(ix, iy, lum_out.w, lum_out.h, r, cos_lat);
        T mu = cos_lat;
        bool ground = O.RayIntersectsGround(r, mu);
        T dist = ground ? O.DistanceToBottomAtmosphereBoundary(r, mu) : O.DistanceToTopAtmosphereBoundary(r, mu);
        V3<T> start = StartPosition(view, dist);
        V3<T> trans(T(1)), lum(T(0));
        if (dist > T(0)) {
            lum = O.ComputeScatteredLuminance(tlut, &mslut, false, T(0.5), F.earth_center, start, view,
                                              F.sun_direction, dist, F.sky_view_lut_steps, trans, nullptr);
        }
        T* pl = lum_out.at(ix, iy);
        T* pt = trans_out.at(ix, iy);
        pl[0] = lum.x; pl[1] = lum.y; pl[2] = lum.z; pl[3] = T(0);
        pt[0] = trans.x; pt[1] = trans.y; pt[2] = trans.z; pt[3] = T(0);
    }

    // AERIAL_PERSPECTIVE program (AtmosphereRenderer.glsl:191-243), start_i = 0.5
    void AerialPerspectiveTexel(const Image<T>& tlut, const Image<T>& mslut, Image<T>& lum_out, Image<T>& trans_out,
                                int ix, int iy, int iz) const {
        T u = T(ix) / T(lum_out.w - 1), v = T(iy) / T(lum_out.h - 1), w = T(iz) / T(lum_out.d - 1);
        V3<T> pos = projective_mul(F.inv_view_projection, V3<T>(u * T(2) - T(1), v * T(2) - T(1), T(0)));
        V3<T> view = normalize(pos - F.camera_position);
        T marching = w * w * F.aerial_perspective_lut_max_distance;
        T r = F.camera_earth_center_distance;
        T mu = dot(view, F.up);
        bool ground = O.RayIntersectsGround(r, mu);
        T max_marching = ground ? marching : O.DistanceToTopAtmosphereBoundary(r, mu);
        V3<T> start = StartPosition(view, max_marching);
        marching = std::min(marching, max_marching);
        V3<T> trans(T(1)), lum(T(0));
        if (marching > T(0)) {
            lum = O.ComputeScatteredLuminance(tlut, &mslut, false, T(0.5), F.earth_center, start, view,
                                              F.sun_direction, marching, F.aerial_perspective_lut_steps, trans,
                                              nullptr);
        }
        T* pl = lum_out.at(ix, iy, iz);
        T* pt = trans_out.at(ix, iy, iz);
        pl[0] = lum.x; pl[1] = lum.y; pl[2] = lum.z; pl[3] = T(0);
        pt[0] = trans.x; pt[1] = trans.y; pt[2] = trans.z; pt[3] = T(0);
    }
};

}  // namespace orc
