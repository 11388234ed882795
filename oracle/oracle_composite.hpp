// oracle_composite.hpp — TEST INFRASTRUCTURE ONLY: FP64 restatement of the
// ATMOSPHERE_RENDER fragment shader (shaders/SkyRendering/AtmosphereRenderer.glsl:
// 325-432) without the G-buffer shading, which the caller supplies as an
// object luminance.  The reference the CUDA composite is checked against.
#pragma once

#include <cmath>
#include <cstdint>

#include "oracle_environment.hpp"
#include "../include/skyr_composite.h"

namespace orc {

struct CompositeOracle {
    const AtmosphereOracle<double>& O;
    const ViewLutOracle<double>& VL;
    const Image<double>& tlut;
    const Image<double>& ms;
    const Image<double>& svl;
    const Image<double>& svt;
    const Image<double>& apl;
    const Image<double>& apt;
    skyr_composite_parameters P;
    skyr_composite_inputs I;  // host pointers

    static double srgb(uint8_t b) {
        double c = b / 255.0;
        return c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4);
    }

    // GetStarLuminance (:325-330), LINEAR + CLAMP_TO_EDGE, sRGB decoded per texel
    V3<double> Star(V3<double> view) const {
        double theta = std::acos(clampg(view.y, -1.0, 1.0)), phi = std::atan2(view.x, view.z);
        double u = 0.5 / kPi * phi + 0.5, v = 1 - theta / kPi;
        double x = u * I.star_width - 0.5, y = v * I.star_height - 0.5;
        double fx = std::floor(x), fy = std::floor(y), a = x - fx, b = y - fy;
        int xi[2], yi[2];
        for (int k = 0; k < 2; ++k) {
            xi[k] = std::min(std::max(int(fx) + k, 0), I.star_width - 1);
            yi[k] = std::min(std::max(int(fy) + k, 0), I.star_height - 1);
        }
        V3<double> r(0.0);
        for (int c = 0; c < 3; ++c) {
            auto t = [&](int i, int j) { return srgb(I.star_map[(size_t(yi[j]) * I.star_width + xi[i]) * 3 + c]); };
            r[c] = (1 - b) * ((1 - a) * t(0, 0) + a * t(1, 0)) + b * ((1 - a) * t(0, 1) + a * t(1, 1));
        }
        return r * double(P.star_luminance_scale);
    }

    // SampleRayScatterVisibility (VolumetricCloudShadowInterface.glsl:10-13)
    double Visibility(double u, double v, double dist) const {
        if (!I.shadow_froxel) return 1.0;
        double w = dist / I.shadow_froxel_max_distance;
        double c[3] = {u * I.froxel_width - 0.5, v * I.froxel_height - 0.5, w * I.froxel_depth - 0.5};
        int n[3] = {I.froxel_width, I.froxel_height, I.froxel_depth}, i0[3], i1[3];
        double f[3];
        for (int k = 0; k < 3; ++k) {
            double fl = std::floor(c[k]);
            f[k] = c[k] - fl;
            i0[k] = std::min(std::max(int(fl), 0), n[k] - 1);
            i1[k] = std::min(std::max(int(fl) + 1, 0), n[k] - 1);
        }
        double s = 0;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    int x = dx ? i1[0] : i0[0], y = dy ? i1[1] : i0[1], z = dz ? i1[2] : i0[2];
                    double wgt = (dx ? f[0] : 1 - f[0]) * (dy ? f[1] : 1 - f[1]) * (dz ? f[2] : 1 - f[2]);
                    s += wgt * I.shadow_froxel[(size_t(z) * n[1] + y) * n[0] + x] / 65535.0;
                }
        return mixg(1.0, s, clampg(1.0 / w, 0.0, 1.0));
    }

    // main (:345-432) for pixel (px, py)
    void Pixel(int px, int py, double out[4]) const {
        const RenderFrame<double>& F = VL.F;
        size_t pix = size_t(py) * I.width + px;
        double depth = I.depth ? double(I.depth[pix]) : 1.0;
        double u = (px + 0.5) / I.width, v = (py + 0.5) / I.height;
        V3<double> frag = projective_mul(F.inv_view_projection, V3<double>(u * 2 - 1, v * 2 - 1, depth * 2 - 1));
        V3<double> view = normalize(frag - F.camera_position);
        double r = F.camera_earth_center_distance, mu = dot(view, F.up);
        double marching = O.RayIntersectsGround(r, mu) ? O.DistanceToBottomAtmosphereBoundary(r, mu)
                                                        : O.DistanceToTopAtmosphereBoundary(r, mu);
        bool object = depth != 1.0;
        if (object) marching = std::min(marching, length(frag - F.camera_position));
        V3<double> start = VL.StartPosition(view, marching);
        V3<double> tr(1.0), lum(0.0);
        if (marching > 0) {
            if (!object && P.use_sky_view_lut) {
                sky_view_sample(O, F, svl, svt, view, lum, tr);
            } else if (object && P.use_aerial_perspective_lut) {
                double w = std::sqrt(marching / F.aerial_perspective_lut_max_distance);
                double uu = 0.5 / apl.w + u * (1 - 1.0 / apl.w), vv = 0.5 / apl.h + v * (1 - 1.0 / apl.h),
                       ww = 0.5 / apl.d + w * (1 - 1.0 / apl.d);
                lum = sample_linear_clamp3(apl, uu, vv, ww);
                tr = sample_linear_clamp3(apt, uu, vv, ww);
            } else {
                double start_i = P.dither_sample_point ? double(I.blue_noise[(py & 63) * 64 + (px & 63)]) : 0.5;
                lum = O.ComputeScatteredLuminance(tlut, &ms, false, start_i, F.earth_center, start, view,
                                                  F.sun_direction, marching, double(P.raymarching_steps), tr, nullptr);
            }
        }
        lum = lum * Visibility(u, v, marching);
        double sar = O.A.sun_angular_radius;
        double nu = dot(view, F.sun_direction);
        if (object) {
            if (I.object_luminance)
                for (int c = 0; c < 3; ++c) lum[c] += tr[c] * double(I.object_luminance[4 * pix + c]);
        } else if (nu >= std::cos(sar)) {
            static const double a[3] = {0.397, 0.503, 0.652};
            double sin_vs = std::sqrt(1 - nu * nu);
            double c2e = clampg(sin_vs / std::sin(sar), 0.0, 1.0), m = std::sqrt(1 - c2e * c2e);
            for (int c = 0; c < 3; ++c)
                lum[c] += O.A.solar_illuminance[c] * tr[c] / (kPi * sar * sar) * (1 - (1 - std::pow(m, a[c])));
        } else if (I.star_map) {
            lum = lum + tr * Star(view);
        }
        out[0] = lum.x;
        out[1] = lum.y;
        out[2] = lum.z;
        out[3] = 1.0;
    }
};

}  // namespace orc
