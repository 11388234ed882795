// oracle_quarter.hpp — TEST INFRASTRUCTURE ONLY: FP64 restatement of the
// reference's quarter-resolution cloud pass (VolumetricCloud::Render,
// src/SkyRendering/VolumetricCloud.cpp:327-423): CheckerboardGen.comp,
// VolumetricCloudIndexGen.comp, VolumetricCloudReconstruct.comp and
// VolumetricCloudUpscale.comp (the raymarch itself is CloudOracle::PixelAt).
// It is the reference the CUDA passes are checked against; nothing in the
// library calls it.
//
// textureGather footprints are taken in integers (see gather_base) and a
// texelFetch outside an image reads 0 (GL robust access), as the kernels do.
#pragma once

#include <cmath>
#include <cstdint>

#include "oracle_cloud.hpp"

namespace orc {

struct QuarterDims {
    int W, H, hw, hh, qw, qh;
};

inline QuarterDims quarter_dims(int W, int H) {
    QuarterDims d{W, H, W / 2, H / 2, 0, 0};
    d.qw = d.hw / 2;
    d.qh = d.hh / 2;
    return d;
}

// DepthToLinearDepth (VolumetricCloudCommon.glsl:32-34) with uLinearDepthParam
// (VolumetricCloud.cpp:240)
struct LinearDepth {
    double x, y;
    LinearDepth(double zn, double zf) : x(1.0 / zn), y((zf - zn) / (zf * zn)) {}
    double operator()(double d) const { return 1.0 / (x - y * d); }
};

// the first texel of a textureGather at the centre of texel i of an n-texel
// image from an m-texel texture: floor((i + 0.5) m / n - 0.5)
inline int gather_base(int i, int n, int m) { return int(((long long)(2 * i + 1) * m - n) / (2LL * n)); }

// IndexToOffset (VolumetricCloudCommon.glsl:41-51)
inline void index_offset(unsigned i, int& ox, int& oy) {
    ox = int(((i + 1) >> 1) & 1);
    oy = int(((i + 2) >> 1) & 1);
}

inline int clampi(int v, int lo, int hi) { return std::min(std::max(v, lo), hi); }

// CheckerboardGen.comp:7-13 (depth NULL: an empty depth buffer, 1)
inline void checkerboard(const float* depth, const QuarterDims& D, double* out) {
    for (int y = 0; y < D.hh; ++y)
        for (int x = 0; x < D.hw; ++x) {
            double d = 1.0;
            if (depth) {
                int x0 = std::min(gather_base(x, D.hw, D.W), D.W - 1), y0 = std::min(gather_base(y, D.hh, D.H), D.H - 1);
                int x1 = std::min(x0 + 1, D.W - 1), y1 = std::min(y0 + 1, D.H - 1);
                double v[4] = {depth[size_t(y1) * D.W + x0], depth[size_t(y1) * D.W + x1], depth[size_t(y0) * D.W + x1],
                               depth[size_t(y0) * D.W + x0]};
                bool bmax = (x & 1) == (y & 1);
                d = bmax ? std::max(std::max(v[0], v[1]), std::max(v[2], v[3]))
                         : std::min(std::min(v[0], v[1]), std::min(v[2], v[3]));
            }
            out[size_t(y) * D.hw + x] = d;
        }
}

// VolumetricCloudIndexGen.comp:12-41; out[2 i] = index, out[2 i + 1] = its linear depth
inline void index_gen(const double* cb, const QuarterDims& D, const LinearDepth& LD, int base, double* out) {
    auto pos_to_index = [&](int x, int y) { return (unsigned(base) + unsigned((x + y) & 1)) & 3u; };
    static const int ox[8] = {0, 1, 1, 1, 0, -1, -1, -1}, oy[8] = {1, 1, 0, -1, -1, -1, 0, 1};
    for (int y = 0; y < D.qh; ++y)
        for (int x = 0; x < D.qw; ++x) {
            int x0 = std::min(gather_base(x, D.qw, D.hw), D.hw - 1), y0 = std::min(gather_base(y, D.qh, D.hh), D.hh - 1);
            int x1 = std::min(x0 + 1, D.hw - 1), y1 = std::min(y0 + 1, D.hh - 1);
            double tile[4] = {cb[size_t(y1) * D.hw + x0], cb[size_t(y1) * D.hw + x1], cb[size_t(y0) * D.hw + x1],
                              cb[size_t(y0) * D.hw + x0]};
            unsigned ni = 0, fi = 0;
            for (unsigned i = 1; i < 4; ++i) {
                ni = tile[i] < tile[ni] ? i : ni;
                fi = tile[i] > tile[fi] ? i : fi;
            }
            double nld = LD(tile[ni]), fld = LD(tile[fi]);
            unsigned cn = 0, cf = 0;
            for (int k = 0; k < 8; ++k) {
                int tx = x + ox[k], ty = y + oy[k], dx, dy;
                index_offset(pos_to_index(tx, ty), dx, dy);
                int cx = 2 * tx + dx, cy = 2 * ty + dy;
                double d = (cx >= 0 && cx < D.hw && cy >= 0 && cy < D.hh) ? cb[size_t(cy) * D.hw + cx] : 0.0;
                double ld = LD(d), tol = ld * 0.25;
                if (std::fabs(ld - nld) < tol) ++cn;
                if (std::fabs(ld - fld) < tol) ++cf;
            }
            unsigned idx = cn == 0 ? ni : cf == 0 ? fi : pos_to_index(x, y);
            out[2 * (size_t(y) * D.qw + x)] = double(idx);
            out[2 * (size_t(y) * D.qw + x) + 1] = LD(tile[idx]);
        }
}

inline void reinhard(double c[4]) {
    for (int k = 0; k < 3; ++k) c[k] = c[k] / (1.0 + c[k]);
}
inline void inverse_reinhard(double c[4]) {
    for (int k = 0; k < 3; ++k) c[k] = c[k] / (1.0 - c[k]);
}

// VolumetricCloudReconstruct.comp:28-110 for half-resolution texel (x, y);
// render / previous hold 4 doubles per texel, index 2
inline void reconstruct_texel(const CloudFrame<double>& F, const QuarterDims& D, const LinearDepth& LD,
                              const M4<double>& reproject, bool history, const double* cb, const double* index,
                              const double* render, const double* rdist, const double* previous, int x, int y,
                              double out[4]) {
    double u = (x + 0.5) / D.hw, v = (y + 0.5) / D.hh;
    double depth = cb[size_t(y) * D.hw + x];
    double ld = LD(depth);
    int qx = x >> 1, qy = y >> 1;
    static const int ox[9] = {0, 0, 1, 1, 1, 0, -1, -1, -1}, oy[9] = {0, 1, 1, 0, -1, -1, -1, 0, 1};
    size_t at[9];
    double rld[9], dl[9], mind = 1e10;
    int ni = 0;
    for (int i = 0; i < 9; ++i) {
        at[i] = size_t(clampi(qy + oy[i], 0, D.qh - 1)) * D.qw + clampi(qx + ox[i], 0, D.qw - 1);
        rld[i] = index[2 * at[i] + 1];
        dl[i] = std::fabs(rld[i] - ld);
        if (dl[i] < mind) {
            mind = dl[i];
            ni = i;
        }
    }
    double rn[4], lo[4], hi[4];
    for (int k = 0; k < 4; ++k) rn[k] = render[4 * at[ni] + k];
    reinhard(rn);
    for (int k = 0; k < 4; ++k) lo[k] = hi[k] = rn[k];
    for (int i = 0; i < 9; ++i) {
        double r[4];
        for (int k = 0; k < 4; ++k) r[k] = render[4 * at[i] + k];
        reinhard(r);
        if (dl[i] < rld[i] * 0.3 || std::fabs(r[3] - rn[3]) / std::max(1e-6, 1.0 - std::max(r[3], rn[3])) < 0.2)
            for (int k = 0; k < 4; ++k) {
                lo[k] = std::min(lo[k], r[k]);
                hi[k] = std::max(hi[k], r[k]);
            }
    }
    bool inside = qx < D.qw && qy < D.qh;  // texelFetch at pos >> 1
    size_t q = size_t(qy) * D.qw + qx;
    double rendered[4] = {0, 0, 0, 0};
    if (inside)
        for (int k = 0; k < 4; ++k) rendered[k] = render[4 * q + k];
    reinhard(rendered);
    V3<double> frag = projective_mul(F.inv_mvp, V3<double>(u * 2 - 1, v * 2 - 1, depth * 2 - 1));
    V3<double> view = normalize(frag - F.cam);
    double rd = inside ? rdist[q] : 0.0;
    V3<double> cp = F.cam + view * rd;
    // ProjectiveMul(uReprojectMat, cloud_pos).xy
    double hx = reproject(0, 0) * cp.x + reproject(0, 1) * cp.y + reproject(0, 2) * cp.z + reproject(0, 3);
    double hy = reproject(1, 0) * cp.x + reproject(1, 1) * cp.y + reproject(1, 2) * cp.z + reproject(1, 3);
    double hw = reproject(3, 0) * cp.x + reproject(3, 1) * cp.y + reproject(3, 2) * cp.z + reproject(3, 3);
    double pnx = hx / hw, pny = hy / hw;
    double pre[4] = {0, 0, 0, 0};
    if (history) {  // LINEAR + CLAMP_TO_EDGE
        double px = (pnx * 0.5 + 0.5) * D.hw - 0.5, py = (pny * 0.5 + 0.5) * D.hh - 0.5;
        double fx = std::floor(px), fy = std::floor(py), a = px - fx, b = py - fy;
        int xi[2] = {clampi(int(fx), 0, D.hw - 1), clampi(int(fx) + 1, 0, D.hw - 1)};
        int yi[2] = {clampi(int(fy), 0, D.hh - 1), clampi(int(fy) + 1, 0, D.hh - 1)};
        for (int k = 0; k < 4; ++k) {
            double t00 = previous[4 * (size_t(yi[0]) * D.hw + xi[0]) + k], t10 = previous[4 * (size_t(yi[0]) * D.hw + xi[1]) + k];
            double t01 = previous[4 * (size_t(yi[1]) * D.hw + xi[0]) + k], t11 = previous[4 * (size_t(yi[1]) * D.hw + xi[1]) + k];
            pre[k] = (1 - b) * ((1 - a) * t00 + a * t10) + b * ((1 - a) * t01 + a * t11);
        }
    }
    reinhard(pre);
    for (int k = 0; k < 4; ++k) pre[k] = clampg(pre[k], lo[k], hi[k]);
    bool out_of_screen = std::max(std::fabs(pnx), std::fabs(pny)) > 1.0;
    unsigned ri = inside ? unsigned(int(index[2 * q])) & 3u : 0u;
    int dx, dy;
    index_offset(ri, dx, dy);
    bool is_rendered = (x & 1) == dx && (y & 1) == dy;
    double w = (!history || out_of_screen) ? 1.0 : is_rendered ? 0.2 : 0.0;
    for (int k = 0; k < 4; ++k) out[k] = mixg(pre[k], rendered[k], w);
    inverse_reinhard(out);
}

// VolumetricCloudUpscale.comp:11-55 for pixel (x, y); hdr_in / out 4 doubles
inline void upscale_pixel(const QuarterDims& D, const LinearDepth& LD, const float* depth, const double* cb,
                          const double* rec, const double* hdr_in, int x, int y, double out[4]) {
    double ld = LD(depth ? double(depth[size_t(y) * D.W + x]) : 1.0);
    static const int ox[4] = {-1, 1, 1, -1}, oy[4] = {1, 1, -1, -1};
    double n[4][4], mind = 1e10;
    int ni = 0;
    bool edge = false;
    for (int i = 0; i < 4; ++i) {
        size_t h = size_t(clampi((y + oy[i]) >> 1, 0, D.hh - 1)) * D.hw + clampi((x + ox[i]) >> 1, 0, D.hw - 1);
        for (int k = 0; k < 4; ++k) n[i][k] = rec[4 * h + k];
        double dlt = std::fabs(ld - LD(cb[h]));
        if (dlt < mind) {
            ni = i;
            mind = dlt;
        }
        if (dlt > ld * 0.1) edge = true;
    }
    double max_a = std::max(std::max(n[0][3], n[1][3]), std::max(n[2][3], n[3][3]));
    double min_a = std::min(std::min(n[0][3], n[1][3]), std::min(n[2][3], n[3][3]));
    double up[4];
    bool pick = edge && (max_a - min_a) / std::max(1e-6, 1.0 - min_a) > 0.2;
    for (int k = 0; k < 4; ++k) up[k] = pick ? n[ni][k] : ((n[0][k] + n[1][k]) + (n[2][k] + n[3][k])) * 0.25;
    size_t p = size_t(y) * D.W + x;
    double t = up[3] <= 0.01 ? 0.0 : up[3];
    for (int k = 0; k < 3; ++k) out[k] = hdr_in[4 * p + k] * t + up[k];
    out[3] = hdr_in[4 * p + 3];
}

}  // namespace orc
