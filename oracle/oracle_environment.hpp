// oracle_environment.hpp — TEST INFRASTRUCTURE ONLY: FP64 restatement of the
// ENVIRONMENT_LUMINANCE program (shaders/SkyRendering/AtmosphereRenderer.glsl:
// 248-275) and of glGenerateTextureMipmap's box filter, the reference the CUDA
// environment cube is checked against.  The path tracer oracle uses the same
// radiance for escaping paths.
#pragma once

#include "oracle_atmosphere.hpp"

namespace orc {

// ConvertCubUvToDir (shaders/Base/Common.glsl:13-30)
template <class T>
V3<T> cube_uv_to_dir(int face, T u, T v) {
    T uc = T(2) * u - T(1), vc = T(2) * v - T(1);
    V3<T> d;
    switch (face) {
        case 0: d = V3<T>(T(1), vc, -uc); break;
        case 1: d = V3<T>(T(-1), vc, uc); break;
        case 2: d = V3<T>(uc, T(1), -vc); break;
        case 3: d = V3<T>(uc, T(-1), vc); break;
        case 4: d = V3<T>(uc, vc, T(1)); break;
        default: d = V3<T>(-uc, vc, T(-1)); break;
    }
    return normalize(d);
}

// GetCosLatLonFromViewDirection + GetSkyViewTextureUvFromCosLatLon
// (AtmosphereRenderer.glsl:113-145) and the sky-view LUT samples for world
// direction w seen from the frame's camera.
template <class T>
void sky_view_sample(const AtmosphereOracle<T>& O, const RenderFrame<T>& F, const Image<T>& svl, const Image<T>& svt,
                     V3<T> w, V3<T>& lum, V3<T>& tr) {
    T cos_lat = dot(F.up, w);
    V3<T> lon = w - F.up * cos_lat;
    T l2 = dot(lon, lon);
    T cos_lon = l2 == T(0) ? T(1) : dot(lon / std::sqrt(l2), F.front);
    T r = F.camera_earth_center_distance;
    T hd = std::acos(std::sqrt(r * r - O.A.bottom_radius * O.A.bottom_radius) / r);
    T hu = T(kPi) - hd;
    T lat = std::acos(clampg(cos_lat, T(-1), T(1)));
    T xl;
    if (lat < hu) xl = T(0.5) - T(0.5) * std::sqrt(T(1) - lat / hu);
    else xl = std::sqrt((lat - hu) / hd) * T(0.5) + T(0.5);
    T xo = std::sqrt(std::max(T(0.5) - T(0.5) * cos_lon, T(0)));
    T u = T(0.5) / T(svl.w) + xo * (T(1) - T(1) / T(svl.w));
    T v = T(0.5) / T(svl.h) + xl * (T(1) - T(1) / T(svl.h));
    lum = sample_linear_clamp(svl, u, v);
    tr = sample_linear_clamp(svt, u, v);
}

// The sky-view lookups and the ground term (AtmosphereRenderer.glsl:258-270)
// for world direction w.
template <class T>
V3<T> environment_luminance(const AtmosphereOracle<T>& O, const RenderFrame<T>& F, const Image<T>& tlut,
                            const Image<T>& svl, const Image<T>& svt, V3<T> w) {
    T cos_lat = dot(F.up, w);
    V3<T> lon = w - F.up * cos_lat;
    T l2 = dot(lon, lon);
    T cos_lon = l2 == T(0) ? T(1) : dot(lon / std::sqrt(l2), F.front);
    T r = F.camera_earth_center_distance;
    T hd = std::acos(std::sqrt(r * r - O.A.bottom_radius * O.A.bottom_radius) / r);
    T hu = T(kPi) - hd;
    T lat = std::acos(clampg(cos_lat, T(-1), T(1)));
    T xl;
    if (lat < hu) xl = T(0.5) - T(0.5) * std::sqrt(T(1) - lat / hu);
    else xl = std::sqrt((lat - hu) / hd) * T(0.5) + T(0.5);
    T xo = std::sqrt(std::max(T(0.5) - T(0.5) * cos_lon, T(0)));
    T u = T(0.5) / T(svl.w) + xo * (T(1) - T(1) / T(svl.w));
    T v = T(0.5) / T(svl.h) + xl * (T(1) - T(1) / T(svl.h));
    V3<T> lum = sample_linear_clamp(svl, u, v);
    V3<T> tr = sample_linear_clamp(svt, u, v);
    if (O.RayIntersectsGround(r, cos_lat)) {
        T dist = O.DistanceToBottomAtmosphereBoundary(r, cos_lat);
        V3<T> gp = F.camera_position + w * dist;
        lum += O.ComputeGroundLuminance(tlut, false, F.earth_center, gp, F.sun_direction) * tr;
    }
    return lum;
}

// Texel (face, x, y) of level 0 of a size^2 cube: the program's face_uv with
// its y flip.
template <class T>
V3<T> environment_cube_texel(const AtmosphereOracle<T>& O, const RenderFrame<T>& F, const Image<T>& tlut,
                             const Image<T>& svl, const Image<T>& svt, int size, int face, int x, int y) {
    T u = (T(x) + T(0.5)) / T(size), v = T(1) - (T(y) + T(0.5)) / T(size);
    return environment_luminance(O, F, tlut, svl, svt, cube_uv_to_dir(face, u, v));
}

// ---- cube sampling with TEXTURE_CUBE_MAP_SEAMLESS (GL 4.6 8.13-8.14) -------
// A cube of `levels` levels, 4 doubles per texel, layout as skyr_environment_cube.
struct CubeImage {
    const double* data;
    int size, levels;
    size_t offset(int l) const {
        size_t off = 0;
        for (int k = 0; k < l; ++k) {
            size_t s = size_t(std::max(size >> k, 1));
            off += 6 * s * s;
        }
        return off;
    }
    int side(int l) const { return std::max(size >> l, 1); }
    const double* texel(int l, int face, int i, int j) const {
        int n = side(l);
        return data + 4 * (offset(l) + (size_t(face) * n + j) * n + i);
    }
};

// face and (s, t) of a direction (GL 4.6 table 8.19), ties to x then y
inline int cube_face(V3<double> d, double& s, double& t) {
    double ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z), sc, tc, ma;
    int face;
    if (ax >= ay && ax >= az) {
        ma = ax;
        face = d.x >= 0 ? 0 : 1;
        sc = d.x >= 0 ? -d.z : d.z;
        tc = -d.y;
    } else if (ay >= az) {
        ma = ay;
        face = d.y >= 0 ? 2 : 3;
        sc = d.x;
        tc = d.y >= 0 ? d.z : -d.z;
    } else {
        ma = az;
        face = d.z >= 0 ? 4 : 5;
        sc = d.z >= 0 ? d.x : -d.x;
        tc = -d.y;
    }
    s = 0.5 * (sc / ma + 1);
    t = 0.5 * (tc / ma + 1);
    return face;
}

// the direction of texel (i, j)'s centre on face `face`, from the inverse of the table
inline V3<double> texel_direction(int face, int i, int j, int n) {
    double sc = 2 * (i + 0.5) / n - 1, tc = 2 * (j + 0.5) / n - 1;
    switch (face) {
        case 0: return V3<double>(1, -tc, -sc);
        case 1: return V3<double>(-1, -tc, sc);
        case 2: return V3<double>(sc, 1, tc);
        case 3: return V3<double>(sc, -1, -tc);
        case 4: return V3<double>(sc, -tc, 1);
        default: return V3<double>(-sc, -tc, -1);
    }
}

inline void cube_neighbour(const CubeImage& C, int l, int face, int i, int j, double out[4]) {
    int n = C.side(l);
    double s, t;
    int f = cube_face(texel_direction(face, i, j, n), s, t);
    int i2 = std::min(std::max(int(std::floor(s * n)), 0), n - 1), j2 = std::min(std::max(int(std::floor(t * n)), 0), n - 1);
    const double* p = C.texel(l, f, i2, j2);
    for (int k = 0; k < 4; ++k) out[k] = p[k];
}

// a texel, past an edge from the adjacent face, past a corner the mean of the three meeting texels
inline void cube_texel(const CubeImage& C, int l, int face, int i, int j, double out[4]) {
    int n = C.side(l);
    bool oi = i < 0 || i >= n, oj = j < 0 || j >= n;
    if (!oi && !oj) {
        const double* p = C.texel(l, face, i, j);
        for (int k = 0; k < 4; ++k) out[k] = p[k];
        return;
    }
    if (oi && oj) {
        int ci = std::min(std::max(i, 0), n - 1), cj = std::min(std::max(j, 0), n - 1);
        double b[4], c[4];
        const double* a = C.texel(l, face, ci, cj);
        cube_neighbour(C, l, face, i, cj, b);
        cube_neighbour(C, l, face, ci, j, c);
        for (int k = 0; k < 4; ++k) out[k] = (a[k] + b[k] + c[k]) / 3.0;
        return;
    }
    cube_neighbour(C, l, face, i, j, out);
}

inline V3<double> cube_bilinear(const CubeImage& C, int l, V3<double> d) {
    int n = C.side(l);
    double s, t;
    int face = cube_face(d, s, t);
    double x = s * n - 0.5, y = t * n - 0.5;
    double fx = std::floor(x), fy = std::floor(y), a = x - fx, b = y - fy;
    int i0 = int(fx), j0 = int(fy);
    double t00[4], t10[4], t01[4], t11[4];
    cube_texel(C, l, face, i0, j0, t00);
    cube_texel(C, l, face, i0 + 1, j0, t10);
    cube_texel(C, l, face, i0, j0 + 1, t01);
    cube_texel(C, l, face, i0 + 1, j0 + 1, t11);
    V3<double> r;
    for (int k = 0; k < 3; ++k) r[k] = (1 - b) * ((1 - a) * t00[k] + a * t10[k]) + b * ((1 - a) * t01[k] + a * t11[k]);
    return r;
}

// textureLod, LINEAR / LINEAR_MIPMAP_LINEAR
inline V3<double> cube_trilinear(const CubeImage& C, V3<double> d, double lod) {
    double lam = std::min(std::max(lod, 0.0), double(C.levels - 1));
    int l0 = int(std::floor(lam));
    double f = lam - l0;
    V3<double> a = cube_bilinear(C, l0, d);
    if (f == 0 || l0 + 1 > C.levels - 1) return a;
    return a + (cube_bilinear(C, l0 + 1, d) - a) * f;
}

// EnvRadianceSH.comp: the 9 coefficients (out[9][3])
inline void environment_sh(const CubeImage& C, double out[9][3]) {
    for (int k = 0; k < 9; ++k)
        for (int c = 0; c < 3; ++c) out[k][c] = 0;
    for (int i = 0; i < 1024; ++i) {
        double ut = (0.5 + (i >> 5)) / 32.0, up = (0.5 + (i & 31)) / 32.0;
        double ct = 1 - 2 * ut, st = std::sqrt(clampg(1 - ct * ct, 0.0, 1.0)), ph = 2 * kPi * up;
        V3<double> d(std::cos(ph) * st, ct, std::sin(ph) * st);
        V3<double> L = cube_bilinear(C, 0, d);
        double y[9] = {0.282095, 0.488603 * d.y, 0.488603 * d.z, 0.488603 * d.x, 1.092548 * d.x * d.y,
                       1.092548 * d.y * d.z, 0.315392 * (3 * d.z * d.z - 1), 1.092548 * d.x * d.z,
                       0.546274 * (d.x * d.x - d.y * d.y)};
        for (int k = 0; k < 9; ++k)
            for (int c = 0; c < 3; ++c) out[k][c] += L[c] * y[k] * (4 * kPi / 1024.0);
    }
}

// PrefilterRadiance.comp: texel (face, x, y) of a level of side n and roughness r
inline V3<double> prefilter_texel(const CubeImage& C, int n, double roughness, int face, int x, int y) {
    double u = (x + 0.5) / n, v = 1 - (y + 0.5) / n;
    V3<double> R = cube_uv_to_dir(face, u, v);
    double a = roughness * roughness, a2 = a * a;
    unsigned ns = unsigned(1.0f + (64.0f - 1.0f) * std::pow(float(roughness), 0.3f));  // GLSL float
    double sg = R.z >= 0 ? 1 : -1, ia = -1 / (sg + R.z), bb = R.x * R.y * ia;
    V3<double> t0(1 + sg * R.x * R.x * ia, sg * bb, -sg * R.x), t1(bb, sg + R.y * R.y * ia, -R.y);
    double inv_sa_texel = (6.0 * n * n) / (4 * kPi);
    V3<double> col(0, 0, 0);
    double wsum = 0;
    for (unsigned i = 0; i < ns; ++i) {
        double e1 = double(i) / ns;
        e1 -= std::floor(e1);
        unsigned b = i;
        b = (b << 16) | (b >> 16);
        b = ((b & 0x00ff00ffu) << 8) | ((b & 0xff00ff00u) >> 8);
        b = ((b & 0x0f0f0f0fu) << 4) | ((b & 0xf0f0f0f0u) >> 4);
        b = ((b & 0x33333333u) << 2) | ((b & 0xccccccccu) >> 2);
        b = ((b & 0x55555555u) << 1) | ((b & 0xaaaaaaaau) >> 1);
        double e2 = double(b) * 2.3283064365386963e-10;
        double phi = 2 * kPi * e1, cth = std::sqrt((1 - e2) / (1 + (a2 - 1) * e2)), sth = std::sqrt(1 - cth * cth);
        V3<double> H = t0 * (sth * std::cos(phi)) + t1 * (sth * std::sin(phi)) + R * cth;
        double vh = dot(R, H);
        V3<double> L = H * (2 * vh) - R;
        double nol = clampg(dot(R, L), 0.0, 1.0);
        if (nol > 0) {
            double noh = clampg(dot(R, H), 0.0, 1.0), hov = clampg(vh, 0.0, 1.0);
            double dd = (noh * a2 - noh) * noh + 1, D = a2 / (kPi * dd * dd);
            double pdf = std::max(D * noh / (4 * hov), 0.0001), sa = 1 / std::max(ns * pdf, 0.00001);
            double lod = roughness == 0 ? 0.0 : 0.5 * std::log2(sa * inv_sa_texel) + 2.5;
            col += cube_trilinear(C, L, lod) * nol;
            wsum += nol;
        }
    }
    return col / wsum;
}

}  // namespace orc
