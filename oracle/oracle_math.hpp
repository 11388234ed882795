// oracle_math.hpp — TEST INFRASTRUCTURE ONLY (the parity checker and the timed
// CPU baseline).  Nothing in the product links this file.
//
// Small GLSL-semantics vector/matrix/sampler helpers templated on the scalar
// type, so that the same restatement runs in double (the oracle) and in float
// (the like-for-like CPU baseline).
//
// Parity status: unpinned.  The reference is GLSL run by an OpenGL driver and
// ships no tests, golden vectors or fixtures; its GL path cannot run on these
// machines.  The oracle is pinned only by the analytic known-answer tests under
// tests/ (closed-form transmittance, top-boundary identity, constant-density
// Beer-Lambert, hash vectors, noise periodicity).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace orc {

constexpr double kPi = 3.1415926535897932384626433832795;

template <class T>
struct V2 {
    T x, y;
};

template <class T>
struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a) : x(a), y(a), z(a) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> operator*(T s, V3<T> a) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> V3<T>& operator+=(V3<T>& a, V3<T> b) { a = a + b; return a; }
template <class T> V3<T>& operator*=(V3<T>& a, V3<T> b) { a = a * b; return a; }
template <class T> V3<T>& operator*=(V3<T>& a, T s) { a = a * s; return a; }

template <class T> T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> V3<T> normalize(V3<T> a) { return a / length(a); }
template <class T> V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> V3<T> vexp(V3<T> a) { return {std::exp(a.x), std::exp(a.y), std::exp(a.z)}; }

// GLSL clamp(x, lo, hi) = min(max(x, lo), hi)
template <class T> T clampg(T x, T lo, T hi) { return std::min(std::max(x, lo), hi); }
template <class T> T mixg(T a, T b, T t) { return a * (T(1) - t) + b * t; }
template <class T> T fractg(T x) { return x - std::floor(x); }
template <class T> T smoothstepg(T e0, T e1, T x) {
    T t = clampg((x - e0) / (e1 - e0), T(0), T(1));
    return t * t * (T(3) - T(2) * t);
}

// Column-major 4x4 matrix (glm memory order): m[c*4 + r].
template <class T>
struct M4 {
    T m[16];
    T operator()(int r, int c) const { return m[c * 4 + r]; }
    T& operator()(int r, int c) { return m[c * 4 + r]; }
};

template <class T>
M4<T> mat_from_floats(const float* f) {
    M4<T> a;
    for (int i = 0; i < 16; ++i) a.m[i] = T(f[i]);
    return a;
}

template <class T>
M4<T> matmul(const M4<T>& a, const M4<T>& b) {
    M4<T> c;
    for (int r = 0; r < 4; ++r)
        for (int col = 0; col < 4; ++col) {
            T s = 0;
            for (int k = 0; k < 4; ++k) s += a(r, k) * b(k, col);
            c(r, col) = s;
        }
    return c;
}

// General 4x4 inverse by Gauss-Jordan elimination with partial pivoting.
template <class T>
M4<T> inverse(const M4<T>& a) {
    T w[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            w[r][c] = a(r, c);
            w[r][c + 4] = (r == c) ? T(1) : T(0);
        }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(w[r][c]) > std::fabs(w[p][c])) p = r;
        if (p != c)
            for (int k = 0; k < 8; ++k) std::swap(w[c][k], w[p][k]);
        T inv = T(1) / w[c][c];
        for (int k = 0; k < 8; ++k) w[c][k] *= inv;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            T f = w[r][c];
            if (f == T(0)) continue;
            for (int k = 0; k < 8; ++k) w[r][k] -= f * w[c][k];
        }
    }
    M4<T> o;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) o(r, c) = w[r][c + 4];
    return o;
}

// ProjectiveMul (shaders/Base/Common.glsl:7-10)
template <class T>
V3<T> projective_mul(const M4<T>& m, V3<T> v) {
    T x = m(0, 0) * v.x + m(0, 1) * v.y + m(0, 2) * v.z + m(0, 3);
    T y = m(1, 0) * v.x + m(1, 1) * v.y + m(1, 2) * v.z + m(1, 3);
    T z = m(2, 0) * v.x + m(2, 1) * v.y + m(2, 2) * v.z + m(2, 3);
    T w = m(3, 0) * v.x + m(3, 1) * v.y + m(3, 2) * v.z + m(3, 3);
    return {x / w, y / w, z / w};
}

template <class T>
V3<T> mul_dir(const M4<T>& m, V3<T> v) {  // mat3(m) * v
    return {m(0, 0) * v.x + m(0, 1) * v.y + m(0, 2) * v.z,
            m(1, 0) * v.x + m(1, 1) * v.y + m(1, 2) * v.z,
            m(2, 0) * v.x + m(2, 1) * v.y + m(2, 2) * v.z};
}

template <class T>
V3<T> mul_point(const M4<T>& m, V3<T> v) {  // (m * vec4(v, 1)).xyz
    return {m(0, 0) * v.x + m(0, 1) * v.y + m(0, 2) * v.z + m(0, 3),
            m(1, 0) * v.x + m(1, 1) * v.y + m(1, 2) * v.z + m(1, 3),
            m(2, 0) * v.x + m(2, 1) * v.y + m(2, 2) * v.z + m(2, 3)};
}

// RGBA image of scalar T, x fastest.
template <class T>
struct Image {
    int w = 0, h = 0, d = 1;
    std::vector<T> px;
    Image() = default;
    Image(int w_, int h_, int d_ = 1) : w(w_), h(h_), d(d_), px(size_t(w_) * h_ * d_ * 4, T(0)) {}
    T* at(int x, int y, int z = 0) { return &px[((size_t(z) * h + y) * w + x) * 4]; }
    const T* at(int x, int y, int z = 0) const { return &px[((size_t(z) * h + y) * w + x) * 4]; }
};

// GL LINEAR filtering with CLAMP_TO_EDGE on a 2D RGBA image; returns rgb.
template <class T>
V3<T> sample_linear_clamp(const Image<T>& img, T u, T v) {
    T x = u * T(img.w) - T(0.5), y = v * T(img.h) - T(0.5);
    T fx = std::floor(x), fy = std::floor(y);
    T a = x - fx, b = y - fy;
    int x0 = int(fx), y0 = int(fy);
    int x1 = std::min(std::max(x0 + 1, 0), img.w - 1);
    int y1 = std::min(std::max(y0 + 1, 0), img.h - 1);
    x0 = std::min(std::max(x0, 0), img.w - 1);
    y0 = std::min(std::max(y0, 0), img.h - 1);
    V3<T> r;
    for (int c = 0; c < 3; ++c) {
        T t00 = img.at(x0, y0)[c], t10 = img.at(x1, y0)[c];
        T t01 = img.at(x0, y1)[c], t11 = img.at(x1, y1)[c];
        r[c] = (T(1) - b) * ((T(1) - a) * t00 + a * t10) + b * ((T(1) - a) * t01 + a * t11);
    }
    return r;
}

// GL LINEAR filtering with CLAMP_TO_EDGE on a 3D RGBA image; returns rgb.
template <class T>
V3<T> sample_linear_clamp3(const Image<T>& img, T u, T v, T w) {
    T x = u * T(img.w) - T(0.5), y = v * T(img.h) - T(0.5), z = w * T(img.d) - T(0.5);
    T fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    T a = x - fx, b = y - fy, g = z - fz;
    int xi[2] = {int(fx), int(fx) + 1}, yi[2] = {int(fy), int(fy) + 1}, zi[2] = {int(fz), int(fz) + 1};
    for (int k = 0; k < 2; ++k) {
        xi[k] = std::min(std::max(xi[k], 0), img.w - 1);
        yi[k] = std::min(std::max(yi[k], 0), img.h - 1);
        zi[k] = std::min(std::max(zi[k], 0), img.d - 1);
    }
    V3<T> r;
    for (int c = 0; c < 3; ++c) {
        T s = 0;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    T wgt = (dx ? a : T(1) - a) * (dy ? b : T(1) - b) * (dz ? g : T(1) - g);
                    s += wgt * img.at(xi[dx], yi[dy], zi[dz])[c];
                }
        r[c] = s;
    }
    return r;
}

}  // namespace orc
