// oracle_mlp.hpp — test infrastructure only (never linked into the product):
// FP64 restatement of the surrogate network of include/skyr_mlp.h, its
// relative-L2 loss, the analytic backward pass and one Adam step.
//
// The network has no counterpart in the reference (it stands in for the
// multiple-scattering heuristic of VolumetricCloudRender.comp:125-130), so
// there is nothing of the reference to pin: the forward / backward formulas are
// checked against central finite differences of this same FP64 code, and the
// GPU kernels are checked against this code.
//
// With `mirror` set, the values the GPU rounds to BF16 are rounded here at the
// same points: the weights, each hidden activation after ReLU, and the
// back-propagated dZ that feeds the weight-gradient and dX products (the bias
// gradients use the unrounded dZ, as on the GPU).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace orc {

constexpr int kMlpIn = 103, kMlpWidth = 64, kMlpOut = 3, kMlpLayers = 5;
constexpr int kMlpParams = 19331;

inline int mlp_fan_in(int l) { return l == 0 ? kMlpIn : kMlpWidth; }
inline int mlp_fan_out(int l) { return l == kMlpLayers - 1 ? kMlpOut : kMlpWidth; }
// offset of layer l's weights in the parameter vector; its biases follow them
inline int mlp_w_offset(int l) {
    int o = 0;
    for (int i = 0; i < l; ++i) o += mlp_fan_in(i) * mlp_fan_out(i) + mlp_fan_out(i);
    return o;
}
inline int mlp_b_offset(int l) { return mlp_w_offset(l) + mlp_fan_in(l) * mlp_fan_out(l); }

// round-to-nearest-even to bfloat16, value returned as float
inline float bf16_round(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;  // inf / nan unchanged
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
inline double bf16_to_float(uint16_t h) {
    uint32_t u = (uint32_t)h << 16;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
inline double bfr(double x, bool mirror) { return mirror ? (double)bf16_round((float)x) : x; }

struct MlpOracle {
    std::vector<double> p;  // parameters (BF16-rounded weights when mirroring)
    bool mirror = false;

    MlpOracle(const float* params, bool mirror_bf16) : p(kMlpParams), mirror(mirror_bf16) {
        for (int l = 0; l < kMlpLayers; ++l) {
            int w = mlp_w_offset(l), b = mlp_b_offset(l), nw = mlp_fan_in(l) * mlp_fan_out(l);
            for (int i = 0; i < nw; ++i) p[w + i] = bfr(params[w + i], mirror);
            for (int i = 0; i < mlp_fan_out(l); ++i) p[b + i] = params[b + i];
        }
    }
    double W(int l, int o, int i) const { return p[mlp_w_offset(l) + o * mlp_fan_in(l) + i]; }
    double B(int l, int o) const { return p[mlp_b_offset(l) + o]; }

    // forward of one sample; h[l] are the layer inputs (h[0] = x), z the
    // pre-activations of every layer, y the outputs
    void forward(const double* x, std::vector<double> h[kMlpLayers], std::vector<double> z[kMlpLayers],
                 double* y) const {
        h[0].assign(x, x + kMlpIn);
        for (int l = 0; l < kMlpLayers; ++l) {
            int fi = mlp_fan_in(l), fo = mlp_fan_out(l);
            z[l].assign(fo, 0.0);
            for (int o = 0; o < fo; ++o) {
                double s = B(l, o);
                for (int i = 0; i < fi; ++i) s += W(l, o, i) * h[l][i];
                z[l][o] = s;
            }
            if (l + 1 < kMlpLayers) {
                h[l + 1].assign(fo, 0.0);
                for (int o = 0; o < fo; ++o) h[l + 1][o] = bfr(z[l][o] > 0.0 ? z[l][o] : 0.0, mirror);
            }
        }
        for (int o = 0; o < kMlpOut; ++o) y[o] = z[kMlpLayers - 1][o];
    }

    void predict(const double* x, double* y) const {
        std::vector<double> h[kMlpLayers], z[kMlpLayers];
        forward(x, h, z, y);
    }

    // Mean over the n samples and 3 outputs of (y - t/scale)^2 / (y_sg^2 + eps),
    // y_sg the prediction held constant (stop-gradient); its gradient is added
    // to grad[kMlpParams].
    double gradient(const double* x, const double* t, int n, double label_scale, double loss_eps,
                    double* grad) const {
        double loss = 0.0;
        std::vector<double> h[kMlpLayers], z[kMlpLayers];
        std::vector<double> dz, dzr, dh;
        for (int s = 0; s < n; ++s) {
            double y[kMlpOut];
            forward(x + (size_t)s * kMlpIn, h, z, y);
            dz.assign(kMlpOut, 0.0);
            for (int c = 0; c < kMlpOut; ++c) {
                double d = y[c] - t[(size_t)s * kMlpOut + c] / label_scale;
                double w = 1.0 / (y[c] * y[c] + loss_eps);
                loss += d * d * w / (3.0 * n);
                dz[c] = 2.0 * d * w / (3.0 * n);
            }
            for (int l = kMlpLayers - 1; l >= 0; --l) {
                int fi = mlp_fan_in(l), fo = mlp_fan_out(l);
                dzr.assign(fo, 0.0);
                for (int o = 0; o < fo; ++o) {
                    dzr[o] = bfr(dz[o], mirror);
                    grad[mlp_b_offset(l) + o] += dz[o];
                    for (int i = 0; i < fi; ++i) grad[mlp_w_offset(l) + o * fi + i] += dzr[o] * h[l][i];
                }
                if (l == 0) break;
                dh.assign(fi, 0.0);
                for (int i = 0; i < fi; ++i) {
                    double sacc = 0.0;
                    for (int o = 0; o < fo; ++o) sacc += dzr[o] * W(l, o, i);
                    dh[i] = z[l - 1][i] > 0.0 ? sacc : 0.0;
                }
                dz = dh;
            }
        }
        return loss;
    }
};

// One Adam step (bias-corrected, step = 1-based count after this update)
inline void adam_step(double* p, double* m, double* v, const double* g, int n, double lr, double b1, double b2,
                      double eps, int step) {
    double c1 = 1.0 - std::pow(b1, step), c2 = 1.0 - std::pow(b2, step);
    for (int i = 0; i < n; ++i) {
        m[i] = b1 * m[i] + (1.0 - b1) * g[i];
        v[i] = b2 * v[i] + (1.0 - b2) * g[i] * g[i];
        p[i] -= lr * (m[i] / c1) / (std::sqrt(v[i] / c2) + eps);
    }
}

}  // namespace orc
