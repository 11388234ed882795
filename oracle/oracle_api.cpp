// oracle_api.cpp — TEST INFRASTRUCTURE ONLY: extern "C" surface of the CPU
// oracle (precision 64) and of the like-for-like CPU baseline (precision 32),
// loaded by tests/ and bench.py through ctypes.  Parity status: unpinned
// (see oracle_math.hpp).
#include <atomic>
#include <memory>
#include <cstring>
#include <thread>

#include "oracle_atmosphere.hpp"
#include "oracle_cloud.hpp"
#include "oracle_noise.hpp"
#include "oracle_pathtrace.hpp"
#include "oracle_shadow.hpp"
#include "oracle_quarter.hpp"
#include "oracle_environment.hpp"
#include "oracle_composite.hpp"
#include "../include/skyr_cloud_shadow.h"
#include "../include/skyr_surrogate.h"

namespace {

template <class F>
void parallel_for(int n, int threads, F&& fn) {
    if (threads <= 1 || n <= 1) {
        for (int i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    int nt = std::min(threads, n);
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&] {
            for (int i = next.fetch_add(1); i < n; i = next.fetch_add(1)) fn(i);
        });
    for (auto& th : pool) th.join();
}

template <class T>
orc::Image<T> image_from(const double* src, int w, int h, int d = 1) {
    orc::Image<T> img(w, h, d);
    for (size_t i = 0; i < img.px.size(); ++i) img.px[i] = T(src[i]);
    return img;
}

template <class T>
void image_to(const orc::Image<T>& img, double* dst) {
    if (!dst) return;
    for (size_t i = 0; i < img.px.size(); ++i) dst[i] = double(img.px[i]);
}

template <class T>
void transmittance(const skyr_atmosphere_parameters* p, int w, int h, int threads, orc::Image<T>& out) {
    orc::AtmosphereOracle<T> O{orc::derive_atmosphere<T>(*p)};
    out = orc::Image<T>(w, h);
    parallel_for(h, threads, [&](int y) {
        for (int x = 0; x < w; ++x) O.TransmittanceTexel(out, x, y);
    });
}

template <class T>
void multiscattering(const skyr_atmosphere_parameters* p, const orc::Image<T>& tlut, int w, int h, int threads,
                     orc::Image<T>& out) {
    orc::AtmosphereOracle<T> O{orc::derive_atmosphere<T>(*p)};
    out = orc::Image<T>(w, h);
    parallel_for(h * w, threads, [&](int i) { O.MultiscatteringTexel(tlut, out, i % w, i / w); });
}

template <class T>
void view_luts(const skyr_atmosphere_parameters* p, const skyr_atmosphere_render_parameters* r,
               const skyr_lut_sizes* s, const orc::Image<T>& tlut, const orc::Image<T>& mslut, int threads,
               orc::Image<T>& svl, orc::Image<T>& svt, orc::Image<T>& apl, orc::Image<T>& apt, bool do_sv,
               bool do_ap) {
    orc::AtmosphereOracle<T> O{orc::derive_atmosphere<T>(*p)};
    orc::ViewLutOracle<T> V{O, orc::derive_render_frame<T>(*p, *r)};
    if (do_sv) {
        svl = orc::Image<T>(s->sky_view_width, s->sky_view_height);
        svt = orc::Image<T>(s->sky_view_width, s->sky_view_height);
        parallel_for(s->sky_view_height, threads, [&](int y) {
            for (int x = 0; x < s->sky_view_width; ++x) V.SkyViewTexel(tlut, mslut, svl, svt, x, y);
        });
    }
    if (do_ap) {
        int W = s->aerial_perspective_width, H = s->aerial_perspective_height, D = s->aerial_perspective_depth;
        apl = orc::Image<T>(W, H, D);
        apt = orc::Image<T>(W, H, D);
        parallel_for(H * D, threads, [&](int i) {
            int y = i % H, z = i / H;
            for (int x = 0; x < W; ++x) V.AerialPerspectiveTexel(tlut, mslut, apl, apt, x, y, z);
        });
    }
}

template <class T>
int lut_set(const skyr_atmosphere_parameters* p, const skyr_atmosphere_render_parameters* r,
            const skyr_lut_sizes* s, int threads, double* t_out, double* ms_out, double* svl_out, double* svt_out,
            double* apl_out, double* apt_out) {
    orc::Image<T> tl, ms, svl, svt, apl, apt;
    transmittance<T>(p, s->transmittance_width, s->transmittance_height, threads, tl);
    multiscattering<T>(p, tl, s->multiscattering_width, s->multiscattering_height, threads, ms);
    bool views = r != nullptr && (svl_out || svt_out || apl_out || apt_out);
    if (views) view_luts<T>(p, r, s, tl, ms, threads, svl, svt, apl, apt, svl_out || svt_out, apl_out || apt_out);
    image_to(tl, t_out);
    image_to(ms, ms_out);
    if (views) {
        image_to(svl, svl_out);
        image_to(svt, svt_out);
        image_to(apl, apl_out);
        image_to(apt, apt_out);
    }
    return 0;
}

}  // namespace

extern "C" {

// Whole LUT set from parameters alone (transmittance -> MS -> sky-view/AP).
// Any output pointer may be null.  precision: 64 (oracle) or 32 (baseline).
int oracle_lut_set(const skyr_atmosphere_parameters* p, const skyr_atmosphere_render_parameters* r,
                   const skyr_lut_sizes* s, int precision, int threads, double* t_out, double* ms_out,
                   double* svl_out, double* svt_out, double* apl_out, double* apt_out) {
    if (precision == 32) return lut_set<float>(p, r, s, threads, t_out, ms_out, svl_out, svt_out, apl_out, apt_out);
    return lut_set<double>(p, r, s, threads, t_out, ms_out, svl_out, svt_out, apl_out, apt_out);
}

// Multi-scattering LUT from a given transmittance LUT (stage isolation).
int oracle_multiscattering(const skyr_atmosphere_parameters* p, const skyr_lut_sizes* s, const double* t_in,
                           int threads, double* ms_out) {
    orc::Image<double> tl = image_from<double>(t_in, s->transmittance_width, s->transmittance_height);
    orc::Image<double> ms;
    multiscattering<double>(p, tl, s->multiscattering_width, s->multiscattering_height, threads, ms);
    image_to(ms, ms_out);
    return 0;
}

// Sky-view and AP LUTs from given transmittance and MS LUTs (stage isolation).
int oracle_view_luts(const skyr_atmosphere_parameters* p, const skyr_atmosphere_render_parameters* r,
                     const skyr_lut_sizes* s, const double* t_in, const double* ms_in, int threads, double* svl_out,
                     double* svt_out, double* apl_out, double* apt_out) {
    orc::Image<double> tl = image_from<double>(t_in, s->transmittance_width, s->transmittance_height);
    orc::Image<double> ms = image_from<double>(ms_in, s->multiscattering_width, s->multiscattering_height);
    orc::Image<double> svl, svt, apl, apt;
    bool sv = svl_out || svt_out, ap = apl_out || apt_out;
    view_luts<double>(p, r, s, tl, ms, threads, svl, svt, apl, apt, sv, ap);
    if (sv) { image_to(svl, svl_out); image_to(svt, svt_out); }
    if (ap) { image_to(apl, apl_out); image_to(apt, apt_out); }
    return 0;
}

// Transmittance at an arbitrary (r, mu) by the reference integrator, FP64.
int oracle_transmittance_at(const skyr_atmosphere_parameters* p, double r, double mu, double* out3) {
    orc::AtmosphereOracle<double> O{orc::derive_atmosphere<double>(*p)};
    orc::V3<double> t = O.ComputeTransmittance(r, mu);
    out3[0] = t.x; out3[1] = t.y; out3[2] = t.z;
    return 0;
}

}  // extern "C"

// ---- noise ---------------------------------------------------------------
namespace {

int noise_levels(const skyr_noise_texture_desc* d) {
    int m = std::max(d->width, std::max(d->height, d->depth)), l = 1;
    while ((m >> l) > 0) ++l;
    return l;
}

size_t level_bytes(const skyr_noise_texture_desc* d, int l) {
    return (size_t)std::max(d->width >> l, 1) * std::max(d->height >> l, 1) * std::max(d->depth >> l, 1) *
           d->channels;
}

}  // namespace

extern "C" {

// Mip chain of levels 1.. from level 0 already in `tex` (bit-exact integer work).
int oracle_noise_mips(const skyr_noise_texture_desc* d, uint8_t* tex) {
    size_t off = 0;
    int L = noise_levels(d);
    for (int l = 0; l + 1 < L; ++l) {
        size_t nb = level_bytes(d, l);
        orc::box_reduce(tex + off, std::max(d->width >> l, 1), std::max(d->height >> l, 1),
                        std::max(d->depth >> l, 1), tex + off + nb, d->channels);
        off += nb;
    }
    return 0;
}

// Level 0 and the mip chain.  precision 64 or 32.
int oracle_noise_generate(const skyr_noise_texture_desc* d, int precision, int threads, uint8_t* tex) {
    int w = d->width, h = d->height, dd = d->depth;
    size_t plane = (size_t)w * h * dd;
    parallel_for(h * dd, threads, [&](int row) {
        int y = row % h, z = row / h;
        for (int c = 0; c < d->channels; ++c)
            for (int x = 0; x < w; ++x) {
                uint8_t b = precision == 32
                                ? orc::unorm8(orc::channel_value<float>(d->channel[c], x, y, z, w, h, dd, d->octaves))
                                : orc::unorm8(orc::channel_value<double>(d->channel[c], x, y, z, w, h, dd, d->octaves));
                tex[c * plane + ((size_t)z * h + y) * w + x] = b;
            }
    });
    return oracle_noise_mips(d, tex);
}

// Noise values (unquantised) at level-0 texels, for error analysis.
int oracle_noise_values(const skyr_noise_texture_desc* d, int channel, const int* idx, int n, double* out) {
    int w = d->width, h = d->height, dd = d->depth;
    for (int i = 0; i < n; ++i) {
        int x = idx[i] % w, y = (idx[i] / w) % h, z = idx[i] / (w * h);
        out[i] = orc::channel_value<double>(d->channel[channel], x, y, z, w, h, dd, d->octaves);
    }
    return 0;
}

uint32_t oracle_wang_hash(uint32_t x) { return orc::WangHash(x); }
uint32_t oracle_pcg_hash(uint32_t x) { return orc::PCGHash(x); }

}  // extern "C"

// ---- cloud raymarch --------------------------------------------------------
namespace {

template <class T>
int cloud_render_t(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                          const skyr_cloud_material* m, const skyr_cloud_textures* tx, const skyr_cloud_view* v,
                          const skyr_lut_sizes* s, const double* tlut_in, const double* apl_in,
                          const double* apt_in, const float* blue_noise, const float* depth, const int* pixels,
                          int n_pixels, int threads, double* out_rgba, double* out_dist) {
    orc::AtmosphereOracle<T> O{orc::derive_atmosphere<T>(*atmo)};
    orc::Image<T> tl = image_from<T>(tlut_in, s->transmittance_width, s->transmittance_height);
    int W = s->aerial_perspective_width, H = s->aerial_perspective_height, D = s->aerial_perspective_depth;
    orc::Image<T> al = image_from<T>(apl_in, W, H, D), at = image_from<T>(apt_in, W, H, D);
    orc::CloudOracle<T> C{O, orc::derive_cloud_frame<T>(*atmo, *cp, *m, *tx, *v), {}, {}, {}, {}, nullptr,
                          nullptr, nullptr, nullptr};
    auto set = [](orc::Tex8& t, const void* p, const skyr_noise_texture_desc& d, bool border) {
        t.data = (const uint8_t*)p;
        t.w = d.width; t.h = d.height; t.d = d.depth; t.channels = d.channels;
        t.border = border;
        t.init();
    };
    set(C.cloud_map, tx->cloud_map, tx->cloud_map_desc, false);
    set(C.detail, tx->detail, tx->detail_desc, false);
    set(C.displacement, tx->displacement, tx->displacement_desc, false);
    set(C.voxel, tx->voxel, tx->voxel_desc, true);
    C.tlut = &tl;
    C.ap_lum = &al;
    C.ap_trans = &at;
    C.blue_noise = blue_noise;
    parallel_for(n_pixels, threads, [&](int i) {
        int p = pixels ? pixels[i] : i;
        int px = p % v->width, py = p / v->width;
        T rgba[4], dist;
        C.Pixel(px, py, v->width, v->height, depth ? depth[p] : 1.0f, rgba, dist);
        for (int k = 0; k < 4; ++k) out_rgba[(size_t)i * 4 + k] = double(rgba[k]);
        if (out_dist) out_dist[i] = double(dist);
    });
    return 0;
}

}  // namespace

extern "C" {

// Raymarch the listed pixels (or all when pixels == NULL) of the view.
int oracle_cloud_render(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                        const skyr_cloud_material* m, const skyr_cloud_textures* tx, const skyr_cloud_view* v,
                        const skyr_lut_sizes* s, const double* tlut, const double* apl, const double* apt,
                        const float* blue_noise, const float* depth, const int* pixels, int n_pixels, int precision,
                        int threads, double* out_rgba, double* out_dist) {
    if (precision == 32)
        return cloud_render_t<float>(atmo, cp, m, tx, v, s, tlut, apl, apt, blue_noise, depth, pixels, n_pixels,
                                     threads, out_rgba, out_dist);
    return cloud_render_t<double>(atmo, cp, m, tx, v, s, tlut, apl, apt, blue_noise, depth, pixels, n_pixels,
                                  threads, out_rgba, out_dist);
}

}  // extern "C"

// ---- path tracer -----------------------------------------------------------

extern "C" {

// Grid values (FP64 or FP32) of the synthetic generator, x fastest.
int oracle_grid_generate(const skyr_grid_generator* g, int precision, int threads, double* out) {
    parallel_for(g->ny * g->nz, threads, [&](int row) {
        int y = row % g->ny, z = row / g->ny;
        for (int x = 0; x < g->nx; ++x)
            out[((size_t)z * g->ny + y) * g->nx + x] = precision == 32 ? (double)orc::grid_value<float>(*g, x, y, z)
                                                                        : orc::grid_value<double>(*g, x, y, z);
    });
    return 0;
}

// Brick majorants of a host half grid (same definition as skyr_grid_majorants).
int oracle_grid_majorants(const skyr_density_grid* gd, const uint16_t* data, float* out) {
    int bs = gd->brick;
    int bx = (gd->nx + bs - 1) / bs, by = (gd->ny + bs - 1) / bs, bz = (gd->nz + bs - 1) / bs;
    for (int k = 0; k < bz; ++k)
        for (int j = 0; j < by; ++j)
            for (int i = 0; i < bx; ++i) {
                float m = 0.f;
                for (int z = k * bs - 1; z <= (k + 1) * bs; ++z)
                    for (int y = j * bs - 1; y <= (j + 1) * bs; ++y)
                        for (int x = i * bs - 1; x <= (i + 1) * bs; ++x) {
                            if (x < 0 || y < 0 || z < 0 || x >= gd->nx || y >= gd->ny || z >= gd->nz) continue;
                            m = std::max(m, orc::half_to_float(data[((size_t)z * gd->ny + y) * gd->nx + x]));
                        }
                out[((size_t)k * by + j) * bx + i] = m * gd->density;
            }
    return 0;
}

}  // extern "C"

namespace {

// The path-tracer oracle and everything it references, built from the ABI
// structs (one heap object: the members refer to one another).
template <class T>
struct PtWorld {
    orc::AtmosphereOracle<T> O;
    orc::Image<T> tl, sl, st, al, at;
    orc::CloudOracle<T> C;
    orc::ViewLutOracle<T> V;
    orc::PathTracerOracle<T> PT;

    PtWorld(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp, const skyr_cloud_material* m,
            const skyr_cloud_textures* tx, const skyr_density_grid* gd, const skyr_pathtrace_parameters* pt,
            const skyr_cloud_view* v, const skyr_atmosphere_render_parameters* ev, const skyr_lut_sizes* s,
            const double* tlut_in, const double* svl_in, const double* svt_in, const double* apl_in,
            const double* apt_in)
        : O{orc::derive_atmosphere<T>(*atmo)},
          tl(image_from<T>(tlut_in, s->transmittance_width, s->transmittance_height)),
          sl(svl_in ? image_from<T>(svl_in, s->sky_view_width, s->sky_view_height) : orc::Image<T>{}),
          st(svt_in ? image_from<T>(svt_in, s->sky_view_width, s->sky_view_height) : orc::Image<T>{}),
          al(image_from<T>(apl_in, s->aerial_perspective_width, s->aerial_perspective_height,
                           s->aerial_perspective_depth)),
          at(image_from<T>(apt_in, s->aerial_perspective_width, s->aerial_perspective_height,
                           s->aerial_perspective_depth)),
          C{O, orc::derive_cloud_frame<T>(*atmo, *cp, *m, *tx, *v), {}, {}, {}, {}, nullptr, nullptr, nullptr, nullptr},
          V{O, orc::derive_render_frame<T>(*atmo, *ev)},
          PT{O, C, V, &sl, &st, *pt} {
        auto set = [](orc::Tex8& t, const void* p, const skyr_noise_texture_desc& d, bool border) {
            t.data = (const uint8_t*)p;
            t.w = d.width; t.h = d.height; t.d = d.depth; t.channels = d.channels;
            t.border = border;
            t.init();
        };
        if (tx->cloud_map) set(C.cloud_map, tx->cloud_map, tx->cloud_map_desc, false);
        if (tx->detail) set(C.detail, tx->detail, tx->detail_desc, false);
        if (tx->displacement) set(C.displacement, tx->displacement, tx->displacement_desc, false);
        if (tx->voxel) set(C.voxel, tx->voxel, tx->voxel_desc, true);
        C.tlut = &tl;
        C.ap_lum = &al;
        C.ap_trans = &at;
        // box: the flat AABB [-w, w]^2 x [bottom, top], clipped to the grid
        T hw = T(pt->region_box_half_width);
        PT.box_min = orc::V3<T>(-hw, -hw, C.F.bottom);
        PT.box_max = orc::V3<T>(hw, hw, C.F.top);
        if (gd && gd->data) {
            PT.grid = (const uint16_t*)gd->data;
            PT.nx = gd->nx; PT.ny = gd->ny; PT.nz = gd->nz;
            PT.origin = orc::V3<T>(T(gd->origin[0]), T(gd->origin[1]), T(gd->origin[2]));
            PT.voxel = T(gd->voxel_size);
            PT.density = T(gd->density);
            PT.maj = gd->majorant;
            PT.brick = gd->brick;
            PT.bx = (gd->nx + gd->brick - 1) / gd->brick;
            PT.by = (gd->ny + gd->brick - 1) / gd->brick;
            PT.bz = (gd->nz + gd->brick - 1) / gd->brick;
            orc::V3<T> gmax = PT.origin + orc::V3<T>(T(gd->nx), T(gd->ny), T(gd->nz)) * PT.voxel;
            for (int a = 0; a < 3; ++a) {
                PT.box_min[a] = std::max(PT.box_min[a], PT.origin[a]);
                PT.box_max[a] = std::min(PT.box_max[a], gmax[a]);
            }
        }
        // kModelMatrix3: columns front, right, up of VolumetricCloud::Update (VolumetricCloud.cpp:188-200)
        T R = T(atmo->bottom_radius);
        orc::V3<T> center(T(0), -R, T(0));
        orc::V3<T> up = orc::normalize(orc::v3f<T>(v->camera_position) - center);
        orc::V3<T> front = orc::normalize(orc::cross(up, orc::V3<T>(T(1), T(0), T(0))));
        orc::V3<T> right = orc::normalize(orc::cross(up, front));
        for (int i = 0; i < 16; ++i) PT.model3.m[i] = T(0);
        for (int r = 0; r < 3; ++r) {
            PT.model3(r, 0) = front[r];
            PT.model3(r, 1) = right[r];
            PT.model3(r, 2) = up[r];
        }
        PT.model3(3, 3) = T(1);
    }
};

template <class T>
int pathtrace_t(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                const skyr_cloud_material* m, const skyr_cloud_textures* tx, const skyr_density_grid* gd,
                const skyr_pathtrace_parameters* pt, const skyr_cloud_view* v,
                const skyr_atmosphere_render_parameters* ev, const skyr_lut_sizes* s, const double* tlut_in,
                const double* svl_in, const double* svt_in, const double* apl_in, const double* apt_in,
                unsigned frame_begin, int n_frames, const int* pixels, int n_pixels, int threads, double* sum,
                double* sumsq) {
    auto W = std::make_unique<PtWorld<T>>(atmo, cp, m, tx, gd, pt, v, ev, s, tlut_in, svl_in, svt_in, apl_in,
                                          apt_in);
    const orc::PathTracerOracle<T>& PT = W->PT;
    parallel_for(n_pixels, threads, [&](int i) {
        int p = pixels ? pixels[i] : i;
        int px = p % v->width, py = p / v->width;
        double a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0};
        for (int f = 0; f < n_frames; ++f) {
            T o[4];
            PT.Pixel(px, py, v->width, v->height, frame_begin + (unsigned)f, o);
            for (int k = 0; k < 4; ++k) {
                a[k] += double(o[k]);
                b[k] += double(o[k]) * double(o[k]);
            }
        }
        for (int k = 0; k < 4; ++k) {
            sum[(size_t)i * 4 + k] = a[k];
            sumsq[(size_t)i * 4 + k] = b[k];
        }
    });
    return 0;
}

}  // namespace

extern "C" {

int oracle_pathtrace(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                     const skyr_cloud_material* m, const skyr_cloud_textures* tx, const skyr_density_grid* gd,
                     const skyr_pathtrace_parameters* pt, const skyr_cloud_view* v,
                     const skyr_atmosphere_render_parameters* ev, const skyr_lut_sizes* s, const double* tlut,
                     const double* svl, const double* svt, const double* apl, const double* apt,
                     unsigned frame_begin, int n_frames, const int* pixels, int n_pixels, int precision,
                     int threads, double* sum, double* sumsq) {
    if (precision == 32)
        return pathtrace_t<float>(atmo, cp, m, tx, gd, pt, v, ev, s, tlut, svl, svt, apl, apt, frame_begin, n_frames,
                                  pixels, n_pixels, threads, sum, sumsq);
    return pathtrace_t<double>(atmo, cp, m, tx, gd, pt, v, ev, s, tlut, svl, svt, apl, apt, frame_begin, n_frames,
                               pixels, n_pixels, threads, sum, sumsq);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// surrogate network (oracle_mlp.hpp)
// ---------------------------------------------------------------------------
#include "oracle_mlp.hpp"

extern "C" {

// y[n][3] = MLP(x[n][103]) in FP64 (BF16 rounding points mirrored when `mirror`)
int oracle_mlp_predict(const float* params, const float* x, int n, int mirror, int threads, double* y) {
    orc::MlpOracle net(params, mirror != 0);
    parallel_for(n, threads, [&](int s) {
        double xd[orc::kMlpIn];
        for (int i = 0; i < orc::kMlpIn; ++i) xd[i] = x[(size_t)s * orc::kMlpIn + i];
        net.predict(xd, y + (size_t)s * orc::kMlpOut);
    });
    return 0;
}

// gradient of the mean relative-L2 loss (grad[19331] overwritten); returns the loss
double oracle_mlp_gradient(const float* params, const float* x, const float* t, int n, double label_scale,
                           double loss_eps, int mirror, double* grad) {
    orc::MlpOracle net(params, mirror != 0);
    std::vector<double> xd((size_t)n * orc::kMlpIn), td((size_t)n * orc::kMlpOut);
    for (size_t i = 0; i < xd.size(); ++i) xd[i] = x[i];
    for (size_t i = 0; i < td.size(); ++i) td[i] = t[i];
    std::fill(grad, grad + orc::kMlpParams, 0.0);
    return net.gradient(xd.data(), td.data(), n, label_scale, loss_eps, grad);
}

void oracle_mlp_adam(double* p, double* m, double* v, const double* g, int n, double lr, double b1, double b2,
                     double eps, int step) {
    orc::adam_step(p, m, v, g, n, lr, b1, b2, eps, step);
}

int oracle_mlp_param_count(void) { return orc::kMlpParams; }

}  // extern "C"


// ---------------------------------------------------------------------------
// surrogate: grid lookups, point-source paths, the surrogate raymarch
// ---------------------------------------------------------------------------
namespace {

skyr_cloud_material minimal_material() {
    skyr_cloud_material m{};
    m.type = SKYR_MATERIAL_MINIMAL;
    m.density = 1.f;
    return m;
}

inline uint32_t pcg(uint32_t v) { return orc::PCGHash(v); }

inline float bf16_of(double x) { return orc::bf16_round((float)x); }

}  // namespace

extern "C" {

// trilinear extinction of the grid at points[n][3]
int oracle_grid_sigma(const skyr_density_grid* gd, const double* points, int n, double* out) {
    orc::V3<double> o(gd->origin[0], gd->origin[1], gd->origin[2]);
    for (int i = 0; i < n; ++i) {
        orc::V3<double> p(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
        out[i] = orc::grid_trilinear<double>((const uint16_t*)gd->data, gd->nx, gd->ny, gd->nz, o,
                                             (double)gd->voxel_size, (double)gd->density, p);
    }
    return 0;
}

// sum over paths k in [0, n_paths) of the point-source radiance of points[n][6]
int oracle_point_radiance(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                          const skyr_density_grid* gd, const skyr_pathtrace_parameters* pt, const skyr_cloud_view* v,
                          const skyr_atmosphere_render_parameters* ev, const skyr_lut_sizes* s, const double* tlut,
                          const double* svl, const double* svt, const double* apl, const double* apt,
                          unsigned frame_begin, int n_paths, const double* points, int n, int threads, double* sum,
                          double* sumsq) {
    skyr_cloud_material m = minimal_material();
    skyr_cloud_textures tx{};
    auto W = std::make_unique<PtWorld<double>>(atmo, cp, &m, &tx, gd, pt, v, ev, s, tlut, svl, svt, apl, apt);
    parallel_for(n, threads, [&](int i) {
        const double* q = points + 6 * (size_t)i;
        orc::V3<double> p(q[0], q[1], q[2]), w(q[3], q[4], q[5]);
        double a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
        for (int k = 0; k < n_paths; ++k) {
            orc::V3<double> L = W->PT.PointPath((uint32_t)i, frame_begin + (unsigned)k, p, w);
            for (int c = 0; c < 3; ++c) {
                a[c] += L[c];
                b[c] += L[c] * L[c];
            }
        }
        for (int c = 0; c < 3; ++c) {
            sum[3 * (size_t)i + c] = a[c];
            sumsq[3 * (size_t)i + c] = b[c];
        }
    });
    return 0;
}

// The surrogate raymarch of skyr_surrogate_render for listed pixels, in FP64
// over the GPU-built feature lattice `lattice_raw` (node records bf16
// [nodes][80], sun optical depth f32 [nodes], then the grid's FP16 mip levels
// 1..6, each 256-byte aligned); the network is oracle_mlp.hpp with the BF16
// rounding points mirrored.  The far-side feature (43) of sample k is the
// transmittance of what remains of the ray's optical depth at the march's
// samples past it: exp(-(sum_j>k sigma_j dt + sigma_k dt / 2)); features
// 79..102 are the view-oriented stencil over mip levels 3..6.  out[n][4] = (luminance rgb, transmittance),
// err[n] = the error estimate with a single relative error `rel_err`.
int oracle_surrogate_render(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                            const skyr_density_grid* gd, const skyr_pathtrace_parameters* pt,
                            const skyr_cloud_view* v, const skyr_lut_sizes* s, const double* tlut,
                            const double* apl, const double* apt, const uint8_t* lattice_raw,
                            const skyr_feature_volume* fv, const float* params,
                            double out_scale, int steps, int use_network, double min_t, double rel_err,
                            const int* pixels, int n, int threads, double* out, double* err) {
    skyr_cloud_material m = minimal_material();
    skyr_cloud_textures tx{};
    skyr_atmosphere_render_parameters ev{};
    ev.sun_direction_theta = v->sun_direction_theta;
    ev.sun_direction_phi = v->sun_direction_phi;
    std::memcpy(ev.camera_position, v->camera_position, sizeof(ev.camera_position));
    std::memcpy(ev.view_projection, v->view_projection, sizeof(ev.view_projection));
    ev.sky_view_lut_steps = 1;
    ev.aerial_perspective_lut_steps = 1;
    ev.aerial_perspective_lut_max_distance = v->aerial_perspective_lut_max_distance;
    auto W = std::make_unique<PtWorld<double>>(atmo, cp, &m, &tx, gd, pt, v, &ev, s, tlut, nullptr, nullptr, apl, apt);
    const orc::PathTracerOracle<double>& PT = W->PT;
    const auto& F = W->C.F;
    orc::MlpOracle net(params, true);
    const double cell = (double)gd->voxel_size * fv->stride;
    const orc::V3<double> og(gd->origin[0], gd->origin[1], gd->origin[2]);
    const orc::V3<double> sun(fv->sun[0], fv->sun[1], fv->sun[2]);
    constexpr int kLat = 80, kIn = orc::kMlpIn;
    const size_t nodes = (size_t)fv->nx * fv->ny * fv->nz;
    const uint16_t* lattice_rec = reinterpret_cast<const uint16_t*>(lattice_raw);
    const float* lattice_tau = reinterpret_cast<const float*>(lattice_raw + nodes * kLat * 2);
    struct Mip {
        const uint16_t* d;
        int nx, ny, nz;
        double voxel;
    };
    Mip mip[7];
    {
        size_t off = nodes * (kLat * 2 + 4);
        int nx = gd->nx, ny = gd->ny, nz = gd->nz;
        for (int l = 1; l <= 6; ++l) {
            off = (off + 255) & ~(size_t)255;
            nx = (nx + 1) / 2, ny = (ny + 1) / 2, nz = (nz + 1) / 2;
            mip[l] = Mip{reinterpret_cast<const uint16_t*>(lattice_raw + off), nx, ny, nz,
                         (double)gd->voxel_size * (1 << l)};
            off += (size_t)nx * ny * nz * 2;
        }
    }
    // trilinear between texel centres, zero border
    auto mip_value = [&](int l, orc::V3<double> p) {
        const Mip& M = mip[l];
        double g[3];
        for (int a = 0; a < 3; ++a) g[a] = (p[a] - gd->origin[a]) / M.voxel - 0.5;
        int i0[3];
        double fr[3];
        for (int a = 0; a < 3; ++a) {
            i0[a] = (int)std::floor(g[a]);
            fr[a] = g[a] - i0[a];
        }
        double v = 0.0;
        for (int c = 0; c < 8; ++c) {
            int x = i0[0] + (c & 1), y = i0[1] + ((c >> 1) & 1), z = i0[2] + (c >> 2);
            if (x < 0 || y < 0 || z < 0 || x >= M.nx || y >= M.ny || z >= M.nz) continue;
            double w = ((c & 1) ? fr[0] : 1 - fr[0]) * (((c >> 1) & 1) ? fr[1] : 1 - fr[1]) *
                       ((c >> 2) ? fr[2] : 1 - fr[2]);
            v += w * orc::half_to_float(M.d[((size_t)z * M.ny + y) * M.nx + x]);
        }
        return v;
    };
    auto lattice = [&](orc::V3<double> x, double f[kIn], double& tau) {
        orc::V3<double> g = (x - og) / cell;
        int i0[3];
        double fr[3];
        int nn[3] = {fv->nx, fv->ny, fv->nz};
        for (int a = 0; a < 3; ++a) {
            i0[a] = std::min(std::max((int)std::floor(g[a]), 0), nn[a] - 2);
            fr[a] = std::min(std::max(g[a] - i0[a], 0.0), 1.0);
        }
        for (int k = 0; k < kIn; ++k) f[k] = 0.0;
        tau = 0.0;
        for (int c = 0; c < 8; ++c) {
            int d[3] = {c & 1, (c >> 1) & 1, c >> 2};
            double w = 1.0;
            for (int a = 0; a < 3; ++a) w *= d[a] ? fr[a] : 1.0 - fr[a];
            size_t node = ((size_t)(i0[2] + d[2]) * fv->ny + (i0[1] + d[1])) * fv->nx + (i0[0] + d[0]);
            tau += w * lattice_tau[node];
            for (int k = 0; k < kLat; ++k) f[k] += w * orc::bf16_to_float(lattice_rec[node * kLat + k]);
        }
    };
    // features 33..40: the view-oriented cube corners (skyr_surrogate.h)
    const double span = (double)gd->voxel_size * std::max(gd->nx, std::max(gd->ny, gd->nz));
    const double nbr = 0.1 * span / std::sqrt(3.0), inv_ref = 1.0 / fv->sigma_ref;
    auto view_neighbours = [&](orc::V3<double> x, orc::V3<double> v, double f[kIn]) {
        orc::V3<double> u = sun - v * orc::dot(v, sun);
        double l2 = orc::dot(u, u);
        if (l2 < 1e-8) {
            orc::V3<double> b1;
            orc::PathTracerOracle<double>::basis(v, u, b1);
        } else {
            u = u / std::sqrt(l2);
        }
        orc::V3<double> w = orc::cross(v, u);
        for (int j = 0; j < 8; ++j) {
            orc::V3<double> o = v * ((j & 1) ? nbr : -nbr) + u * ((j & 2) ? nbr : -nbr) + w * ((j & 4) ? nbr : -nbr);
            f[33 + j] = PT.grid_sigma(x + o) * inv_ref;
        }
        // 79..102: +-2^(l+1) voxels along v, u, w at mip levels l = 3..6
        const orc::V3<double> axes[3] = {v, u, w};
        for (int s = 0; s < 24; ++s) {
            int l = 3 + s / 6, j = s % 6;
            double h = (double)gd->voxel_size * (2 << l) * ((j & 1) ? -1.0 : 1.0);
            f[79 + s] = mip_value(l, x + axes[j >> 1] * h) * gd->density * inv_ref;
        }
    };
    const double gb = pt->back_phase_g, gf = pt->forward_phase_g, ratio = pt->forward_scattering_ratio;
    auto hg = [](double c, double g) { return (0.25 / orc::kPi) * (1 - g * g) / std::pow(1 + g * g - 2 * g * c, 1.5); };
    parallel_for(n, threads, [&](int i) {
        int pix = pixels[i];
        int px = pix % v->width, py = pix / v->width;
        double u = (px + 0.5) / v->width, vv = (py + 0.5) / v->height;
        orc::V3<double> frag = orc::projective_mul(F.inv_mvp, orc::V3<double>(u * 2 - 1, vv * 2 - 1, 1.0));
        orc::V3<double> dir = orc::normalize(frag - F.cam);
        double t0, t1;
        PT.region(F.cam, dir, t0, t1);
        double T = 1, errs = 0, wsum = 0, wt = 0;
        orc::V3<double> L(0.0);
        if (t0 < t1) {
            double dt = (t1 - t0) / steps;
            uint32_t js = pcg((uint32_t)(py * v->width + px) * 747796405u + 2891336453u);
            double jitter = (double)(js >> 8) / 16777216.0;
            double mu = orc::dot(dir, sun);
            double ph = hg(mu, gb) * (1 - ratio) + hg(mu, gf) * ratio;
            double tau_total = 0, run = 0;
            for (int k = 0; k < steps; ++k) tau_total += PT.grid_sigma(F.cam + dir * (t0 + (k + jitter) * dt)) * dt;
            for (int k = 0; k < steps && T > min_t; ++k) {
                double t = t0 + (k + jitter) * dt;
                orc::V3<double> x = F.cam + dir * t;
                double sigma = PT.grid_sigma(x);
                run += sigma * dt;
                if (!(sigma > 0)) continue;
                double f[kIn], tau;
                lattice(x, f, tau);
                view_neighbours(x, dir, f);
                f[42] = mu;
                f[43] = std::exp(-std::max(tau_total - run + 0.5 * sigma * dt, 0.0));
                orc::V3<double> ms(0.0);
                if (use_network) {
                    double rec[kIn], y[3];
                    for (int q = 0; q < kIn; ++q) rec[q] = bf16_of(f[q]);
                    net.predict(rec, y);
                    for (int c = 0; c < 3; ++c) ms[c] = std::max(y[c] * (double)(float)out_scale, 0.0);
                }
                orc::V3<double> ss = PT.sun_illuminance(x) * (ph * std::exp(-tau));
                double dT = std::exp(-sigma * dt), w = T * (1 - dT);
                L = L + (ss + ms) * w;
                errs += w * (ms[0] + ms[1] + ms[2]) / 3.0 * rel_err;
                wsum += w;
                wt += w * t;
                T *= dT;
            }
        }
        if (wsum > 0) {
            double ta = wt / wsum;
            double r = F.cam.z + F.R, mu = dir.z;
            if (r > W->O.A.top_radius) {
                double disc = r * r * (mu * mu - 1) + W->O.A.top_radius * W->O.A.top_radius;
                if (mu < 0 && disc >= 0) ta -= std::max(-r * mu - std::sqrt(std::max(disc, 0.0)), 0.0);
                else ta = 0;
            }
            double wz = std::sqrt(std::max(ta, 0.0) / F.ap_max_distance);
            const orc::Image<double>& al = *W->C.ap_lum;
            double uu = 0.5 / al.w + u * (1 - 1.0 / al.w), vq = 0.5 / al.h + vv * (1 - 1.0 / al.h),
                   ww = 0.5 / al.d + wz * (1 - 1.0 / al.d);
            orc::V3<double> at = orc::sample_linear_clamp3(*W->C.ap_trans, uu, vq, ww);
            orc::V3<double> alum = orc::sample_linear_clamp3(al, uu, vq, ww);
            alum = alum * W->C.RayScatterVisibility(u, vv, wt / wsum);
            L = L * at + alum * (1 - T);
        }
        for (int c = 0; c < 3; ++c) out[4 * (size_t)i + c] = L[c];
        out[4 * (size_t)i + 3] = T;
        err[i] = errs;
    });
    return 0;
}

}  // extern "C"

// ---- cloud shadow passes ----------------------------------------------------
namespace {

// A light frame as 4 x 16 doubles: light_vp, inv_light_vp, model, reproject.
orc::LightFrameD frame_from(const double* f, int has_previous) {
    orc::LightFrameD L;
    for (int i = 0; i < 16; ++i) {
        L.light_vp.m[i] = f[i];
        L.inv_light_vp.m[i] = f[16 + i];
        L.model.m[i] = f[32 + i];
        L.reproject.m[i] = f[48 + i];
    }
    L.has_previous = has_previous != 0;
    return L;
}

void frame_to(const orc::LightFrameD& L, double* f) {
    for (int i = 0; i < 16; ++i) {
        f[i] = L.light_vp.m[i];
        f[16 + i] = L.inv_light_vp.m[i];
        f[32 + i] = L.model.m[i];
        f[48 + i] = L.reproject.m[i];
    }
}

// The cloud oracle of a view with its material textures bound (no LUTs).
std::unique_ptr<orc::CloudOracle<double>> cloud_oracle(const orc::AtmosphereOracle<double>& O,
                                                       const skyr_atmosphere_parameters* atmo,
                                                       const skyr_cloud_parameters* cp,
                                                       const skyr_cloud_material* m, const skyr_cloud_textures* tx,
                                                       const skyr_cloud_view* v) {
    auto C = std::unique_ptr<orc::CloudOracle<double>>(new orc::CloudOracle<double>{
        O, orc::derive_cloud_frame<double>(*atmo, *cp, *m, *tx, *v), {}, {}, {}, {}, nullptr, nullptr, nullptr,
        nullptr});
    auto set = [](orc::Tex8& t, const void* p, const skyr_noise_texture_desc& d, bool border) {
        t.data = (const uint8_t*)p;
        t.w = d.width; t.h = d.height; t.d = d.depth; t.channels = d.channels;
        t.border = border;
        t.init();
    };
    set(C->cloud_map, tx->cloud_map, tx->cloud_map_desc, false);
    set(C->detail, tx->detail, tx->detail_desc, false);
    set(C->displacement, tx->displacement, tx->displacement_desc, false);
    set(C->voxel, tx->voxel, tx->voxel_desc, true);
    return C;
}

}  // namespace

extern "C" {

// VolumetricCloud::Update's light transform; previous may be NULL.
int oracle_cloud_light_frame(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                             const skyr_cloud_view* v, int map_w, int map_h, const double* previous,
                             const float* wind, double* out) {
    orc::LightFrameD prev;
    if (previous) prev = frame_from(previous, 0);
    orc::LightFrameD L = orc::derive_light_frame(*atmo, *cp, *v, map_w, map_h, previous ? &prev : nullptr, wind);
    frame_to(L, out);
    return L.has_previous ? 1 : 0;
}

// Shadow-map texels (texels[i] = y * map_w + x, or all when texels == NULL);
// out[2 i + {0, 1}] = (depth, transmittance).
int oracle_cloud_shadow_map(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                            const skyr_cloud_material* m, const skyr_cloud_textures* tx, const skyr_cloud_view* v,
                            int map_w, int map_h, const double* frame, int has_previous, const float* blue_noise,
                            const double* previous_map, const int* texels, int n, int threads, double* out) {
    orc::AtmosphereOracle<double> O{orc::derive_atmosphere<double>(*atmo)};
    auto C = cloud_oracle(O, atmo, cp, m, tx, v);
    orc::ShadowMapOracle S{*C, frame_from(frame, has_previous), map_w, map_h, blue_noise, previous_map};
    parallel_for(n, threads, [&](int i) {
        int p = texels ? texels[i] : i;
        S.Texel(p % map_w, p / map_w, out + 2 * (size_t)i);
    });
    return 0;
}

int oracle_cloud_shadow_blur(int w, int h, const double* in, double* out) {
    orc::shadow_blur(w, h, in, out);
    return 0;
}

// The shadow froxel of a view from a blurred map: out (R16) and, when not
// NULL, exact (the running means before the store); [depth][height][width].
int oracle_cloud_shadow_froxel(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                               const skyr_cloud_material* m, const skyr_cloud_textures* tx, const skyr_cloud_view* v,
                               int map_w, int map_h, int fw, int fh, int fd, const double* frame, const double* map,
                               int threads, uint16_t* out, double* exact) {
    orc::CloudFrame<double> F = orc::derive_cloud_frame<double>(*atmo, *cp, *m, *tx, *v);
    orc::LightFrameD L = frame_from(frame, 0);
    const size_t slice = (size_t)fw * fh;
    parallel_for(fw * fh, threads, [&](int i) {
        std::vector<double> col(fd);
        orc::froxel_column(F, L, map, map_w, map_h, fw, fh, fd, cp->shadow_froxel_max_distance, i % fw, i / fw,
                           col.data());
        for (int z = 0; z < fd; ++z) {
            out[z * slice + i] = orc::unorm16(col[z]);
            if (exact) exact[z * slice + i] = col[z];
        }
    });
    return 0;
}

}  // extern "C"

// ---- quarter-resolution cloud pass ------------------------------------------
extern "C" {

// CheckerboardGen.comp: out (w/2) x (h/2); depth NULL = 1
int oracle_cloud_checkerboard(const float* depth, int w, int h, double* out) {
    orc::checkerboard(depth, orc::quarter_dims(w, h), out);
    return 0;
}

// VolumetricCloudIndexGen.comp from a checkerboard depth: out[2] per quarter texel
int oracle_cloud_index(const double* cb, int w, int h, float z_near, float z_far, int base, double* out) {
    orc::index_gen(cb, orc::quarter_dims(w, h), orc::LinearDepth(z_near, z_far), base, out);
    return 0;
}

// The raymarch of quarter texels (pixels[i] = y * qw + x, or all) of the
// viewport `v` (width / height = the viewport) at the checkerboard texels the
// index selects.
int oracle_cloud_render_quarter(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                                const skyr_cloud_material* m, const skyr_cloud_textures* tx, const skyr_cloud_view* v,
                                const skyr_lut_sizes* s, const double* tlut_in, const double* apl_in,
                                const double* apt_in, const float* blue_noise, const double* index, const double* cb,
                                const int* pixels, int n, int threads, double* out_rgba, double* out_dist) {
    orc::AtmosphereOracle<double> O{orc::derive_atmosphere<double>(*atmo)};
    orc::Image<double> tl = image_from<double>(tlut_in, s->transmittance_width, s->transmittance_height);
    int W = s->aerial_perspective_width, H = s->aerial_perspective_height, D = s->aerial_perspective_depth;
    orc::Image<double> al = image_from<double>(apl_in, W, H, D), at = image_from<double>(apt_in, W, H, D);
    auto C = cloud_oracle(O, atmo, cp, m, tx, v);
    C->tlut = &tl;
    C->ap_lum = &al;
    C->ap_trans = &at;
    C->blue_noise = blue_noise;
    orc::QuarterDims Q = orc::quarter_dims(v->width, v->height);
    parallel_for(n, threads, [&](int i) {
        int p = pixels ? pixels[i] : i;
        int x = p % Q.qw, y = p / Q.qw;
        int dx, dy;
        orc::index_offset(unsigned(int(index[2 * (size_t)p])) & 3u, dx, dy);
        int cx = 2 * x + dx, cy = 2 * y + dy;
        double rgba[4], dist;
        C->PixelAt((cx + 0.5) / Q.hw, (cy + 0.5) / Q.hh, float(cb[(size_t)cy * Q.hw + cx]), x, y, rgba, dist);
        for (int k = 0; k < 4; ++k) out_rgba[4 * (size_t)i + k] = rgba[k];
        if (out_dist) out_dist[i] = dist;
    });
    return 0;
}

// VolumetricCloudReconstruct.comp over the half-resolution image (out[4] per texel)
int oracle_cloud_reconstruct(const skyr_atmosphere_parameters* atmo, const skyr_cloud_parameters* cp,
                             const skyr_cloud_material* m, const skyr_cloud_textures* tx, const skyr_cloud_view* v,
                             const float* reproject, float z_near, float z_far, int history, const double* cb,
                             const double* index, const double* render, const double* rdist, const double* previous,
                             int threads, double* out) {
    orc::CloudFrame<double> F = orc::derive_cloud_frame<double>(*atmo, *cp, *m, *tx, *v);
    orc::QuarterDims Q = orc::quarter_dims(v->width, v->height);
    orc::LinearDepth LD(z_near, z_far);
    orc::M4<double> rp = orc::mat_from_floats<double>(reproject);
    parallel_for(Q.hw * Q.hh, threads, [&](int i) {
        orc::reconstruct_texel(F, Q, LD, rp, history != 0 && previous != nullptr, cb, index, render, rdist, previous,
                               i % Q.hw, i / Q.hw, out + 4 * (size_t)i);
    });
    return 0;
}

// VolumetricCloudUpscale.comp over the viewport (hdr_in / out 4 per pixel; depth NULL = 1)
int oracle_cloud_upscale(int w, int h, const float* depth, float z_near, float z_far, const double* cb,
                         const double* rec, const double* hdr_in, int threads, double* out) {
    orc::QuarterDims Q = orc::quarter_dims(w, h);
    orc::LinearDepth LD(z_near, z_far);
    parallel_for(h, threads, [&](int y) {
        for (int x = 0; x < w; ++x) orc::upscale_pixel(Q, LD, depth, cb, rec, hdr_in, x, y, out + 4 * ((size_t)y * w + x));
    });
    return 0;
}

}  // extern "C"

// ---- environment cube --------------------------------------------------------
extern "C" {

// Level 0 of a size^2 x 6 environment cube (out[4] per texel, a = 0), layout
// as skyr_environment_cube.
int oracle_environment_cube(const skyr_atmosphere_parameters* p, const skyr_atmosphere_render_parameters* r,
                            const skyr_lut_sizes* s, const double* t_in, const double* svl_in, const double* svt_in,
                            int size, int threads, double* out) {
    orc::AtmosphereOracle<double> O{orc::derive_atmosphere<double>(*p)};
    orc::RenderFrame<double> F = orc::derive_render_frame<double>(*p, *r);
    orc::Image<double> tl = image_from<double>(t_in, s->transmittance_width, s->transmittance_height);
    orc::Image<double> svl = image_from<double>(svl_in, s->sky_view_width, s->sky_view_height);
    orc::Image<double> svt = image_from<double>(svt_in, s->sky_view_width, s->sky_view_height);
    parallel_for(6 * size, threads, [&](int row) {
        int face = row / size, y = row % size;
        for (int x = 0; x < size; ++x) {
            orc::V3<double> c = orc::environment_cube_texel(O, F, tl, svl, svt, size, face, x, y);
            double* o = out + 4 * (((size_t)face * size + y) * size + x);
            o[0] = c.x;
            o[1] = c.y;
            o[2] = c.z;
            o[3] = 0.0;
        }
    });
    return 0;
}

}  // extern "C"

extern "C" {

// EnvRadianceSH.comp on a cube (4 doubles per texel, `levels` levels): out[9][3]
int oracle_environment_sh(const double* cube, int size, int levels, double* out) {
    orc::CubeImage C{cube, size, levels};
    double r[9][3];
    orc::environment_sh(C, r);
    for (int k = 0; k < 9; ++k)
        for (int c = 0; c < 3; ++c) out[3 * k + c] = r[k][c];
    return 0;
}

// PrefilterRadiance.comp, one level of side n and roughness r: out[6][n][n][3]
int oracle_environment_prefilter(const double* cube, int size, int levels, int n, double roughness, int threads,
                                 double* out) {
    orc::CubeImage C{cube, size, levels};
    parallel_for(6 * n, threads, [&](int row) {
        int face = row / n, y = row % n;
        for (int x = 0; x < n; ++x) {
            orc::V3<double> c = orc::prefilter_texel(C, n, roughness, face, x, y);
            double* o = out + 3 * (((size_t)face * n + y) * n + x);
            o[0] = c.x;
            o[1] = c.y;
            o[2] = c.z;
        }
    });
    return 0;
}

}  // extern "C"

extern "C" {

// The seamless copy of a cube (4 doubles per texel in and out), layout as skyr_environment_seamless.
int oracle_environment_seamless(const double* cube, int size, int levels, double* out) {
    orc::CubeImage C{cube, size, levels};
    size_t k = 0;
    for (int l = 0; l < levels; ++l) {
        int n = C.side(l);
        for (int face = 0; face < 6; ++face)
            for (int j = -1; j <= n; ++j)
                for (int i = -1; i <= n; ++i, ++k) orc::cube_texel(C, l, face, i, j, out + 4 * k);
    }
    return 0;
}

}  // extern "C"

// ---- full-screen composite ----------------------------------------------------
extern "C" {

// The composite of the listed pixels (y * width + x, or all); `in` holds host
// pointers; LUTs as double RGBA images; out[4] per pixel.
int oracle_atmosphere_composite(const skyr_atmosphere_parameters* p, const skyr_atmosphere_render_parameters* r,
                                const skyr_composite_parameters* cp, const skyr_lut_sizes* s, const double* t_in,
                                const double* ms_in, const double* svl_in, const double* svt_in, const double* apl_in,
                                const double* apt_in, const skyr_composite_inputs* in, const int* pixels, int n,
                                int threads, double* out) {
    orc::AtmosphereOracle<double> O{orc::derive_atmosphere<double>(*p)};
    orc::ViewLutOracle<double> VL{O, orc::derive_render_frame<double>(*p, *r)};
    orc::Image<double> tl = image_from<double>(t_in, s->transmittance_width, s->transmittance_height);
    orc::Image<double> ms = image_from<double>(ms_in, s->multiscattering_width, s->multiscattering_height);
    orc::Image<double> svl, svt, apl, apt;
    if (svl_in) svl = image_from<double>(svl_in, s->sky_view_width, s->sky_view_height);
    if (svt_in) svt = image_from<double>(svt_in, s->sky_view_width, s->sky_view_height);
    int aw = s->aerial_perspective_width, ah = s->aerial_perspective_height, ad = s->aerial_perspective_depth;
    if (apl_in) apl = image_from<double>(apl_in, aw, ah, ad);
    if (apt_in) apt = image_from<double>(apt_in, aw, ah, ad);
    orc::CompositeOracle C{O, VL, tl, ms, svl, svt, apl, apt, *cp, *in};
    parallel_for(n, threads, [&](int i) {
        int q = pixels ? pixels[i] : i;
        C.Pixel(q % in->width, q / in->width, out + 4 * (size_t)i);
    });
    return 0;
}

}  // extern "C"
