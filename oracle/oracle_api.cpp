// oracle_api.cpp — TEST INFRASTRUCTURE ONLY: extern "C" surface of the CPU
// oracle (precision 64) and of the like-for-like CPU baseline (precision 32),
// loaded by tests/ and bench.py through ctypes.  Parity status: unpinned
// (see oracle_math.hpp).
#include <atomic>
#include <cstring>
#include <thread>

#include "oracle_atmosphere.hpp"

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
