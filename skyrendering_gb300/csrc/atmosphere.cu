// atmosphere.cu — transmittance, multi-scattering, sky-view and
// aerial-perspective LUT kernels for sm_103a.
//
// Semantics follow shaders/SkyRendering/Atmosphere.glsl and
// shaders/SkyRendering/AtmosphereRenderer.glsl of c52e/SkyRendering; the
// arithmetic is reorganised for the GPU:
//  * every radius difference (r^2 - R^2, top - r) is carried from an exact
//    source instead of being formed by cancellation in FP32;
//  * the samples of one ray are split over a group of LANES lanes, each lane
//    integrating a contiguous chunk, and the chunks are composed with the
//    associative rule (L_a, T_a) o (L_b, T_b) = (L_a + T_a L_b, T_a T_b)
//    through warp shuffles;
//  * the multi-scattering texel is one 256-thread block (64 sphere directions
//    x 4 chunks), reduced with shuffles and one shared-memory pass;
//  * the passes after the first are programmatic dependent launches, so each
//    one's blocks are scheduled while the previous one drains; the view pass
//    lets its own dependents (the raymarch of skyr_render_frame) start at once.
#include <utility>

#include "skyr_internal.cuh"
#include "atmosphere_kernels.cuh"
#include "atmosphere_integrate.cuh"
#include "lut_access.cuh"

namespace skyr {

// Programmatic dependent launch: the multi-scattering and view passes are
// launched with programmatic stream serialisation, so their blocks can be
// scheduled while the previous pass drains.  A dependent pass waits here,
// before its first LUT read, until the previous pass has completed and its
// writes are visible (a no-op for a launch without the attribute); a pass lets
// its dependents be scheduled once its own main work is under way.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// ---------------------------------------------------------------------------
// TRANSMITTANCE (Atmosphere.glsl:309-337): LANES lanes per texel.
// ---------------------------------------------------------------------------
template <int LANES, bool TABLE>
__global__ void __launch_bounds__(128) transmittance_kernel(JobSrc<TABLE> jobs, int n_sets, int w, int h,
                                                            float4* __restrict__ out) {
    pdl_launch_dependents();  // the pass is a single wave: every block is already resident
    int gid = blockIdx.x * blockDim.x + threadIdx.x;
    int lane = gid % LANES;
    int texel = gid / LANES;
    int per_set = w * h;
    int set = texel / per_set;
    bool valid = set < n_sets;
    if (!valid) set = n_sets - 1;  // keep the warp converged for the shuffles
    int t = texel % per_set;
    const AtmoConsts& A = jobs.get(set).a;
    int ix = t % w, iy = t / w;
    // GetRMuFromTransmittanceTextureIndex (Atmosphere.glsl:71-88), with
    // rho^2 = r^2 - R^2 and 2 r mu = (H^2 - rho^2 - d^2) / d kept exact.
    float x_mu = (float)ix / (float)(w - 1);
    float x_r = (float)iy / (float)(h - 1);
    float rho = A.Hh * x_r;
    float rho2 = rho * rho;
    float r = sqrtf(rho2 + A.R2);
    float alt = rho2 / (r + A.R);
    float d_min = A.thickness - alt;
    float d_max = rho + A.Hh;
    float d = d_min + x_mu * (d_max - d_min);
    float b = d == 0.f ? 2.f * r : (A.top2_minus_R2 - rho2 - d * d) / d;  // 2 r mu
    b = fminf(fmaxf(b, -2.f * r), 2.f * r);                               // ClampCosine
    float mu = b / (2.f * r);
    float dist = dist_to_top(r, d_min, A.top, mu);
    float steps = A.transmittance_steps;
    float dx = dist / steps;
    int n = sample_count(0.5f, steps);
    int k0 = (n * lane) / LANES, k1 = (n * (lane + 1)) / LANES;
    // optical length, Kahan-compensated per channel
    float3 sum = f3(0.f), comp = f3(0.f);
    for (int k = k0; k < k1; ++k) {
        float di = ((float)k + 0.5f) * dx;
        float s = fmaf(di, b + di, rho2);
        float r_i = sqrtf(A.R2 + s);
        float h_i = s / (r_i + A.R);
        float3 ray_s, mie_s, ext;
        medium(A, h_i, ray_s, mie_s, ext);
        float3 y = ext * dx - comp;
        float3 tt = sum + y;
        comp = (tt - sum) - y;
        sum = tt;
    }
#pragma unroll
    for (int o = 1; o < LANES; o <<= 1) {
        sum.x += __shfl_down_sync(0xffffffffu, sum.x, o);
        sum.y += __shfl_down_sync(0xffffffffu, sum.y, o);
        sum.z += __shfl_down_sync(0xffffffffu, sum.z, o);
    }
    if (valid && lane == 0) {
        float3 T = f3(expf(-sum.x), expf(-sum.y), expf(-sum.z));
        store_rgba(out, (size_t)set * per_set + t, T, 1.f);
    }
}

// ---------------------------------------------------------------------------
// MULTISCATTERING (Atmosphere.glsl:342-438): one 128-thread block per texel.
// The 64 sphere directions of GetDirectionFromLocalIndex (:344-355) are
// (cos phi sin theta, cos theta, sin phi sin theta) on an 8 x 8 (theta, phi)
// grid, with the start point on the y axis and the sun in the y-z plane.  The
// integrand depends on the direction only through its y and z components
// (the height along the ray, cos(sun, zenith) at each sample, cos(view, sun)),
// so phi and pi - phi give the same luminance: the phi columns 0, 1, 4, 5 are
// integrated and stand for their mirrors 3, 2, 7, 6, and the sums over the 32
// directions are doubled.  Thread t integrates chunk (t % kMsChunks) of
// direction t / kMsChunks; the chunks of a direction are composed through
// shuffles, the directions summed through shuffles and a shared-memory pass
// over the block's warps.
// ---------------------------------------------------------------------------
constexpr int kMsChunks = 4;
constexpr int kMsDirs = 32;  // mirror pairs of the 64 directions
constexpr int kMsThreads = kMsDirs * kMsChunks;

template <class S, bool TABLE>
__global__ void __launch_bounds__(kMsThreads) multiscattering_kernel(JobSrc<TABLE> jobs, int n_sets, LutView L,
                                                                     int tstride, int w, int h,
                                                                     S* __restrict__ out) {
    __shared__ float red[kMsThreads / 32][6];
    int texel = blockIdx.x;
    int per_set = w * h;
    int set = texel / per_set;
    int t = texel % per_set;
    const AtmoConsts& A = jobs.get(set).a;
    LutView Ls = L;
    Ls.t = L.t + (size_t)set * tstride;
    int ix = t % w, iy = t / w;
    float x_mu_s = (float)ix / (float)(w - 1);
    float x_alt = (float)iy / (float)(h - 1);
    float alt = x_alt * A.thickness;
    float mu_s = x_mu_s * 2.f - 1.f;
    float sun_z = sqrtf(1.f - mu_s * mu_s);
    float r = alt + A.R;
    float rho2 = alt * (2.f * A.R + alt);
    float steps = A.multiscattering_steps;
    int n = sample_count(0.5f, steps);
    const float iso = 1.f / (4.f * SKYR_PI);

    int pair = threadIdx.x / kMsChunks;
    int chunk = threadIdx.x % kMsChunks;
    int phi_col = (pair & 1) | ((pair & 2) << 1);  // 0, 1, 4, 5 (mirrors 3, 2, 7, 6)
    float unit_theta = (0.5f + (float)(pair >> 2)) / 8.f;
    float unit_phi = (0.5f + (float)phi_col) / 8.f;
    float cos_theta = 1.f - 2.f * unit_theta;
    float sin_theta = sqrtf(clamp01(1.f - cos_theta * cos_theta));
    float sphi, cphi;
    sincospif(2.f * unit_phi, &sphi, &cphi);
    float3 view = f3(cphi * sin_theta, cos_theta, sphi * sin_theta);
    float mu = view.y;
    bool ground = ray_hits_ground(r, rho2, mu);
    float dist = ground ? dist_to_bottom(r, rho2, mu) : dist_to_top(r, A.thickness - alt, A.top, mu);
    RayStart s0{r, alt, rho2, mu, mu_s, view.z * sun_z + view.y * mu_s};
    int k0 = (n * chunk) / kMsChunks, k1 = (n * (chunk + 1)) / kMsChunks;
    float3 lum, tr, lf;
    pdl_wait();  // the transmittance LUT
    integrate<true, float4>(A, Ls, nullptr, 0, 0, s0, dist / steps, 0.5f, k0, k1, iso, iso, lum, tr, lf);
    pdl_launch_dependents();
    compose_lanes<kMsChunks>(lum, tr, &lf);
    if (chunk == 0 && ground) {
        // ComputeGroundLuminance (Atmosphere.glsl:297-306) at r = R
        float mu_s_g = (r * mu_s + dist * s0.nu) / A.R;
        float3 sv = sun_visibility_lut(A, Ls.t, Ls.tw, Ls.th, A.R, 0.f, 0.f, mu_s_g);
        lum += tr * (A.ground_albedo * sv * (clamp01(mu_s_g) / SKYR_PI));
    }
    if (chunk != 0) lum = lf = f3(0.f);
#pragma unroll
    for (int o = 16; o >= kMsChunks; o >>= 1) {
        lum.x += __shfl_xor_sync(0xffffffffu, lum.x, o);
        lum.y += __shfl_xor_sync(0xffffffffu, lum.y, o);
        lum.z += __shfl_xor_sync(0xffffffffu, lum.z, o);
        lf.x += __shfl_xor_sync(0xffffffffu, lf.x, o);
        lf.y += __shfl_xor_sync(0xffffffffu, lf.y, o);
        lf.z += __shfl_xor_sync(0xffffffffu, lf.z, o);
    }
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        red[warp][0] = lum.x; red[warp][1] = lum.y; red[warp][2] = lum.z;
        red[warp][3] = lf.x; red[warp][4] = lf.y; red[warp][5] = lf.z;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float3 L2 = f3(0.f), F = f3(0.f);
#pragma unroll
        for (int i = 0; i < kMsThreads / 32; ++i) {
            L2 += f3(red[i][0], red[i][1], red[i][2]);
            F += f3(red[i][3], red[i][4], red[i][5]);
        }
        // each pair counts twice: (2 x the sum over 32 pairs) / 64 directions
        float3 l2 = L2 * (1.f / 32.f), fms = F * (1.f / 32.f);
        float3 c = l2 / (f3(1.f) - fms);
        store_rgba(out, (size_t)set * per_set + t, c, 1.f);
    }
}

// ---------------------------------------------------------------------------
// SKY_VIEW (AtmosphereRenderer.glsl:147-188) and AERIAL_PERSPECTIVE
// (:191-245) in one launch: rays [0, n_sv) are sky-view texels, the rest are
// aerial-perspective froxels.  LANES lanes per ray.
// ---------------------------------------------------------------------------

template <int LANES, class S, bool TABLE>
__global__ void __launch_bounds__(128) view_luts_kernel(JobSrc<TABLE> jobs, int n_sets, LutView L, int tstride,
                                                        const S* __restrict__ ms, int mw, int mh, int msstride,
                                                        int sv_w, int sv_h, int ap_w, int ap_h, int ap_d,
                                                        S* __restrict__ sv_lum, S* __restrict__ sv_trans,
                                                        S* __restrict__ ap_lum, S* __restrict__ ap_trans) {
    // A programmatic dependent of this pass (the raymarch of skyr_render_frame)
    // may be scheduled as soon as all its blocks run: it reads the LUTs only
    // after its own griddepcontrol.wait, that is after this pass has ended.
    pdl_launch_dependents();
    int gid = blockIdx.x * blockDim.x + threadIdx.x;
    int lane = gid % LANES;
    int ray = gid / LANES;
    int n_sv = sv_w * sv_h, n_ap = ap_w * ap_h * ap_d;
    int per_set = n_sv + n_ap;
    int set = ray / per_set;
    bool valid = set < n_sets;
    if (!valid) set = n_sets - 1;
    int t = ray % per_set;
    const LutSetJob& J = jobs.get(set);
    const AtmoConsts& A = J.a;
    const ViewConsts& V = J.v;
    LutView Ls = L;
    Ls.t = L.t + (size_t)set * tstride;
    const S* mss = ms + (size_t)set * msstride;

    float3 view;
    float mu, marching, steps;
    RayStart s0;
    bool is_sv = t < n_sv;
    if (is_sv) {
        // GetCosLatLonFromSkyViewTextureIndex / GetViewDirectionFromCosLatLon (:74-111)
        int ix = t % sv_w, iy = t / sv_w;
        float x_cos_lon = (float)ix / (float)(sv_w - 1);
        float x_cos_lat = (float)iy / (float)(sv_h - 1);
        float horizon_down = acosf(sqrtf(fmaxf(V.cam_rho2, 0.f)) / V.cam_r);
        float horizon_up = SKYR_PI - horizon_down;
        float lat;
        if (x_cos_lat < 0.5f) {
            float c = 1.f - 2.f * x_cos_lat;
            lat = horizon_up * (1.f - c * c);
        } else {
            float c = x_cos_lat * 2.f - 1.f;
            lat = horizon_up + horizon_down * (c * c);
        }
        float cos_lat = cosf(lat);
        float cos_lon = -(x_cos_lon * x_cos_lon * 2.f - 1.f);
        float sin_lat = clamp01(sqrtf(1.f - cos_lat * cos_lat));
        float sin_lon = clamp01(sqrtf(1.f - cos_lon * cos_lon));
        view = V.up * cos_lat + V.front * (sin_lat * cos_lon) + V.right * (sin_lat * sin_lon);
        mu = cos_lat;
        bool ground = ray_hits_ground(V.cam_r, V.cam_rho2, mu);
        marching = ground ? dist_to_bottom(V.cam_r, V.cam_rho2, mu)
                          : dist_to_top(V.cam_r, A.thickness - V.cam_h, A.top, mu);
        s0 = ray_start(A, V, mu, dot3(view, V.sun), marching);
        steps = V.sky_view_steps;
    } else {
        // GetMarchingDistanceFromAerialPerspectiveTextureIndex (:191-197) + main (:205-243)
        int q = t - n_sv;
        int ix = q % ap_w, iy = (q / ap_w) % ap_h, iz = q / (ap_w * ap_h);
        float x = 2.f * ((float)ix / (float)(ap_w - 1)) - 1.f;
        float y = 2.f * ((float)iy / (float)(ap_h - 1)) - 1.f;
        float wz = (float)iz / (float)(ap_d - 1);
        float3 dir = V.ap_a0 * x + V.ap_a1 * y + V.ap_a3;
        float wsign = fmaf(V.ap_w0, x, fmaf(V.ap_w1, y, V.ap_w3)) < 0.f ? -1.f : 1.f;
        view = dir * (wsign * rsqrtf(dot3(dir, dir)));
        marching = wz * wz * V.ap_max_distance;
        mu = dot3(view, V.up);
        bool ground = ray_hits_ground(V.cam_r, V.cam_rho2, mu);
        float max_marching = ground ? marching : dist_to_top(V.cam_r, A.thickness - V.cam_h, A.top, mu);
        s0 = ray_start(A, V, mu, dot3(view, V.sun), max_marching);
        marching = fminf(marching, max_marching);
        steps = V.ap_steps;
    }
    float nu = s0.nu;
    float3 lum = f3(0.f), tr = f3(1.f), lf;
    bool active = marching > 0.f;
    pdl_wait();  // the transmittance and multi-scattering LUTs
    if (active) {
        // RayleighPhaseFunction / MiePhaseFunction (Atmosphere.glsl:138-154)
        float ph_r = 3.f / (16.f * SKYR_PI) * (1.f + nu * nu);
        float g = A.mie_g;
        float den = 1.f + g * g - 2.f * g * nu;
        float ph_m = A.mie_phase_k * (1.f + nu * nu) / (den * sqrtf(den));
        int n = sample_count(0.5f, steps);
        int k0 = (n * lane) / LANES, k1 = (n * (lane + 1)) / LANES;
        integrate<false, S>(A, Ls, mss, mw, mh, s0, marching / steps, 0.5f, k0, k1, ph_r, ph_m, lum, tr, lf);
    }
    // every lane of a group shares `active`, so the shuffles stay converged
    compose_lanes<LANES>(lum, tr, nullptr);
    if (valid && lane == 0) {
        if (is_sv) {
            size_t o = (size_t)set * n_sv + t;
            store_rgba(sv_lum, o, lum, 0.f);
            store_rgba(sv_trans, o, tr, 0.f);
        } else {
            size_t o = (size_t)set * n_ap + (t - n_sv);
            store_rgba(ap_lum, o, lum, 0.f);
            store_rgba(ap_trans, o, tr, 0.f);
        }
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
// Lanes per texel / ray are a tuning choice (skyr_tuning): 2, 4, 8 or 16.
template <int LANES, bool TABLE>
static void t_launch(JobSrc<TABLE> jobs, int n_sets, const skyr_lut_sizes& s, float4* out, cudaStream_t st) {
    long long threads = (long long)n_sets * s.transmittance_width * s.transmittance_height * LANES;
    int blocks = (int)((threads + 127) / 128);
    transmittance_kernel<LANES, TABLE>
        <<<blocks, 128, 0, st>>>(jobs, n_sets, s.transmittance_width, s.transmittance_height, out);
}

template <bool TABLE>
cudaError_t launch_transmittance(JobSrc<TABLE> jobs, int n_sets, const skyr_lut_sizes& s, float4* out,
                                 cudaStream_t st, int lanes) {
    switch (lanes) {
        case 2: t_launch<2, TABLE>(jobs, n_sets, s, out, st); break;
        case 4: t_launch<4, TABLE>(jobs, n_sets, s, out, st); break;
        case 16: t_launch<16, TABLE>(jobs, n_sets, s, out, st); break;
        default: t_launch<8, TABLE>(jobs, n_sets, s, out, st); break;
    }
    return cudaGetLastError();
}

// A launch whose blocks may start before the previous kernel on the stream has
// finished (programmatic stream serialisation); the kernel orders its reads with
// pdl_wait.
template <class... P, class... A>
static cudaError_t launch_dependent(void (*kernel)(P...), dim3 grid, dim3 block, cudaStream_t st, A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

template <class S, bool TABLE>
cudaError_t launch_multiscattering(JobSrc<TABLE> jobs, int n_sets, const skyr_lut_sizes& s, const float4* tlut,
                                   S* out, cudaStream_t st) {
    int blocks = n_sets * s.multiscattering_width * s.multiscattering_height;
    LutView L{tlut, s.transmittance_width, s.transmittance_height};
    if (cudaError_t e = launch_dependent(multiscattering_kernel<S, TABLE>, dim3(blocks), dim3(kMsThreads), st, jobs,
                                         n_sets, L, s.transmittance_width * s.transmittance_height,
                                         s.multiscattering_width, s.multiscattering_height, out))
        return e;
    return cudaGetLastError();
}

template <int LANES, class S, bool TABLE>
static void v_launch(JobSrc<TABLE> jobs, int n_sets, const skyr_lut_sizes& s, const float4* tlut, const S* ms,
                     S* svl, S* svt, S* apl, S* apt, cudaStream_t st) {
    long long rays = (long long)n_sets * (s.sky_view_width * s.sky_view_height +
                                          s.aerial_perspective_width * s.aerial_perspective_height *
                                              s.aerial_perspective_depth);
    int blocks = (int)((rays * LANES + 127) / 128);
    LutView L{tlut, s.transmittance_width, s.transmittance_height};
    launch_dependent(view_luts_kernel<LANES, S, TABLE>, dim3(blocks), dim3(128), st, jobs, n_sets, L,
                     s.transmittance_width * s.transmittance_height, ms, s.multiscattering_width,
                     s.multiscattering_height, s.multiscattering_width * s.multiscattering_height, s.sky_view_width,
                     s.sky_view_height, s.aerial_perspective_width, s.aerial_perspective_height,
                     s.aerial_perspective_depth, svl, svt, apl, apt);
}

template <class S, bool TABLE>
cudaError_t launch_view_luts(JobSrc<TABLE> jobs, int n_sets, const skyr_lut_sizes& s, const float4* tlut,
                             const S* ms, S* svl, S* svt, S* apl, S* apt, cudaStream_t st, int lanes) {
    switch (lanes) {
        case 2: v_launch<2, S, TABLE>(jobs, n_sets, s, tlut, ms, svl, svt, apl, apt, st); break;
        case 4: v_launch<4, S, TABLE>(jobs, n_sets, s, tlut, ms, svl, svt, apl, apt, st); break;
        case 16: v_launch<16, S, TABLE>(jobs, n_sets, s, tlut, ms, svl, svt, apl, apt, st); break;
        default: v_launch<8, S, TABLE>(jobs, n_sets, s, tlut, ms, svl, svt, apl, apt, st); break;
    }
    return cudaGetLastError();
}

#define SKYR_INST(TABLE)                                                                                        \
    template cudaError_t launch_transmittance<TABLE>(JobSrc<TABLE>, int, const skyr_lut_sizes&, float4*,        \
                                                     cudaStream_t, int);                                        \
    template cudaError_t launch_multiscattering<float4, TABLE>(JobSrc<TABLE>, int, const skyr_lut_sizes&,       \
                                                               const float4*, float4*, cudaStream_t);           \
    template cudaError_t launch_multiscattering<__half2, TABLE>(JobSrc<TABLE>, int, const skyr_lut_sizes&,      \
                                                                const float4*, __half2*, cudaStream_t);         \
    template cudaError_t launch_view_luts<float4, TABLE>(JobSrc<TABLE>, int, const skyr_lut_sizes&,             \
                                                         const float4*, const float4*, float4*, float4*,        \
                                                         float4*, float4*, cudaStream_t, int);                  \
    template cudaError_t launch_view_luts<__half2, TABLE>(JobSrc<TABLE>, int, const skyr_lut_sizes&,            \
                                                          const float4*, const __half2*, __half2*, __half2*,    \
                                                          __half2*, __half2*, cudaStream_t, int);
SKYR_INST(false)
SKYR_INST(true)
#undef SKYR_INST

}  // namespace skyr
