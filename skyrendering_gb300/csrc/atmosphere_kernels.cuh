// atmosphere_kernels.cuh — launch interface of the atmosphere LUT kernels.
#pragma once

#include "skyr_internal.cuh"

namespace skyr {

// Where a kernel reads its per-set constants: one job by value in the kernel
// parameters (TABLE = false, single set, no upload) or a device table of jobs
// indexed by set (TABLE = true, batched).
template <bool TABLE>
struct JobSrc;
template <>
struct JobSrc<false> {
    LutSetJob j;
    __device__ __forceinline__ const LutSetJob& get(int) const { return j; }
};
template <>
struct JobSrc<true> {
    const LutSetJob* t;
    __device__ __forceinline__ const LutSetJob& get(int s) const { return t[s]; }
};

// `lanes`: lanes per texel / ray (2, 4, 8, 16; anything else is 8)
template <bool TABLE>
cudaError_t launch_transmittance(JobSrc<TABLE> jobs, int n_sets, const skyr_lut_sizes& s, float4* out,
                                 cudaStream_t st, int lanes);
template <class S, bool TABLE>
cudaError_t launch_multiscattering(JobSrc<TABLE> jobs, int n_sets, const skyr_lut_sizes& s, const float4* tlut,
                                   S* out, cudaStream_t st);
template <class S, bool TABLE>
cudaError_t launch_view_luts(JobSrc<TABLE> jobs, int n_sets, const skyr_lut_sizes& s, const float4* tlut,
                             const S* ms, S* svl, S* svt, S* apl, S* apt, cudaStream_t st, int lanes);

}  // namespace skyr
