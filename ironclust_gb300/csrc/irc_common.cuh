// irc_common.cuh -- shared definitions of the sm_103a hot-path library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ircgb300.h"

// The reference's "no candidate" sentinel, a double literal stored into
// float registers (matlab/search_min_drift.cu:10).
#define IRC_SINGLE_INF_F ((float)3.402E+38)

// Largest feature count any kernel here accepts (the reference's shared
// arrays hold 45 for the irc2 kernels and 60 for the irc.m ones).
#define IRC_NC_MAX 64

namespace irc {

// One reference distance term: d = b - a (single rounding), acc += d*d as one
// fused multiply-add -- the contraction nvcc applies to `dist += d*d` in every
// reference kernel.  The intrinsics keep the compiler from re-associating.
__device__ __forceinline__ float dterm(float acc, float b, float a)
{
    const float d = __fsub_rn(b, a);
    return __fmaf_rn(d, d, acc);
}

// sqrt(ABS(x)) of the reference kernels, IEEE round-to-nearest.
__device__ __forceinline__ float ref_sqrt_abs(float x) { return __fsqrt_rn(fabsf(x)); }

// 64-bit sort key of a non-negative float value and a position: MATLAB's
// ascending stable sort order with NaN after every number.  A "taken" entry
// uses key ~0ull, after everything.
__device__ __forceinline__ unsigned long long sort_key(float v, int pos)
{
    unsigned int b = __float_as_uint(v);
    if (v != v) b = 0x7fc00000u;                 // any NaN: after +inf
    else if (b & 0x80000000u) b = 0u;           // -0.0 (only negative value possible)
    return ((unsigned long long)b << 32) | (unsigned int)pos;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long k)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long other = __shfl_xor_sync(0xffffffffu, k, o);
        k = other < k ? other : k;
    }
    return k;
}

}  // namespace irc

// Host-side helpers shared by the translation units.
namespace irc_host {
void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *where);
// Validation of a plan's host arrays (the meaning irc_plan_create gives
// them), shared by every entry point that takes them: non-null arrays,
// 1 <= nChunks < 2^28, roff[0] = 0, strictly increasing roff, every chunk's
// queries inside both [0, nF) and [q_base, q_base + n_out), every run inside
// [0, nF); bounds are formed in 64-bit arithmetic.  Returns IRC_OK or
// IRC_E_INVAL (message prefixed by `who`); on success *pairs and *max_nq
// (either may be null) receive the plan's (query, candidate) pair count and
// its largest query chunk.
int check_plan(const char *who, const int32_t *q0, const int32_t *nq, const int32_t *roff, const int32_t *rs,
               const int32_t *rn, int nChunks, int q_base, int n_out, int nF, long long *pairs, int *max_nq);
}  // namespace irc_host

#define IRC_CHECK_LAUNCH(where)                                                    \
    do {                                                                            \
        cudaError_t _e = cudaGetLastError();                                        \
        if (_e != cudaSuccess) return irc_host::cuda_status(_e, where);             \
    } while (0)
