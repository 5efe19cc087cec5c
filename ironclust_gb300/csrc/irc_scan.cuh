// irc_scan.cuh -- the per-bin minimum scan of the irc2 search kernels.
//
// search_min_drift / search_delta_drift (matlab/search_min_drift.cu:60-84,
// matlab/search_delta_drift.cu:62-96) give every thread tx of an nT-thread
// block one "bin": run b = tx % nBB of the linked-chunk runs, scanned from
// IBB[b] + tx/nBB with stride nT/nBB.  The bin keeps the first strict minimum
// of d2 > 0 (and, for delta, only candidates whose rho exceeds the query's).
// Here one thread evaluates one bin for QB queries at once: the queries'
// features sit in shared memory transposed as sA[c*QB + q] (broadcast
// float4 reads), the candidate's features stream through registers, and the
// per-query minima stay in registers.  Distances use the reference
// arithmetic (irc::dterm), so each bin minimum is bit-identical.
#pragma once
#include "irc_common.cuh"

namespace irc {

template <int QB, bool DELTA>
__device__ __forceinline__ void scan_bin(const float *__restrict__ F, const float *__restrict__ R,
                                         int nC, int start, int end, int stride,
                                         const float *__restrict__ sA, const float *__restrict__ sRA,
                                         float (&mn)[QB], int (&mi)[QB])
{
    static_assert(QB % 4 == 0 && QB <= 32, "QB must be a multiple of 4, at most 32");
    for (int iB = start; iB < end; iB += stride) {
        const float *fb = F + (size_t)iB * nC;
        unsigned live = 0xffffffffu;
        if (DELTA) {
            const float rb = __ldg(R + iB);
            live = 0;
#pragma unroll
            for (int q = 0; q < QB; ++q)
                if (!(rb <= sRA[q])) live |= 1u << q;       // reference masks rb <= ra
            if (!live) continue;
        }
        float acc[QB];
#pragma unroll
        for (int q = 0; q < QB; ++q) acc[q] = 0.0f;
        for (int c = 0; c < nC; ++c) {
            const float bv = __ldg(fb + c);
            const float4 *a4 = reinterpret_cast<const float4 *>(sA + c * QB);
#pragma unroll
            for (int j = 0; j < QB / 4; ++j) {
                const float4 a = a4[j];
                acc[4 * j + 0] = dterm(acc[4 * j + 0], bv, a.x);
                acc[4 * j + 1] = dterm(acc[4 * j + 1], bv, a.y);
                acc[4 * j + 2] = dterm(acc[4 * j + 2], bv, a.z);
                acc[4 * j + 3] = dterm(acc[4 * j + 3], bv, a.w);
            }
        }
#pragma unroll
        for (int q = 0; q < QB; ++q)
            if (((live >> q) & 1u) && acc[q] < mn[q] && acc[q] > 0.0f) {
                mn[q] = acc[q];
                mi[q] = iB;
            }
    }
}

// Stage QB query columns of F (column-major, first query qs, n valid) into
// sA[c*QB + q]; invalid slots repeat the last valid query.
template <int QB>
__device__ __forceinline__ void stage_queries(const float *__restrict__ F, int nC, int qs, int n,
                                              float *sA)
{
    for (int i = threadIdx.x; i < nC * QB; i += blockDim.x) {
        const int c = i / QB, q = i - c * QB;
        const int qa = qs + min(q, n - 1);
        sA[i] = __ldg(F + (size_t)qa * nC + c);
    }
}

}  // namespace irc
