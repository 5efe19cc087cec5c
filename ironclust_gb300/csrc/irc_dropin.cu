// irc_dropin.cu -- the five drop-in kernels (one call == one MATLAB feval).
//
// Each kernel reproduces the output arrays of the reference kernel it
// replaces bit for bit, but is organised for sm_103a: many queries per CTA
// (fewer re-reads of the candidate features from L2), query features staged
// once in shared memory and read as broadcast float4s, bins or candidate
// strides walked by independent threads, and warp-level arg-min reductions
// in place of the reference's single-thread loops.
#include <algorithm>
#include <climits>

#include "irc_common.cuh"
#include "irc_scan.cuh"

namespace {

constexpr int kThreads = 256;   // CTA size of the drop-in search kernels
constexpr int kQB = 16;         // queries per CTA

// search_min_drift / search_delta_drift: D, I [nT x nA].
template <bool DELTA>
__global__ void __launch_bounds__(kThreads)
k_search_drift(float *__restrict__ D, int *__restrict__ I, const float *__restrict__ F,
               const float *__restrict__ R, const int *__restrict__ IBB,
               const int *__restrict__ NBB, int nC, int nBB, int iA0, int nA, int nT)
{
    __shared__ __align__(16) float sA[IRC_NC_MAX * kQB];
    __shared__ float sRA[kQB];
    const int a0 = blockIdx.x * kQB;                 // first query of this CTA (chunk-relative)
    const int n = min(kQB, nA - a0);
    irc::stage_queries<kQB>(F, nC, iA0 + a0, n, sA);
    if (DELTA && threadIdx.x < kQB) sRA[threadIdx.x] = __ldg(R + iA0 + a0 + min((int)threadIdx.x, n - 1));
    __syncthreads();
    const int nT0 = nT / nBB;
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
        const int b = t % nBB;
        const int ib0 = __ldg(IBB + b), nb0 = __ldg(NBB + b);
        float mn[kQB];
        int mi[kQB];
#pragma unroll
        for (int q = 0; q < kQB; ++q) { mn[q] = IRC_SINGLE_INF_F; mi[q] = iA0 + a0 + min(q, n - 1); }
        irc::scan_bin<kQB, DELTA>(F, R, nC, ib0 + t / nBB, ib0 + nb0, nT0, sA, sRA, mn, mi);
#pragma unroll
        for (int q = 0; q < kQB; ++q)
            if (q < n) {
                const size_t o = (size_t)t + (size_t)nT * (a0 + q);
                D[o] = irc::ref_sqrt_abs(mn[q]);
                I[o] = mi[q] + 1;
            }
    }
}

// The binned minimum + selection sort of cuda_knn_index, cuda_knn,
// cuda_knn_full and cuda_knn_ib: per-thread minimum over iiB = t, t+nT, ...
// (self kept; IND maps iiB through IB, 1-based, and records the mapped
// column), then the reference's in-kernel selection sort with swaps, one warp
// per query (each step = first position of the minimum over [iK, nT); a slot
// holding NaN at step iK stays, since nothing compares below NaN there).
// KALL writes every sorted distance [knn x nA], else the knn-th [nA]; I is
// optional.  IB entries outside 1..nF are skipped and counted in *bad.
template <bool IND, bool KALL>
__global__ void __launch_bounds__(kThreads)
k_knn_bins(float *__restrict__ K, int *__restrict__ I, const float *__restrict__ B,
           const float *__restrict__ A, const int *__restrict__ IB, int nF, int *__restrict__ bad, int nB, int nA,
           int nC, int knn, int nT)
{
    __shared__ __align__(16) float sA[IRC_NC_MAX * kQB];
    extern __shared__ __align__(16) unsigned char dyn[];
    float *sD = reinterpret_cast<float *>(dyn);              // [kQB][nT]
    int *sI = reinterpret_cast<int *>(sD + kQB * nT);        // [kQB][nT]
    const int a0 = blockIdx.x * kQB;
    const int n = min(kQB, nA - a0);
    irc::stage_queries<kQB>(A, nC, a0, n, sA);
    __syncthreads();
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
        float mn[kQB];
        int mi[kQB];
#pragma unroll
        for (int q = 0; q < kQB; ++q) { mn[q] = IRC_SINGLE_INF_F; mi[q] = 0; }
        for (int iiB = t; iiB < nB; iiB += nT) {
            int iB = iiB;
            if (IND) {
                iB = __ldg(IB + iiB) - 1;
                if (iB < 0 || iB >= nF) {
                    if (blockIdx.x == 0) atomicAdd(bad, 1);
                    continue;
                }
            }
            const float *fb = B + (size_t)iB * nC;
            float acc[kQB];
#pragma unroll
            for (int q = 0; q < kQB; ++q) acc[q] = 0.0f;
            for (int c = 0; c < nC; ++c) {
                const float bv = __ldg(fb + c);
                const float4 *a4 = reinterpret_cast<const float4 *>(sA + c * kQB);
#pragma unroll
                for (int j = 0; j < kQB / 4; ++j) {
                    const float4 a = a4[j];
                    acc[4 * j + 0] = irc::dterm(acc[4 * j + 0], bv, a.x);
                    acc[4 * j + 1] = irc::dterm(acc[4 * j + 1], bv, a.y);
                    acc[4 * j + 2] = irc::dterm(acc[4 * j + 2], bv, a.z);
                    acc[4 * j + 3] = irc::dterm(acc[4 * j + 3], bv, a.w);
                }
            }
#pragma unroll
            for (int q = 0; q < kQB; ++q)
                if (acc[q] < mn[q]) { mn[q] = acc[q]; mi[q] = iB; }
        }
#pragma unroll
        for (int q = 0; q < kQB; ++q) { sD[q * nT + t] = mn[q]; sI[q * nT + t] = mi[q]; }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = warp; q < n; q += nw) {
        float *d = sD + q * nT;
        int *ix = sI + q * nT;
        for (int iK = 0; iK < knn; ++iK) {
            unsigned long long best = ~0ull;
            for (int p = iK + lane; p < nT; p += 32) {
                const unsigned long long k = irc::sort_key(d[p], p);
                best = k < best ? k : best;
            }
            best = irc::warp_min_u64(best);
            if (lane == 0) {
                const int p = isnan(d[iK]) ? iK : (int)(best & 0xffffffffu);
                const float tf = d[p]; d[p] = d[iK]; d[iK] = tf;
                const int ti = ix[p]; ix[p] = ix[iK]; ix[iK] = ti;
            }
            __syncwarp();
        }
        const int qa = a0 + q;
        if (KALL) {
            for (int iK = lane; iK < knn; iK += 32) K[iK + (size_t)knn * qa] = irc::ref_sqrt_abs(d[iK]);
        } else if (lane == 0) {
            K[qa] = irc::ref_sqrt_abs(d[knn - 1]);
        }
        if (I)
            for (int iK = lane; iK < knn; iK += 32) I[iK + (size_t)knn * qa] = ix[iK] + 1;
        __syncwarp();
    }
}

// cuda_delta_knn: thread t keeps the minimum over iB = t, t+nT, ... with
// R_B > R_A (strict), then the lowest slot holding the overall minimum wins;
// when no slot found a candidate the index falls back to the query (A-space).
__global__ void __launch_bounds__(128)
k_delta_knn(float *__restrict__ D, unsigned *__restrict__ N, const float *__restrict__ B,
            const float *__restrict__ A, const float *__restrict__ RB, const float *__restrict__ RA,
            int nB, int nA, int nC)
{
    __shared__ __align__(16) float sA[IRC_NC_MAX * kQB];
    __shared__ float sRA[kQB];
    __shared__ unsigned long long sKey[kQB][128];
    __shared__ unsigned sN[kQB][128];
    const int nT = blockDim.x, t = threadIdx.x;
    const int a0 = blockIdx.x * kQB;
    const int n = min(kQB, nA - a0);
    irc::stage_queries<kQB>(A, nC, a0, n, sA);
    if (t < kQB) sRA[t] = __ldg(RA + a0 + min(t, n - 1));
    __syncthreads();
    float mn[kQB];
    unsigned mi[kQB];
#pragma unroll
    for (int q = 0; q < kQB; ++q) { mn[q] = IRC_SINGLE_INF_F; mi[q] = 0u; }
    for (int iB = t; iB < nB; iB += nT) {
        const float rb = __ldg(RB + iB);
        unsigned live = 0;
#pragma unroll
        for (int q = 0; q < kQB; ++q)
            if (rb > sRA[q]) live |= 1u << q;
        if (!live) continue;
        const float *fb = B + (size_t)iB * nC;
        float acc[kQB];
#pragma unroll
        for (int q = 0; q < kQB; ++q) acc[q] = 0.0f;
        for (int c = 0; c < nC; ++c) {
            const float bv = __ldg(fb + c);
            const float4 *a4 = reinterpret_cast<const float4 *>(sA + c * kQB);
#pragma unroll
            for (int j = 0; j < kQB / 4; ++j) {
                const float4 a = a4[j];
                acc[4 * j + 0] = irc::dterm(acc[4 * j + 0], bv, a.x);
                acc[4 * j + 1] = irc::dterm(acc[4 * j + 1], bv, a.y);
                acc[4 * j + 2] = irc::dterm(acc[4 * j + 2], bv, a.z);
                acc[4 * j + 3] = irc::dterm(acc[4 * j + 3], bv, a.w);
            }
        }
#pragma unroll
        for (int q = 0; q < kQB; ++q)
            if (((live >> q) & 1u) && acc[q] < mn[q]) { mn[q] = acc[q]; mi[q] = (unsigned)iB; }
    }
#pragma unroll
    for (int q = 0; q < kQB; ++q) { sKey[q][t] = irc::sort_key(mn[q], t); sN[q][t] = mi[q]; }
    __syncthreads();
    const int lane = t & 31, warp = t >> 5, nw = nT >> 5;
    for (int q = warp; q < n; q += nw) {
        unsigned long long best = ~0ull;
        for (int s = lane; s < nT; s += 32) best = sKey[q][s] < best ? sKey[q][s] : best;
        best = irc::warp_min_u64(best);
        if (lane == 0) {
            const int s = (int)(best & 0xffffffffu);
            const float v = __uint_as_float((unsigned)(best >> 32));
            const int qa = a0 + q;
            const bool found = v < IRC_SINGLE_INF_F;
            D[qa] = irc::ref_sqrt_abs(found ? v : IRC_SINGLE_INF_F);
            N[qa] = (found ? sN[q][s] : (unsigned)qa) + 1u;
        }
    }
}

// jrc3_cuda_rho_drift: fraction of site-matched candidates within dc2.
__global__ void __launch_bounds__(128)
k_rho_drift(float *__restrict__ rho, const int *__restrict__ site12, const float *__restrict__ f1,
            const float *__restrict__ f2, int n1, int n12, int nC, float dc2)
{
    __shared__ __align__(16) float sA[IRC_NC_MAX * kQB];
    __shared__ int sSite[kQB];
    __shared__ int sRho[kQB], sComp[kQB];
    const int a0 = blockIdx.x * kQB;
    const int n = min(kQB, n1 - a0);
    irc::stage_queries<kQB>(f1, nC, a0, n, sA);
    if (threadIdx.x < kQB) {
        sSite[threadIdx.x] = threadIdx.x < n ? __ldg(site12 + a0 + threadIdx.x) : INT_MIN;
        sRho[threadIdx.x] = 0;
        sComp[threadIdx.x] = 0;
    }
    __syncthreads();
    int nr[kQB], nc[kQB];
#pragma unroll
    for (int q = 0; q < kQB; ++q) { nr[q] = 0; nc[q] = 0; }
    for (int j = threadIdx.x; j < n12; j += blockDim.x) {
        const int s1 = __ldg(site12 + j), s2 = __ldg(site12 + j + n12);
#pragma unroll
        for (int q = 0; q < kQB; ++q) {
            const float *src = (s1 == sSite[q]) ? f1 : (s2 == sSite[q]) ? f2 : nullptr;
            if (!src) continue;
            src += (size_t)j * nC;
            float acc = 0.0f;
            for (int c = 0; c < nC; ++c) acc = irc::dterm(acc, sA[c * kQB + q], __ldg(src + c));
            nr[q] += (acc <= dc2);
            nc[q] += 1;
        }
    }
#pragma unroll
    for (int q = 0; q < kQB; ++q) {
        int r = nr[q], c = nc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            r += __shfl_xor_sync(0xffffffffu, r, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
        }
        if ((threadIdx.x & 31) == 0 && c) { atomicAdd(&sRho[q], r); atomicAdd(&sComp[q], c); }
    }
    __syncthreads();
    if (threadIdx.x < n)
        rho[a0 + threadIdx.x] = (float)((double)sRho[threadIdx.x] / (double)sComp[threadIdx.x]);
}

// jrc3_cuda_delta_drift: nearest site-matched candidate with strictly higher
// rho.  Thread t keeps its first strict minimum over j = t, t+128, ...; the
// lowest thread holding the overall minimum wins; none -> the query itself.
__global__ void __launch_bounds__(128)
k_delta_drift(float *__restrict__ delta, unsigned *__restrict__ nneigh, const int *__restrict__ site12,
              const float *__restrict__ f1, const float *__restrict__ f2, const float *__restrict__ rho, int n1,
              int n12, int nC, float dc2)
{
    __shared__ __align__(16) float sA[IRC_NC_MAX * kQB];
    __shared__ int sSite[kQB];
    __shared__ float sR[kQB];
    __shared__ unsigned long long sKey[kQB][128 / 32];
    __shared__ unsigned sIdx[kQB][128 / 32];
    const int a0 = blockIdx.x * kQB;
    const int n = min(kQB, n1 - a0);
    irc::stage_queries<kQB>(f1, nC, a0, n, sA);
    if (threadIdx.x < kQB) {
        sSite[threadIdx.x] = threadIdx.x < n ? __ldg(site12 + a0 + threadIdx.x) : INT_MIN;
        sR[threadIdx.x] = __ldg(rho + a0 + min((int)threadIdx.x, n - 1));
    }
    __syncthreads();
    float mn[kQB];
    unsigned mi[kQB];
#pragma unroll
    for (int q = 0; q < kQB; ++q) { mn[q] = IRC_SINGLE_INF_F; mi[q] = 0u; }
    for (int j = threadIdx.x; j < n12; j += blockDim.x) {
        const float rj = __ldg(rho + j);
        const int s1 = __ldg(site12 + j), s2 = __ldg(site12 + j + n12);
#pragma unroll
        for (int q = 0; q < kQB; ++q) {
            if (rj <= sR[q]) continue;
            const float *src = (s1 == sSite[q]) ? f1 : (s2 == sSite[q]) ? f2 : nullptr;
            if (!src) continue;
            src += (size_t)j * nC;
            float acc = 0.0f;
            for (int c = 0; c < nC; ++c) acc = irc::dterm(acc, sA[c * kQB + q], __ldg(src + c));
            if (acc < mn[q]) { mn[q] = acc; mi[q] = (unsigned)j; }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kQB; ++q) {
        unsigned long long k = irc::sort_key(mn[q], threadIdx.x);
        unsigned idx = mi[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ok = __shfl_xor_sync(0xffffffffu, k, o);
            const unsigned oi = __shfl_xor_sync(0xffffffffu, idx, o);
            if (ok < k) { k = ok; idx = oi; }
        }
        if (lane == 0) { sKey[q][warp] = k; sIdx[q][warp] = idx; }
    }
    __syncthreads();
    if (threadIdx.x < n) {
        const int q = threadIdx.x;
        unsigned long long k = sKey[q][0];
        unsigned idx = sIdx[q][0];
        for (int w = 1; w < 4; ++w)
            if (sKey[q][w] < k) { k = sKey[q][w]; idx = sIdx[q][w]; }
        const float v = __uint_as_float((unsigned)(k >> 32));
        const bool found = v < IRC_SINGLE_INF_F;
        const float dmin = found ? v : IRC_SINGLE_INF_F;
        delta[a0 + q] = __fsqrt_rn(__fdiv_rn(fabsf(dmin), dc2));
        nneigh[a0 + q] = (found ? idx : (unsigned)(a0 + q)) + 1u;
    }
}

// jrc3_cuda_rho (irc_cuda_rho.cu): query i1 < n1 counts the candidates j < n12
// within the time window |ord[i1] - ord[j]| <= dn_max (itself included) and
// those at d2 <= dc2 (fdc = 1: d2 < dc2 * |query|^2, fused-accumulated in
// feature order, then one multiply).  Integer counts, so the result does not
// depend on the scan order; rho = count / compared, divided in double.
__global__ void __launch_bounds__(128)
k_rho_st(float *__restrict__ rho, const float *__restrict__ F, const int *__restrict__ ord, int n1, int n12,
         int nC, int dn_max, int fdc, float dc2)
{
    __shared__ __align__(16) float sA[IRC_NC_MAX * kQB];
    __shared__ int sOrd[kQB], sRho[kQB], sComp[kQB];
    __shared__ float sCut[kQB];
    const int a0 = blockIdx.x * kQB;
    const int n = min(kQB, n1 - a0);
    irc::stage_queries<kQB>(F, nC, a0, n, sA);
    if (threadIdx.x < kQB) {
        sOrd[threadIdx.x] = threadIdx.x < n ? __ldg(ord + a0 + threadIdx.x) : 0;
        sRho[threadIdx.x] = 0;
        sComp[threadIdx.x] = 0;
    }
    __syncthreads();
    if (threadIdx.x < kQB) {
        float cut = dc2;
        if (fdc == 1) {
            float v = 0.0f;
            for (int c = 0; c < nC; ++c) v = __fmaf_rn(sA[c * kQB + threadIdx.x], sA[c * kQB + threadIdx.x], v);
            cut = __fmul_rn(v, dc2);
        }
        sCut[threadIdx.x] = cut;
    }
    __syncthreads();
    int nr[kQB], nc[kQB];
#pragma unroll
    for (int q = 0; q < kQB; ++q) { nr[q] = 0; nc[q] = 0; }
    for (int j = threadIdx.x; j < n12; j += blockDim.x) {
        const int oj = __ldg(ord + j);
        const float *src = F + (size_t)j * nC;
#pragma unroll
        for (int q = 0; q < kQB; ++q) {
            if (q >= n || abs(sOrd[q] - oj) > dn_max) continue;
            float acc = 0.0f;
            for (int c = 0; c < nC; ++c) acc = irc::dterm(acc, __ldg(src + c), sA[c * kQB + q]);
            nr[q] += fdc == 0 ? (acc <= sCut[q]) : (acc < sCut[q]);
            nc[q] += 1;
        }
    }
#pragma unroll
    for (int q = 0; q < kQB; ++q) {
        int r = nr[q], c = nc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            r += __shfl_xor_sync(0xffffffffu, r, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
        }
        if ((threadIdx.x & 31) == 0 && c) { atomicAdd(&sRho[q], r); atomicAdd(&sComp[q], c); }
    }
    __syncthreads();
    if (threadIdx.x < n)
        rho[a0 + threadIdx.x] = (float)((double)sRho[threadIdx.x] / (double)sComp[threadIdx.x]);
}

// jrc3_cuda_delta (irc_cuda_delta.cu): nearest candidate within the time
// window ranked before the query in rho order (rr[j] < rr[i1]).  One thread
// per bin (blockDim = the reference's nThreads): thread t keeps its first
// strict minimum over j = t, t+nT, ...; the lowest thread holding the
// overall minimum wins; none below SINGLE_INF -> the query itself.
// delta = sqrt(d2 / dc2) (fdc = 1: / (dc2 * |query|^2)).
__global__ void __launch_bounds__(128)
k_delta_st(float *__restrict__ delta, unsigned *__restrict__ nneigh, const float *__restrict__ F,
           const int *__restrict__ ord, const int *__restrict__ rr, int n1, int n12, int nC, int dn_max, int fdc,
           float dc2)
{
    __shared__ __align__(16) float sA[IRC_NC_MAX * kQB];
    __shared__ int sOrd[kQB], sRR[kQB];
    __shared__ float sCut[kQB];
    __shared__ unsigned long long sKey[kQB][128 / 32];
    __shared__ unsigned sIdx[kQB][128 / 32];
    const int a0 = blockIdx.x * kQB;
    const int n = min(kQB, n1 - a0);
    irc::stage_queries<kQB>(F, nC, a0, n, sA);
    if (threadIdx.x < kQB) {
        sOrd[threadIdx.x] = threadIdx.x < n ? __ldg(ord + a0 + threadIdx.x) : 0;
        sRR[threadIdx.x] = threadIdx.x < n ? __ldg(rr + a0 + threadIdx.x) : INT_MIN;
    }
    __syncthreads();
    if (threadIdx.x < kQB) {
        float cut = dc2;
        if (fdc == 1) {
            float v = 0.0f;
            for (int c = 0; c < nC; ++c) v = __fmaf_rn(sA[c * kQB + threadIdx.x], sA[c * kQB + threadIdx.x], v);
            cut = __fmul_rn(v, dc2);
        }
        sCut[threadIdx.x] = cut;
    }
    __syncthreads();
    float mn[kQB];
    unsigned mi[kQB];
#pragma unroll
    for (int q = 0; q < kQB; ++q) { mn[q] = IRC_SINGLE_INF_F; mi[q] = 0u; }
    for (int j = threadIdx.x; j < n12; j += blockDim.x) {
        const int oj = __ldg(ord + j), rj = __ldg(rr + j);
        const float *src = F + (size_t)j * nC;
#pragma unroll
        for (int q = 0; q < kQB; ++q) {
            if (!(rj < sRR[q]) || abs(sOrd[q] - oj) > dn_max) continue;
            float acc = 0.0f;
            for (int c = 0; c < nC; ++c) acc = irc::dterm(acc, __ldg(src + c), sA[c * kQB + q]);
            if (acc < mn[q]) { mn[q] = acc; mi[q] = (unsigned)j; }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < kQB; ++q) {
        unsigned long long k = irc::sort_key(mn[q], threadIdx.x);
        unsigned idx = mi[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ok = __shfl_xor_sync(0xffffffffu, k, o);
            const unsigned oi = __shfl_xor_sync(0xffffffffu, idx, o);
            if (ok < k) { k = ok; idx = oi; }
        }
        if (lane == 0) { sKey[q][warp] = k; sIdx[q][warp] = idx; }
    }
    __syncthreads();
    if (threadIdx.x < n) {
        const int q = threadIdx.x;
        unsigned long long k = sKey[q][0];
        unsigned idx = sIdx[q][0];
        for (int w = 1; w < nw; ++w)
            if (sKey[q][w] < k) { k = sKey[q][w]; idx = sIdx[q][w]; }
        const float v = __uint_as_float((unsigned)(k >> 32));
        const bool found = v < IRC_SINGLE_INF_F;
        const float dmin = found ? v : IRC_SINGLE_INF_F;
        delta[a0 + q] = __fsqrt_rn(__fdiv_rn(dmin, sCut[q]));
        nneigh[a0 + q] = (found ? idx : (unsigned)(a0 + q)) + 1u;
    }
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace

// Exact top-k fill of the search_min_drift output (IRC_MODE_EXACT), in irc_site.cu.
int irc_exact_chunk_fill(float *D, int32_t *I, const float *F, const int32_t *IBB,
                         const int32_t *NBB, int nC, int nBB, int iA0, int nA, int nT, int knn,
                         int nF, cudaStream_t s);

extern "C" {

int irc_search_min_drift(float *D, int32_t *I, const float *F, const int32_t *IBB,
                         const int32_t *NBB, const int32_t *vnConst, int nThreads, int mode,
                         int knn, void *stream)
{
    if (!D || !I || !F || !IBB || !NBB || !vnConst) {
        irc_host::set_error("irc_search_min_drift: null pointer");
        return IRC_E_INVAL;
    }
    const int nC = vnConst[0], nBB = vnConst[2], iA0 = vnConst[3], nA = vnConst[4];
    if (nC > IRC_NC_MAX) { irc_host::set_error("irc_search_min_drift: nC=%d > %d", nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || nA <= 0 || iA0 < 0 || nBB <= 0 || nThreads <= 0 || nThreads > 1024 || nBB > nThreads) {
        irc_host::set_error("irc_search_min_drift: bad sizes nC=%d nBB=%d iA0=%d nA=%d nThreads=%d",
                            nC, nBB, iA0, nA, nThreads);
        return IRC_E_INVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (mode == IRC_MODE_EXACT) {
        if (knn <= 0 || knn > nThreads) { irc_host::set_error("irc_search_min_drift: bad knn %d", knn); return IRC_E_INVAL; }
        return irc_exact_chunk_fill(D, I, F, IBB, NBB, nC, nBB, iA0, nA, nThreads, knn, vnConst[1], s);
    }
    if (mode != IRC_MODE_REF) { irc_host::set_error("irc_search_min_drift: unsupported mode %d", mode); return IRC_E_UNSUPPORTED; }
    k_search_drift<false><<<cdiv(nA, kQB), kThreads, 0, s>>>(D, I, F, nullptr, IBB, NBB, nC, nBB, iA0, nA, nThreads);
    IRC_CHECK_LAUNCH("irc_search_min_drift");
    return IRC_OK;
}

int irc_search_delta_drift(float *D, int32_t *I, const float *F, const float *R,
                           const int32_t *IBB, const int32_t *NBB, const int32_t *vnConst,
                           int nThreads, void *stream)
{
    if (!D || !I || !F || !R || !IBB || !NBB || !vnConst) {
        irc_host::set_error("irc_search_delta_drift: null pointer");
        return IRC_E_INVAL;
    }
    const int nC = vnConst[0], nBB = vnConst[2], iA0 = vnConst[3], nA = vnConst[4];
    if (nC > IRC_NC_MAX) { irc_host::set_error("irc_search_delta_drift: nC=%d > %d", nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || nA <= 0 || iA0 < 0 || nBB <= 0 || nThreads <= 0 || nThreads > 1024 || nBB > nThreads) {
        irc_host::set_error("irc_search_delta_drift: bad sizes");
        return IRC_E_INVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    k_search_drift<true><<<cdiv(nA, kQB), kThreads, 0, s>>>(D, I, F, R, IBB, NBB, nC, nBB, iA0, nA, nThreads);
    IRC_CHECK_LAUNCH("irc_search_delta_drift");
    return IRC_OK;
}

}  // extern "C"

namespace {

// Shared host side of the four binned-kNN drop-ins.  IB entries outside
// 1..nF are counted on the device and reported after a stream sync.
template <bool IND, bool KALL>
int launch_knn_bins(const char *name, float *K, int32_t *I, const float *B, const float *A, const int32_t *IB,
                    int nF, const int32_t *vnConst, int nThreads, void *stream)
{
    if (!K || !B || !A || !vnConst || (IND && !IB)) { irc_host::set_error("%s: null pointer", name); return IRC_E_INVAL; }
    const int nB = vnConst[0], nA = vnConst[1], nC = vnConst[2], knn = vnConst[3];
    if (nC > IRC_NC_MAX) { irc_host::set_error("%s: nC=%d > %d", name, nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || nA <= 0 || nB <= 0 || knn <= 0 || nThreads <= 0 || nThreads > 1024 || knn > nThreads ||
        (IND && nF <= 0)) {
        irc_host::set_error("%s: bad sizes nB=%d nA=%d nC=%d knn=%d nThreads=%d", name, nB, nA, nC, knn, nThreads);
        return IRC_E_INVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const size_t smem = (size_t)kQB * nThreads * (sizeof(float) + sizeof(int));
    cudaError_t e = cudaFuncSetAttribute(k_knn_bins<IND, KALL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return irc_host::cuda_status(e, name);
    int *bad = nullptr;
    if (IND) {
        e = cudaMallocAsync(&bad, sizeof(int), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), s);
        if (e != cudaSuccess) return irc_host::cuda_status(e, name);
    }
    k_knn_bins<IND, KALL><<<cdiv(nA, kQB), kThreads, smem, s>>>(K, I, B, A, IB, nF, bad, nB, nA, nC, knn, nThreads);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        if (bad) cudaFreeAsync(bad, s);
        return irc_host::cuda_status(e, name);
    }
    if (IND) {
        int hbad = 0;
        e = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(bad, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return irc_host::cuda_status(e, name);
        if (hbad) {
            irc_host::set_error("%s: %d IB entries outside 1..%d (skipped)", name, hbad, nF);
            return IRC_E_INVAL;
        }
    }
    return IRC_OK;
}

}  // namespace

extern "C" {

int irc_cuda_knn_index(float *K, int32_t *I, const float *B, const float *A,
                       const int32_t *vnConst, int nThreads, void *stream)
{
    if (!I) { irc_host::set_error("irc_cuda_knn_index: null pointer"); return IRC_E_INVAL; }
    return launch_knn_bins<false, false>("irc_cuda_knn_index", K, I, B, A, nullptr, 0, vnConst, nThreads, stream);
}

int irc_cuda_knn(float *K, const float *B, const float *A, const int32_t *vnConst, int nThreads, void *stream)
{
    return launch_knn_bins<false, false>("irc_cuda_knn", K, nullptr, B, A, nullptr, 0, vnConst, nThreads, stream);
}

int irc_cuda_knn_full(float *K, int32_t *I, const float *B, const float *A, const int32_t *vnConst, int nThreads,
                      void *stream)
{
    if (!I) { irc_host::set_error("irc_cuda_knn_full: null pointer"); return IRC_E_INVAL; }
    return launch_knn_bins<false, true>("irc_cuda_knn_full", K, I, B, A, nullptr, 0, vnConst, nThreads, stream);
}

int irc_cuda_knn_ib(float *K, int32_t *I, const float *B, const float *A, const int32_t *IB, int nF,
                    const int32_t *vnConst, int nThreads, void *stream)
{
    if (!I) { irc_host::set_error("irc_cuda_knn_ib: null pointer"); return IRC_E_INVAL; }
    return launch_knn_bins<true, false>("irc_cuda_knn_ib", K, I, B, A, IB, nF, vnConst, nThreads, stream);
}

int irc_cuda_rho(float *vrRho1, const float *mrFet12, const int32_t *viiSpk12_ord, const int32_t *vnConst,
                 float dc2, void *stream)
{
    if (!vrRho1 || !mrFet12 || !viiSpk12_ord || !vnConst) { irc_host::set_error("irc_cuda_rho: null pointer"); return IRC_E_INVAL; }
    const int n1 = vnConst[0], n12 = vnConst[1], nC = vnConst[2], dn_max = vnConst[3], fdc = vnConst[4];
    if (nC > IRC_NC_MAX) { irc_host::set_error("irc_cuda_rho: nC=%d > %d", nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || n1 <= 0 || n12 < n1 || dn_max < 0 || (fdc != 0 && fdc != 1)) {
        irc_host::set_error("irc_cuda_rho: bad sizes n1=%d n12=%d nC=%d dn_max=%d fDc_spk=%d", n1, n12, nC, dn_max, fdc);
        return IRC_E_INVAL;
    }
    k_rho_st<<<cdiv(n1, kQB), 128, 0, (cudaStream_t)stream>>>(vrRho1, mrFet12, viiSpk12_ord, n1, n12, nC, dn_max,
                                                              fdc, dc2);
    IRC_CHECK_LAUNCH("irc_cuda_rho");
    return IRC_OK;
}

int irc_cuda_delta(float *vrDelta1, uint32_t *viNneigh1, const float *mrFet12, const int32_t *viiSpk12_ord,
                   const int32_t *viiRho12_ord, const int32_t *vnConst, float dc2, int nThreads, void *stream)
{
    if (!vrDelta1 || !viNneigh1 || !mrFet12 || !viiSpk12_ord || !viiRho12_ord || !vnConst) {
        irc_host::set_error("irc_cuda_delta: null pointer");
        return IRC_E_INVAL;
    }
    const int n1 = vnConst[0], n12 = vnConst[1], nC = vnConst[2], dn_max = vnConst[3], fdc = vnConst[4];
    if (nC > IRC_NC_MAX) { irc_host::set_error("irc_cuda_delta: nC=%d > %d", nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || n1 <= 0 || n12 < n1 || dn_max < 0 || (fdc != 0 && fdc != 1) || nThreads < 32 ||
        nThreads > 128 || nThreads % 32) {
        irc_host::set_error("irc_cuda_delta: bad sizes n1=%d n12=%d nC=%d dn_max=%d fDc_spk=%d nThreads=%d "
                            "(nThreads: a multiple of 32 up to 128, the reference's NTHREADS)",
                            n1, n12, nC, dn_max, fdc, nThreads);
        return IRC_E_INVAL;
    }
    k_delta_st<<<cdiv(n1, kQB), nThreads, 0, (cudaStream_t)stream>>>(vrDelta1, viNneigh1, mrFet12, viiSpk12_ord,
                                                                     viiRho12_ord, n1, n12, nC, dn_max, fdc, dc2);
    IRC_CHECK_LAUNCH("irc_cuda_delta");
    return IRC_OK;
}

int irc_cuda_delta_knn(float *D, uint32_t *N, const float *B, const float *A, const float *R_B,
                       const float *R_A, const int32_t *vnConst, int nThreads, void *stream)
{
    if (!D || !N || !B || !A || !R_B || !R_A || !vnConst) { irc_host::set_error("irc_cuda_delta_knn: null pointer"); return IRC_E_INVAL; }
    const int nB = vnConst[0], nA = vnConst[1], nC = vnConst[2];
    if (nC > IRC_NC_MAX) { irc_host::set_error("irc_cuda_delta_knn: nC=%d > %d", nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || nA <= 0 || nB < 0 || nThreads != 128) {
        irc_host::set_error("irc_cuda_delta_knn: bad sizes (nThreads must be 128, the reference block size)");
        return IRC_E_INVAL;
    }
    k_delta_knn<<<cdiv(nA, kQB), 128, 0, (cudaStream_t)stream>>>(D, N, B, A, R_B, R_A, nB, nA, nC);
    IRC_CHECK_LAUNCH("irc_cuda_delta_knn");
    return IRC_OK;
}

int irc_rho_drift(float *vrRho1, const int32_t *miSite12, const float *mrFet1, const float *mrFet2,
                  const int32_t *vnConst, float dc2, void *stream)
{
    if (!vrRho1 || !miSite12 || !mrFet1 || !mrFet2 || !vnConst) { irc_host::set_error("irc_rho_drift: null pointer"); return IRC_E_INVAL; }
    const int n1 = vnConst[0], n12 = vnConst[1], nC = vnConst[2];
    if (nC > IRC_NC_MAX) { irc_host::set_error("irc_rho_drift: nC=%d > %d", nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || n1 <= 0 || n12 < n1) { irc_host::set_error("irc_rho_drift: bad sizes n1=%d n12=%d nC=%d", n1, n12, nC); return IRC_E_INVAL; }
    k_rho_drift<<<cdiv(n1, kQB), 128, 0, (cudaStream_t)stream>>>(vrRho1, miSite12, mrFet1, mrFet2, n1, n12, nC, dc2);
    IRC_CHECK_LAUNCH("irc_rho_drift");
    return IRC_OK;
}

int irc_delta_drift(float *vrDelta1, uint32_t *viNneigh1, const int32_t *miSite12, const float *mrFet1,
                    const float *mrFet2, const float *vrRho1, const int32_t *vnConst, float dc2, void *stream)
{
    if (!vrDelta1 || !viNneigh1 || !miSite12 || !mrFet1 || !mrFet2 || !vrRho1 || !vnConst) {
        irc_host::set_error("irc_delta_drift: null pointer");
        return IRC_E_INVAL;
    }
    const int n1 = vnConst[0], n12 = vnConst[1], nC = vnConst[2];
    if (nC > IRC_NC_MAX) { irc_host::set_error("irc_delta_drift: nC=%d > %d", nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || n1 <= 0 || n12 < n1) { irc_host::set_error("irc_delta_drift: bad sizes n1=%d n12=%d nC=%d", n1, n12, nC); return IRC_E_INVAL; }
    k_delta_drift<<<cdiv(n1, kQB), 128, 0, (cudaStream_t)stream>>>(vrDelta1, viNneigh1, miSite12, mrFet1, mrFet2,
                                                                  vrRho1, n1, n12, nC, dc2);
    IRC_CHECK_LAUNCH("irc_delta_drift");
    return IRC_OK;
}

}  // extern "C"
