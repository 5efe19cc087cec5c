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

// cuda_knn_index: per-thread minimum over iB = t, t+nT, ... (self kept),
// then the reference's in-kernel selection sort with swaps, one warp per
// query (each step = first position of the minimum over [iK, nT)).
__global__ void __launch_bounds__(kThreads)
k_knn_index(float *__restrict__ K, int *__restrict__ I, const float *__restrict__ B,
            const float *__restrict__ A, int nB, int nA, int nC, int knn, int nT)
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
        for (int iB = t; iB < nB; iB += nT) {
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
                const int p = (int)(best & 0xffffffffu);
                const float tf = d[p]; d[p] = d[iK]; d[iK] = tf;
                const int ti = ix[p]; ix[p] = ix[iK]; ix[iK] = ti;
            }
            __syncwarp();
        }
        const int qa = a0 + q;
        if (lane == 0) K[qa] = irc::ref_sqrt_abs(d[knn - 1]);
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

int irc_cuda_knn_index(float *K, int32_t *I, const float *B, const float *A,
                       const int32_t *vnConst, int nThreads, void *stream)
{
    if (!K || !I || !B || !A || !vnConst) { irc_host::set_error("irc_cuda_knn_index: null pointer"); return IRC_E_INVAL; }
    const int nB = vnConst[0], nA = vnConst[1], nC = vnConst[2], knn = vnConst[3];
    if (nC > IRC_NC_MAX) { irc_host::set_error("irc_cuda_knn_index: nC=%d > %d", nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || nA <= 0 || nB <= 0 || knn <= 0 || nThreads <= 0 || nThreads > 1024 || knn > nThreads) {
        irc_host::set_error("irc_cuda_knn_index: bad sizes nB=%d nA=%d nC=%d knn=%d nThreads=%d", nB, nA, nC, knn, nThreads);
        return IRC_E_INVAL;
    }
    const size_t smem = (size_t)kQB * nThreads * (sizeof(float) + sizeof(int));
    cudaError_t e = cudaFuncSetAttribute(k_knn_index, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_cuda_knn_index: smem attribute");
    k_knn_index<<<cdiv(nA, kQB), kThreads, smem, (cudaStream_t)stream>>>(K, I, B, A, nB, nA, nC, knn, nThreads);
    IRC_CHECK_LAUNCH("irc_cuda_knn_index");
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
