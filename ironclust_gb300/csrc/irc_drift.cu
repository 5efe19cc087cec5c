// irc_drift.cu -- the drift linkage of calc_drift_ (matlab/irc2.m:6373-6465)
// on the device: which drift chunks a chunk's spikes are compared with.
//
//   limits     viLim = [0, ceil((1:n)/n * nSpk)] (equal spike counts)
//   edges      quantile_vr_ (matlab/irc2.m:6481-6490) of the amplitudes
//              (nQuantile + 1 edges) and of the positions (nSites + 1 edges):
//              a fixed subsample (subsample_vr_, chosen on the host from the
//              spike count alone) sorted on the device, picked at
//              round(m * q) -- MATLAB's sort 'ascend' is a stable radix sort
//              of an order-preserving 32-bit key here
//   counts     histcounts2 of (amplitude, position) per chunk into
//              [nQuantile x nSites] bins (bins [e_k, e_k+1), the last closed;
//              values outside the edges dropped), one atomic per spike
//   linkage    per chunk j, the nTime_batch nearest chunks by the Euclidean
//              distance between count columns, ties by chunk index (MATLAB's
//              stable sort), over all chunks when n <= nTime_max_drift, else
//              over the band calc_drift_ masks (|i - j| <= nTime_max_drift/4
//              widened at both ends) -- for every column that mask is one
//              contiguous interval of rows.  Counts are integers, so the
//              squared distances are exact int64 and the order is the order
//              of the true distances.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cub/cub.cuh>
#include <vector>

#include "ircgb300.h"
#include "irc_common.cuh"

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ uint32_t asc_key(float f)
{
    if (isnan(f)) return 0xffffffffu;                 // NaN last
    uint32_t u = __float_as_uint(f);
    if (f == 0.0f) u = 0u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float asc_float(uint32_t o)
{
    if (o == 0xffffffffu) return __uint_as_float(0x7fc00000u);
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

__global__ void k_gather_keys(const float *__restrict__ v, const int64_t *__restrict__ pos, int m,
                              uint32_t *__restrict__ keys)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) keys[i] = asc_key(v[pos[i]]);
}

__global__ void k_pick(const uint32_t *__restrict__ sorted, const int32_t *__restrict__ idx, int ne,
                       float *__restrict__ edges)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ne) edges[k] = asc_float(sorted[idx[k]]);
}

// histcounts2 bin of x for edges e[0..nb]: -1 when outside
__device__ __forceinline__ int hbin(float x, const float *e, int nb)
{
    if (!(x >= e[0]) || !(x <= e[nb])) return -1;
    if (x == e[nb]) return nb - 1;
    int lo = 0, hi = nb;                              // largest k with e[k] <= x
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (e[mid] <= x) lo = mid; else hi = mid;
    }
    return lo;
}

__global__ void k_hist2(const float *__restrict__ amp, const float *__restrict__ pos, int64_t nSpk,
                        const int64_t *__restrict__ lim, int n, const float *__restrict__ ampE, int nA,
                        const float *__restrict__ posE, int nP, int *__restrict__ counts)
{
    __shared__ float sA[1025], sP[1025];
    for (int k = threadIdx.x; k <= nA; k += blockDim.x) sA[k] = ampE[k];
    for (int k = threadIdx.x; k <= nP; k += blockDim.x) sP[k] = posE[k];
    __syncthreads();
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nSpk; s += (int64_t)gridDim.x * blockDim.x) {
        const int ia = hbin(amp[s], sA, nA), ip = hbin(pos[s], sP, nP);
        if (ia < 0 || ip < 0) continue;
        int lo = 0, hi = n;                           // chunk c: lim[c] <= s < lim[c+1]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (lim[mid] <= s) lo = mid; else hi = mid;
        }
        atomicAdd(&counts[(size_t)lo * (nA * nP) + ia + nA * ip], 1);
    }
}

// One CTA per chunk j: the nb nearest rows of [lo, hi] by (squared distance, row).
__global__ void __launch_bounds__(TPB) k_link(const int *__restrict__ counts, int nBins, int n, int nb, int quarter,
                                              int masked, int32_t *__restrict__ members)
{
    constexpr int MAXC = 1024;
    __shared__ long long sD[MAXC];
    __shared__ long long rd[TPB / 32];
    __shared__ int ri[TPB / 32];
    const int j = blockIdx.x;
    int lo = 0, hi = n - 1;
    if (masked) {
        if (j < quarter) { lo = 0; hi = min(n - 1, 2 * quarter); }
        else if (j >= n - quarter) { lo = max(0, n - 2 * quarter - 1); hi = n - 1; }
        else { lo = j - quarter; hi = j + quarter; }
    }
    const int m = hi - lo + 1;                        // <= MAXC (checked on the host)
    const int *cj = counts + (size_t)j * nBins;
    for (int t = threadIdx.x; t < m; t += TPB) {
        const int *ci = counts + (size_t)(lo + t) * nBins;
        long long d = 0;
        for (int b = 0; b < nBins; ++b) {
            const long long x = (long long)ci[b] - (long long)cj[b];
            d += x * x;
        }
        sD[t] = d;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < nb; ++k) {
        long long bd = LLONG_MAX;
        int bi = INT_MAX;
        for (int t = threadIdx.x; t < m; t += TPB)
            if (sD[t] < bd || (sD[t] == bd && t < bi)) { bd = sD[t]; bi = t; }
        for (int o = 16; o; o >>= 1) {
            const long long od = __shfl_xor_sync(0xffffffffu, bd, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (od < bd || (od == bd && oi < bi)) { bd = od; bi = oi; }
        }
        if (lane == 0) { rd[w] = bd; ri[w] = bi; }
        __syncthreads();
        if (threadIdx.x == 0) {
            long long d0 = rd[0];
            int i0 = ri[0];
            for (int u = 1; u < TPB / 32; ++u)
                if (rd[u] < d0 || (rd[u] == d0 && ri[u] < i0)) { d0 = rd[u]; i0 = ri[u]; }
            members[k + (size_t)nb * j] = lo + i0;
            sD[i0] = LLONG_MAX;                       // taken
        }
        __syncthreads();
    }
}

// subsample_vr_ (matlab/irc2.m:1557-1573) of the positions 0..N-1
std::vector<int64_t> subsample_positions(int64_t N, int64_t nMax)
{
    std::vector<int64_t> v;
    if (N <= nMax) {
        v.resize((size_t)N);
        for (int64_t i = 0; i < N; ++i) v[(size_t)i] = i;
        return v;
    }
    const int64_t nSkip = N / nMax;
    for (int64_t i = 0; i < N; i += (nSkip > 1 ? nSkip : 1)) v.push_back(i);
    const int64_t m = (int64_t)v.size();
    if (m > nMax) {
        const int64_t nRemove = m - nMax;
        std::vector<char> drop((size_t)m, 0);
        // round(linspace(1, m, nRemove)) clamped to 1..m; linspace as
        // k * step + 1 with step = (m - 1) / (nRemove - 1), the last point m
        const double step = nRemove > 1 ? ((double)m - 1.0) / (double)(nRemove - 1) : 0.0;
        for (int64_t k = 0; k < nRemove; ++k) {
            const double x = (k == nRemove - 1) ? (double)m : (double)k * step + 1.0;
            int64_t r = (int64_t)std::floor(x + 0.5);
            r = r < 1 ? 1 : (r > m ? m : r);
            drop[(size_t)(r - 1)] = 1;
        }
        std::vector<int64_t> w;
        for (int64_t i = 0; i < m; ++i)
            if (!drop[(size_t)i]) w.push_back(v[(size_t)i]);
        v.swap(w);
    }
    return v;
}

struct Scratch {
    cudaStream_t s;
    std::vector<void *> ptrs;
    cudaError_t err = cudaSuccess;
    explicit Scratch(cudaStream_t st) : s(st) {}
    template <class T>
    T *get(size_t n)
    {
        void *q = nullptr;
        if (err == cudaSuccess) err = cudaMallocAsync(&q, sizeof(T) * (n ? n : 1), s);
        if (err != cudaSuccess) return nullptr;
        ptrs.push_back(q);
        return (T *)q;
    }
    ~Scratch()
    {
        for (void *q : ptrs) cudaFreeAsync(q, s);
    }
};

// quantile_vr_ edges of v (device) for the fractions (0:nq)/nq
cudaError_t quantile_edges(Scratch &sc, const float *v, const std::vector<int64_t> &sub, int nq, float *edges)
{
    const int m = (int)sub.size();
    int64_t *dpos = sc.get<int64_t>(m);
    uint32_t *k0 = sc.get<uint32_t>(m), *k1 = sc.get<uint32_t>(m);
    int32_t *didx = sc.get<int32_t>(nq + 1);
    if (sc.err != cudaSuccess) return sc.err;
    std::vector<int32_t> idx((size_t)nq + 1);
    for (int k = 0; k <= nq; ++k) {
        const double q = (double)k / (double)nq;
        double r = std::floor((double)m * q + 0.5);     // round(n * q), n * q >= 0
        r = r > m ? m : r;
        r = r < 1 ? 1 : r;
        idx[(size_t)k] = (int32_t)r - 1;
    }
    cudaError_t e = cudaMemcpyAsync(dpos, sub.data(), sizeof(int64_t) * (size_t)m, cudaMemcpyHostToDevice, sc.s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(didx, idx.data(), sizeof(int32_t) * idx.size(), cudaMemcpyHostToDevice, sc.s);
    if (e != cudaSuccess) return e;
    k_gather_keys<<<(m + TPB - 1) / TPB, TPB, 0, sc.s>>>(v, dpos, m, k0);
    size_t tb = 0;
    e = cub::DeviceRadixSort::SortKeys(nullptr, tb, k0, k1, m, 0, 32, sc.s);
    if (e != cudaSuccess) return e;
    void *tmp = sc.get<char>(tb);
    if (!tmp) return sc.err;
    e = cub::DeviceRadixSort::SortKeys(tmp, tb, k0, k1, m, 0, 32, sc.s);
    if (e != cudaSuccess) return e;
    k_pick<<<(nq + 1 + TPB - 1) / TPB, TPB, 0, sc.s>>>(k1, didx, nq + 1, edges);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(sc.s);              // the host vectors above are read by the copies
}

}  // namespace

extern "C" int irc_calc_drift(int32_t *miDrift, int64_t *viLim, int *nDrift_out, const float *vrAmp,
                              const float *vrPos, int64_t nSpk, int nSites, int nTime_drift, int nTime_batch,
                              int nTime_max_drift, int nQuantile, void *stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (!miDrift || !viLim || !nDrift_out || !vrAmp || !vrPos || nSpk < 1 || nSites < 1 || nQuantile < 1 ||
        nSites > 1024 || nQuantile > 1024 || nTime_max_drift < 4 || nTime_max_drift % 4) {
        irc_host::set_error("irc_calc_drift: need non-null arrays, nSpk >= 1, 1 <= nSites, nQuantile <= 1024, "
                            "nTime_max_drift a positive multiple of 4");
        return IRC_E_INVAL;
    }
    // the single-chunk branch (matlab/irc2.m:6386-6389)
    if (nTime_batch <= 0 || nTime_drift <= 0 || nTime_batch >= nTime_drift) {
        const int64_t lim[2] = {0, nSpk};
        std::vector<int32_t> mem((size_t)(nTime_batch > 0 ? nTime_batch : 1), 0);
        cudaError_t e = cudaMemcpyAsync(viLim, lim, sizeof(lim), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(miDrift, mem.data(), sizeof(int32_t) * mem.size(), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_calc_drift");
        *nDrift_out = 1;
        return IRC_OK;
    }
    const int n = nTime_drift;
    const bool masked = n > nTime_max_drift;
    const int quarter = nTime_max_drift / 4;
    const int span = masked ? 2 * quarter + 1 : n;
    if (span > 1024 || nTime_batch > span) {
        irc_host::set_error("irc_calc_drift: %d candidate chunks per chunk (limit 1024, and >= nTime_batch = %d)",
                            span, nTime_batch);
        return IRC_E_INVAL;
    }
    std::vector<int64_t> lim((size_t)n + 1);
    lim[0] = 0;
    for (int k = 1; k <= n; ++k) lim[(size_t)k] = (int64_t)std::ceil((double)k / (double)n * (double)nSpk);
    const std::vector<int64_t> sub = subsample_positions(nSpk, 100000);

    Scratch sc(s);
    const int nBins = nQuantile * nSites;
    float *ampE = sc.get<float>(nQuantile + 1), *posE = sc.get<float>(nSites + 1);
    int *counts = sc.get<int>((size_t)nBins * n);
    if (sc.err != cudaSuccess) return irc_host::cuda_status(sc.err, "irc_calc_drift: scratch");
    cudaError_t e = cudaMemcpyAsync(viLim, lim.data(), sizeof(int64_t) * lim.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = quantile_edges(sc, vrAmp, sub, nQuantile, ampE);
    if (e == cudaSuccess) e = quantile_edges(sc, vrPos, sub, nSites, posE);
    if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)nBins * n, s);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_calc_drift: edges");
    const int64_t hb = (nSpk + TPB - 1) / TPB;
    k_hist2<<<(unsigned)(hb < 152 * 8 ? hb : 152 * 8), TPB, 0, s>>>(vrAmp, vrPos, nSpk, viLim, n, ampE, nQuantile,
                                                                    posE, nSites, counts);
    k_link<<<n, TPB, 0, s>>>(counts, nBins, n, nTime_batch, quarter, masked ? 1 : 0, miDrift);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_calc_drift");
    *nDrift_out = n;
    return IRC_OK;
}
