// irc_cluster.cu -- the clustering step that consumes the path's outputs, on
// the device:
//
//   irc_sort_rho            sort_'s normalisation: rho / max(rho) and the
//                           descending order ordrho (matlab/irc2.m:3263-3264)
//   irc_assign_cluster_knn  postCluster_ (matlab/irc2.m:6520-6535):
//                           assignCluster_knn_ (:6640-6694), cell2map_
//                           (:6754-6805), dpclus_remove_count_ (:6735-6750)
//
// Layout and method.  Everything is integer or ordering work over arrays in
// HBM, bound by memory traffic and, for the peak merge, by L2:
//
//  * Orders.  MATLAB's sort(..., 'descend') (NaN first, stable) becomes an
//    ascending, stable radix sort (CUB) of a 32-bit key that inverts the
//    float's total order and maps NaN to 0.
//  * Peak merge.  The sets cvi{i} of cell2map_ are rows of a P x P bit
//    matrix (P peaks, one bit per peak).  Row i starts as the peaks whose kNN
//    list shares a value with peak i: the (value, peak) pairs of all lists
//    are radix-sorted by value and every run of equal values sets its pairs.
//    A cell2map_ repeat is one CTA per row: the union of row i with the rows
//    of its members (a boolean row product in shared memory), then the
//    "later set overwrites" rule as an atomicMax of the row index into an
//    owner per peak, then each row becomes its owner's union.  The repeat
//    loop and its size-equality stop test run as in MATLAB, up to ten times.
//  * Label propagation.  One MATLAB pass visits the unassigned spikes in
//    ordrho order and copies the label of nneigh in place.  In rank space
//    (r = position in ordrho) a spike takes the label its nneigh has at
//    the moment it is visited: the final label of this pass when nneigh is
//    unassigned and visited earlier (smaller rank), otherwise the label
//    nneigh had when the pass started.  That is a forest whose edges go to
//    strictly smaller ranks; pointer jumping over a packed 64-bit state
//    (done flag | label, or the rank it points to) resolves it in
//    O(log depth) rounds of coalesced passes.  Passes repeat (at most ten)
//    while spikes stay unassigned, as in MATLAB.
//  * Cluster sizes.  A shared-memory histogram (or warp-aggregated global
//    atomics for many clusters), a scan of the keep flags, one remap pass.
//
// Host round trips: the peak count, each cell2map_ repeat's stop test, the
// cluster count, each pass's unassigned count and convergence checks of the
// jumping rounds, the final counts.  The call synchronises its stream.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cub/cub.cuh>
#include <vector>

#include "ircgb300.h"
#include "irc_common.cuh"

namespace {

constexpr int TPB = 256;
constexpr int CTILE = 2048;                         // compaction tile (8 items per thread)
constexpr unsigned long long DONE = 1ull << 63;     // propagation state: resolved
constexpr int ERR_ORDRHO_RANGE = 1, ERR_ORDRHO_PERM = 2, ERR_NNEIGH_RANGE = 4;

unsigned blocks_for(int64_t n, int per = TPB)
{
    int64_t b = (n + per - 1) / per;
    return (unsigned)(b < 1 ? 1 : b);
}

// Key for an ascending sort that yields MATLAB's sort(x, 'descend') on
// single data: NaN first (key 0), then larger first; -0 and +0 equal.
__device__ __forceinline__ uint32_t desc_key(float f)
{
    if (isnan(f)) return 0u;
    uint32_t u = __float_as_uint(f);
    if (f == 0.0f) u = 0u;
    const uint32_t ord = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return ~ord;
}

// Float total order as an unsigned integer (0 is below every non-NaN value).
__device__ __forceinline__ uint32_t ord_bits(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float ord_float(uint32_t o)
{
    if (o == 0u) return __uint_as_float(0x7fc00000u);     // every value NaN: max is NaN
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// ---------------------------------------------------------------------------
// sort_ normalisation

__global__ void k_rho_max(const float *__restrict__ rho, int64_t n, uint32_t *__restrict__ mx)
{
    uint32_t m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = rho[i];
        if (!isnan(v)) m = max(m, ord_bits(v));
    }
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(mx, m);
}

__global__ void k_rho_div(float *__restrict__ rho, int64_t n, const uint32_t *__restrict__ mx,
                          uint32_t *__restrict__ keys, int32_t *__restrict__ vals)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float r = __fdiv_rn(rho[i], ord_float(*mx));
    rho[i] = r;
    keys[i] = desc_key(r);
    vals[i] = (int32_t)i;
}

__global__ void k_to_ids(const int32_t *__restrict__ v, int64_t n, int64_t *__restrict__ out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int64_t)v[i] + 1;
}

// ---------------------------------------------------------------------------
// stable compaction of the peak indices (delta >= cut), ascending

__global__ void k_peak_count(const float *__restrict__ delta, int64_t n, float cut, int *__restrict__ bcount)
{
    const int64_t base = (int64_t)blockIdx.x * CTILE;
    int c = 0;
    for (int k = threadIdx.x; k < CTILE; k += TPB) {
        const int64_t i = base + k;
        c += (i < n && delta[i] >= cut);
    }
    typedef cub::BlockReduce<int, TPB> BR;
    __shared__ typename BR::TempStorage ts;
    const int tot = BR(ts).Sum(c);
    if (threadIdx.x == 0) bcount[blockIdx.x] = tot;
}

__global__ void k_peak_scatter(const float *__restrict__ delta, int64_t n, float cut,
                               const int *__restrict__ boff, int32_t *__restrict__ pk)
{
    const int64_t base = (int64_t)blockIdx.x * CTILE + (int64_t)threadIdx.x * (CTILE / TPB);
    bool f[CTILE / TPB];
    int c = 0;
#pragma unroll
    for (int k = 0; k < CTILE / TPB; ++k) {
        const int64_t i = base + k;
        f[k] = (i < n && delta[i] >= cut);
        c += f[k];
    }
    typedef cub::BlockScan<int, TPB> BS;
    __shared__ typename BS::TempStorage ts;
    int pre;
    BS(ts).ExclusiveSum(c, pre);
    int o = boff[blockIdx.x] + pre;
#pragma unroll
    for (int k = 0; k < CTILE / TPB; ++k)
        if (f[k]) pk[o++] = (int32_t)(base + k);
}

// ---------------------------------------------------------------------------
// peaks in descending rho order and the kNN-overlap bit matrix

__global__ void k_peak_keys(const float *__restrict__ rho, const int32_t *__restrict__ pk, int P,
                            uint32_t *__restrict__ keys)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P) keys[i] = desc_key(rho[pk[i]]);
}

__global__ void k_edges(const int64_t *__restrict__ miKnn, const int32_t *__restrict__ pks, int P, int knn,
                        int64_t *__restrict__ key, int32_t *__restrict__ col)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= (int64_t)P * knn) return;
    const int j = (int)(e / knn), k = (int)(e % knn);
    key[e] = miKnn[(int64_t)pks[j] * knn + k];
    col[e] = j;
}

__device__ __forceinline__ void set_bit(uint32_t *S, int W, int r, int c)
{
    atomicOr(&S[(size_t)r * W + (c >> 5)], 1u << (c & 31));
}

// Every pair of lists holding the same value: the value runs of the sorted
// (value, peak) pairs.  Thread p pairs its entry with the rest of its run.
__global__ void k_overlap(const int64_t *__restrict__ key, const int32_t *__restrict__ col, int64_t E,
                          uint32_t *__restrict__ S, int W)
{
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= E) return;
    const int64_t v = key[p];
    const int j = col[p];
    set_bit(S, W, j, j);
    for (int64_t q = p + 1; q < E && key[q] == v; ++q) {
        const int i = col[q];
        if (i != j) { set_bit(S, W, j, i); set_bit(S, W, i, j); }
    }
}

// popcount of each row (one warp per row)
__global__ void k_row_count(const uint32_t *__restrict__ S, int P, int W, int *__restrict__ cnt)
{
    const int r = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (r >= P) return;
    int c = 0;
    for (int w = lane; w < W; w += 32) c += __popc(S[(size_t)r * W + w]);
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) cnt[r] = c;
}

// ---------------------------------------------------------------------------
// one cell2map_ repeat

// U_i = S_i | OR over members m of S_i of S_m, for rows with more than one
// member; owner[m] = the largest such i whose union holds m (cvi_clu1(viClu1)
// = {viClu1} visits iClu ascending, so the last writer is the largest).
__global__ void k_union(const uint32_t *__restrict__ S, const int *__restrict__ cnt, int P, int W,
                        uint32_t *__restrict__ U, int *__restrict__ ucnt, int *__restrict__ owner)
{
    extern __shared__ uint32_t sm[];
    uint32_t *row = sm, *acc = sm + W;
    const int i = blockIdx.x;
    if (cnt[i] <= 1) {
        if (threadIdx.x == 0) ucnt[i] = 0;
        return;
    }
    const uint32_t *Si = S + (size_t)i * W;
    for (int w = threadIdx.x; w < W; w += blockDim.x) row[w] = acc[w] = Si[w];
    __syncthreads();
    for (int w0 = 0; w0 < W; ++w0) {
        uint32_t bits = row[w0];
        while (bits) {
            const int m = w0 * 32 + __ffs(bits) - 1;
            bits &= bits - 1;
            const uint32_t *Sm = S + (size_t)m * W;
            for (int w = threadIdx.x; w < W; w += blockDim.x) acc[w] |= Sm[w];
        }
    }
    int c = 0;
    uint32_t *Ui = U + (size_t)i * W;
    for (int w = threadIdx.x; w < W; w += blockDim.x) {
        uint32_t a = acc[w];
        Ui[w] = a;
        c += __popc(a);
        while (a) {
            atomicMax(&owner[w * 32 + __ffs(a) - 1], i);
            a &= a - 1;
        }
    }
    typedef cub::BlockReduce<int, 128> BR;
    __shared__ typename BR::TempStorage ts;
    const int tot = BR(ts).Sum(c);
    if (threadIdx.x == 0) ucnt[i] = tot;
}

// the new set sizes, and whether any differs from the old (the stop test)
__global__ void k_new_count(const int *__restrict__ owner, const int *__restrict__ ucnt,
                            const int *__restrict__ cnt, int P, int *__restrict__ ncnt, int *__restrict__ changed)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= P) return;
    const int o = owner[m];
    const int nc = o >= 0 ? ucnt[o] : 0;
    ncnt[m] = nc;
    if (nc != cnt[m]) atomicOr(changed, 1);
}

// cvi_clu = cvi_clu1: row m becomes its owner's union (empty without owner)
__global__ void k_gather(const int *__restrict__ owner, const uint32_t *__restrict__ U, int W,
                         uint32_t *__restrict__ S, int *__restrict__ cnt, const int *__restrict__ ncnt)
{
    const int m = blockIdx.x, o = owner[m];
    uint32_t *Sm = S + (size_t)m * W;
    if (o >= 0) {
        const uint32_t *Uo = U + (size_t)o * W;
        for (int w = threadIdx.x; w < W; w += blockDim.x) Sm[w] = Uo[w];
    } else {
        for (int w = threadIdx.x; w < W; w += blockDim.x) Sm[w] = 0u;
    }
    if (threadIdx.x == 0) cnt[m] = ncnt[m];
}

// viMapClu(i) = min(cvi{i}) (1-based) or i when empty; mark representatives
__global__ void k_row_min(const uint32_t *__restrict__ S, const int *__restrict__ cnt, int P, int W,
                          int *__restrict__ mapc, int *__restrict__ isrep)
{
    const int r = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (r >= P) return;
    int first = r;
    if (cnt[r] > 0) {
        for (int w0 = 0; w0 < W; w0 += 32) {
            const uint32_t v = (w0 + lane < W) ? S[(size_t)r * W + w0 + lane] : 0u;
            const unsigned nz = __ballot_sync(0xffffffffu, v != 0u);
            if (nz) {
                const int l = __ffs(nz) - 1;
                const uint32_t vw = __shfl_sync(0xffffffffu, v, l);
                first = (w0 + l) * 32 + __ffs(vw) - 1;
                break;
            }
        }
    }
    if (lane == 0) {
        mapc[r] = first + 1;
        isrep[first + 1] = 1;
    }
}

// peak labels (rank of the representative) and the centre list
__global__ void k_peak_labels(const int *__restrict__ mapc, const int *__restrict__ rank,
                              const int *__restrict__ isrep, const int32_t *__restrict__ pks, int P,
                              int32_t *__restrict__ viClu, int64_t *__restrict__ icl_tmp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    viClu[pks[i]] = rank[mapc[i]];
    if (isrep[i + 1]) icl_tmp[rank[i + 1] - 1] = (int64_t)pks[i] + 1;
}

__global__ void k_fill_i32(int32_t *__restrict__ a, int64_t n, int32_t v)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

// one cluster: every spike in it, centre ordrho(1)
__global__ void k_first_centre(const int64_t *__restrict__ ordrho, int64_t n, int64_t *__restrict__ icl_tmp,
                               int *__restrict__ err)
{
    const int64_t o = ordrho[0];
    if (o < 1 || o > n) atomicOr(err, ERR_ORDRHO_RANGE);
    icl_tmp[0] = o;
}

// ---------------------------------------------------------------------------
// label propagation along nneigh in ordrho order

__global__ void k_rank(const int64_t *__restrict__ ordrho, int64_t n, int32_t *__restrict__ rank,
                       int *__restrict__ err)
{
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int64_t o = ordrho[r];
    if (o < 1 || o > n) { atomicOr(err, ERR_ORDRHO_RANGE); return; }
    if (atomicExch(&rank[o - 1], (int32_t)r) != -1) atomicOr(err, ERR_ORDRHO_PERM);
}

__device__ __forceinline__ void count_warp(bool pred, int *ctr)
{
    const unsigned b = __ballot_sync(0xffffffffu, pred);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(ctr, __popc(b));
}

// The state of one pass: resolved spikes carry DONE | label; an unassigned
// spike whose nneigh is unassigned and ranked earlier points to that rank.
__global__ void k_pass_state(const int64_t *__restrict__ ordrho, const int64_t *__restrict__ nneigh,
                             const int32_t *__restrict__ rank, const int32_t *__restrict__ viClu, int64_t n,
                             unsigned long long *__restrict__ st, int *__restrict__ act, int *__restrict__ err,
                             int *__restrict__ lastbuf)
{
    const int64_t r0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r0 == 0) *lastbuf = 0;
    const int64_t r = r0 < n ? r0 : n - 1;
    unsigned long long w = DONE;
    const int64_t o = ordrho[r] - 1;
    if (o >= 0 && o < n) {
        const int32_t L = viClu[o];
        if (L > 0) {
            w = DONE | (uint32_t)L;
        } else {
            const int64_t nn = nneigh[o];
            if (nn < 1 || nn > n) {
                if (r0 < n) atomicOr(err, ERR_NNEIGH_RANGE);
            } else {
                const int32_t Ln = viClu[nn - 1];
                const int32_t t = rank[nn - 1];
                if (Ln > 0) w = DONE | (uint32_t)Ln;
                else if (t >= 0 && t < r) w = (unsigned long long)(uint32_t)t;
                // else: nneigh is visited later (or is the spike itself): label 0
            }
        }
    }
    if (r0 < n) st[r] = w;
    count_warp(r0 < n && !(w & DONE), &act[0]);
}

// One pointer-jumping round, src -> dst; returns at once when the previous
// round left nothing unresolved.
__global__ void k_jump(const unsigned long long *__restrict__ src, unsigned long long *__restrict__ dst,
                       int64_t n, int *__restrict__ act, int round, int *__restrict__ lastbuf, int dstbuf)
{
    if (act[round - 1] == 0) return;
    const int64_t r0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t r = r0 < n ? r0 : n - 1;
    unsigned long long w = src[r];
    // A resolved target hands over its label; an unresolved one its own
    // target: either way the new state is the target's state.
    if (!(w & DONE)) w = src[(uint32_t)w];
    if (r0 < n) dst[r] = w;
    count_warp(r0 < n && !(w & DONE), &act[round]);
    if (r0 == 0) *lastbuf = dstbuf;
}

__global__ void k_pass_finish(const unsigned long long *__restrict__ a, const unsigned long long *__restrict__ b,
                              const int *__restrict__ lastbuf, const int64_t *__restrict__ ordrho, int64_t n,
                              int32_t *__restrict__ viClu, int *__restrict__ zeros)
{
    const int64_t r0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t r = r0 < n ? r0 : n - 1;
    const unsigned long long w = (*lastbuf ? b : a)[r];
    const int32_t L = (w & DONE) ? (int32_t)(uint32_t)w : 0;
    const int64_t o = ordrho[r] - 1;
    if (r0 < n && o >= 0 && o < n) viClu[o] = L;
    count_warp(r0 < n && L <= 0, zeros);
}

// ---------------------------------------------------------------------------
// dpclus_remove_count_

constexpr int HIST_SMEM_MAX = 8192;

__global__ void k_hist(const int32_t *__restrict__ viClu, int64_t n, int nIcl, int *__restrict__ cnt)
{
    __shared__ int h[HIST_SMEM_MAX];
    const bool local = nIcl + 1 <= HIST_SMEM_MAX;
    if (local) {
        for (int c = threadIdx.x; c <= nIcl; c += blockDim.x) h[c] = 0;
        __syncthreads();
    }
    for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x; i0 < n; i0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = i0 + threadIdx.x;
        const int c = i < n ? viClu[i] : 0;
        const bool ok = (c >= 1 && c <= nIcl);
        if (local) {
            if (ok) atomicAdd(&h[c], 1);
        } else {
            const unsigned peers = __match_any_sync(0xffffffffu, ok ? c : 0);
            const int lead = __ffs(peers) - 1;
            if (ok && (int)(threadIdx.x & 31) == lead) atomicAdd(&cnt[c], __popc(peers));
        }
    }
    if (local) {
        __syncthreads();
        for (int c = threadIdx.x; c <= nIcl; c += blockDim.x)
            if (h[c]) atomicAdd(&cnt[c], h[c]);
    }
}

__global__ void k_keep(const int *__restrict__ cnt, int nIcl, int min_count, int *__restrict__ keep)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c <= nIcl) keep[c] = (c >= 1 && cnt[c] >= min_count) ? 1 : 0;
}

__global__ void k_remap(int32_t *__restrict__ viClu, int64_t n, int nIcl, const int *__restrict__ keep,
                        const int *__restrict__ newid)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = viClu[i];
    viClu[i] = (c >= 1 && c <= nIcl && keep[c]) ? newid[c] : 0;
}

__global__ void k_centres(const int64_t *__restrict__ icl_tmp, const int *__restrict__ cnt, int nIcl,
                          const int *__restrict__ keep, const int *__restrict__ newid, int64_t cap,
                          int64_t *__restrict__ icl, int32_t *__restrict__ vn)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (c > nIcl || !keep[c]) return;
    const int64_t o = newid[c] - 1;
    if (o < cap) {
        icl[o] = icl_tmp[c - 1];
        if (vn) vn[o] = cnt[c];
    }
}

}  // namespace

namespace {

// Device scratch of one call: stream-ordered allocations, released in stream
// order when the call returns.
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

template <class T>
cudaError_t read_back(T *h, const T *d, size_t n, cudaStream_t s)
{
    cudaError_t e = cudaMemcpyAsync(h, d, sizeof(T) * n, cudaMemcpyDeviceToHost, s);
    return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
}

template <class K, class V>
cudaError_t sort_pairs(Scratch &sc, const K *k0, K *k1, const V *v0, V *v1, int n)
{
    size_t tb = 0;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, tb, k0, k1, v0, v1, n, 0, (int)sizeof(K) * 8, sc.s);
    if (e != cudaSuccess) return e;
    void *tmp = sc.get<char>(tb);
    if (!tmp) return sc.err;
    return cub::DeviceRadixSort::SortPairs(tmp, tb, k0, k1, v0, v1, n, 0, (int)sizeof(K) * 8, sc.s);
}

cudaError_t inclusive_sum(Scratch &sc, const int *in, int *out, int n)
{
    size_t tb = 0;
    cudaError_t e = cub::DeviceScan::InclusiveSum(nullptr, tb, in, out, n, sc.s);
    if (e != cudaSuccess) return e;
    void *tmp = sc.get<char>(tb);
    if (!tmp) return sc.err;
    return cub::DeviceScan::InclusiveSum(tmp, tb, in, out, n, sc.s);
}

cudaError_t exclusive_sum(Scratch &sc, const int *in, int *out, int n)
{
    size_t tb = 0;
    cudaError_t e = cub::DeviceScan::ExclusiveSum(nullptr, tb, in, out, n, sc.s);
    if (e != cudaSuccess) return e;
    void *tmp = sc.get<char>(tb);
    if (!tmp) return sc.err;
    return cub::DeviceScan::ExclusiveSum(tmp, tb, in, out, n, sc.s);
}

constexpr int JUMP_BATCH = 8;      // pointer-jumping rounds between convergence checks
constexpr int JUMP_MAX = 32;       // 2^32 > any chain length

}  // namespace

#define IRC_TRY(expr, where)                                                \
    do {                                                                    \
        cudaError_t _e = (expr);                                            \
        if (_e != cudaSuccess) return irc_host::cuda_status(_e, where);     \
    } while (0)

extern "C" int irc_sort_rho(float *rho, int64_t *ordrho, int64_t nSpk, void *stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (nSpk < 0 || nSpk >= INT32_MAX || (nSpk > 0 && (!rho || !ordrho))) {
        irc_host::set_error("irc_sort_rho: need 0 <= nSpk < 2^31 and non-null rho, ordrho");
        return IRC_E_INVAL;
    }
    if (nSpk == 0) return IRC_OK;
    const int64_t n = nSpk;
    Scratch sc(s);
    uint32_t *mx = sc.get<uint32_t>(1), *k0 = sc.get<uint32_t>(n), *k1 = sc.get<uint32_t>(n);
    int32_t *v0 = sc.get<int32_t>(n), *v1 = sc.get<int32_t>(n);
    IRC_TRY(sc.err, "irc_sort_rho: scratch");
    IRC_TRY(cudaMemsetAsync(mx, 0, sizeof(uint32_t), s), "irc_sort_rho");
    const unsigned gmax = blocks_for(n) < 152u * 8u ? blocks_for(n) : 152u * 8u;
    k_rho_max<<<gmax, TPB, 0, s>>>(rho, n, mx);
    k_rho_div<<<blocks_for(n), TPB, 0, s>>>(rho, n, mx, k0, v0);
    IRC_TRY(sort_pairs(sc, k0, k1, v0, v1, (int)n), "irc_sort_rho: sort");
    k_to_ids<<<blocks_for(n), TPB, 0, s>>>(v1, n, ordrho);
    IRC_CHECK_LAUNCH("irc_sort_rho");
    return IRC_OK;
}

extern "C" int irc_assign_cluster_knn(int32_t *viClu, int64_t *icl, int32_t *vnSpk_clu, int64_t cap,
                                      int64_t *counts, const float *rho, const float *delta,
                                      const int64_t *ordrho, const int64_t *nneigh, const int64_t *miKnn,
                                      int knn, int64_t nSpk, float delta_cut, int min_count, void *stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (!counts || !viClu || !icl || !rho || !delta || !ordrho || !nneigh || !miKnn || cap < 0 || knn < 1 ||
        nSpk < 1 || nSpk >= INT32_MAX) {
        irc_host::set_error("irc_assign_cluster_knn: need 1 <= nSpk < 2^31, knn >= 1, cap >= 0 and non-null arrays");
        return IRC_E_INVAL;
    }
    const int64_t n = nSpk;
    Scratch sc(s);
    // hdr: [0] error bits, [1] stop test of a cell2map_ repeat, [2] unassigned count, [3] state buffer
    int *hdr = sc.get<int>(4);
    const int nb = (int)((n + CTILE - 1) / CTILE);
    int *bcount = sc.get<int>(nb), *boff = sc.get<int>(nb);
    IRC_TRY(sc.err, "irc_assign_cluster_knn: scratch");
    IRC_TRY(cudaMemsetAsync(hdr, 0, 4 * sizeof(int), s), "irc_assign_cluster_knn");

    // viSpk_peak = find(vrDelta_spk(:) >= delta_cut)
    k_peak_count<<<nb, TPB, 0, s>>>(delta, n, delta_cut, bcount);
    IRC_TRY(exclusive_sum(sc, bcount, boff, nb), "irc_assign_cluster_knn: scan");
    int tail[2] = {0, 0};
    IRC_TRY(read_back(&tail[0], boff + nb - 1, 1, s), "irc_assign_cluster_knn: peak count");
    IRC_TRY(read_back(&tail[1], bcount + nb - 1, 1, s), "irc_assign_cluster_knn: peak count");
    const int P = tail[0] + tail[1];
    counts[0] = 0;
    counts[1] = P;
    counts[2] = 0;
    if (P > IRC_CLUSTER_MAX_PEAKS) {
        irc_host::set_error("irc_assign_cluster_knn: %d peaks (delta >= %g), above IRC_CLUSTER_MAX_PEAKS = %d", P,
                            (double)delta_cut, IRC_CLUSTER_MAX_PEAKS);
        return IRC_E_UNSUPPORTED;
    }
    const int Pa = P > 0 ? P : 1;
    const int W = (Pa + 31) / 32;
    int32_t *pk = sc.get<int32_t>(Pa), *pks = sc.get<int32_t>(Pa);
    uint32_t *pkey0 = sc.get<uint32_t>(Pa), *pkey1 = sc.get<uint32_t>(Pa);
    int *cnt = sc.get<int>(Pa), *ncnt = sc.get<int>(Pa), *ucnt = sc.get<int>(Pa), *owner = sc.get<int>(Pa);
    int *mapc = sc.get<int>(Pa), *isrep = sc.get<int>(Pa + 1), *rankc = sc.get<int>(Pa + 1);
    int64_t *icl_tmp = sc.get<int64_t>(Pa);
    IRC_TRY(sc.err, "irc_assign_cluster_knn: scratch");
    int nUniq = 0;
    if (P > 0) {
        k_peak_scatter<<<nb, TPB, 0, s>>>(delta, n, delta_cut, boff, pk);
        // [vrRho_peak, ix_] = sort(vrRho_spk(viSpk_peak), 'descend')
        k_peak_keys<<<blocks_for(P), TPB, 0, s>>>(rho, pk, P, pkey0);
        IRC_TRY(sort_pairs(sc, pkey0, pkey1, pk, pks, P), "irc_assign_cluster_knn: peak sort");
        // cvi_peak{i}: peaks whose kNN lists share a value with peak i
        const int64_t E = (int64_t)P * knn;
        if (E >= INT32_MAX) {
            irc_host::set_error("irc_assign_cluster_knn: peaks x knn = %lld, above 2^31", (long long)E);
            return IRC_E_UNSUPPORTED;
        }
        uint32_t *S = sc.get<uint32_t>((size_t)P * W), *U = sc.get<uint32_t>((size_t)P * W);
        int64_t *ek0 = sc.get<int64_t>(E), *ek1 = sc.get<int64_t>(E);
        int32_t *ec0 = sc.get<int32_t>(E), *ec1 = sc.get<int32_t>(E);
        IRC_TRY(sc.err, "irc_assign_cluster_knn: peak matrices");
        IRC_TRY(cudaMemsetAsync(S, 0, sizeof(uint32_t) * (size_t)P * W, s), "irc_assign_cluster_knn");
        k_edges<<<blocks_for(E), TPB, 0, s>>>(miKnn, pks, P, knn, ek0, ec0);
        IRC_TRY(sort_pairs(sc, ek0, ek1, ec0, ec1, (int)E), "irc_assign_cluster_knn: list sort");
        k_overlap<<<blocks_for(E), TPB, 0, s>>>(ek1, ec1, E, S, W);
        k_row_count<<<blocks_for((int64_t)P * 32), TPB, 0, s>>>(S, P, W, cnt);
        // cell2map_: at most ten repeats, stop when no set size changes
        const size_t usmem = 2 * sizeof(uint32_t) * (size_t)W;
        if (usmem > 48 * 1024)
            IRC_TRY(cudaFuncSetAttribute(k_union, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)usmem),
                    "irc_assign_cluster_knn: union smem");
        for (int rep = 0; rep < 10; ++rep) {
            IRC_TRY(cudaMemsetAsync(owner, 0xff, sizeof(int) * (size_t)P, s), "irc_assign_cluster_knn");
            IRC_TRY(cudaMemsetAsync(hdr + 1, 0, sizeof(int), s), "irc_assign_cluster_knn");
            k_union<<<P, 128, usmem, s>>>(S, cnt, P, W, U, ucnt, owner);
            k_new_count<<<blocks_for(P), TPB, 0, s>>>(owner, ucnt, cnt, P, ncnt, hdr + 1);
            int changed = 0;
            IRC_TRY(read_back(&changed, hdr + 1, 1, s), "irc_assign_cluster_knn: cell2map_");
            if (!changed) break;
            k_gather<<<P, 128, 0, s>>>(owner, U, W, S, cnt, ncnt);
        }
        // viMapClu, viUniq_ and the compacted map
        IRC_TRY(cudaMemsetAsync(isrep, 0, sizeof(int) * (size_t)(P + 1), s), "irc_assign_cluster_knn");
        k_row_min<<<blocks_for((int64_t)P * 32), TPB, 0, s>>>(S, cnt, P, W, mapc, isrep);
        IRC_TRY(inclusive_sum(sc, isrep, rankc, P + 1), "irc_assign_cluster_knn: rank");
        IRC_TRY(read_back(&nUniq, rankc + P, 1, s), "irc_assign_cluster_knn: cluster count");
    }
    IRC_TRY(cudaMemsetAsync(viClu, 0, sizeof(int32_t) * (size_t)n, s), "irc_assign_cluster_knn");
    if (P > 0) k_peak_labels<<<blocks_for(P), TPB, 0, s>>>(mapc, rankc, isrep, pks, P, viClu, icl_tmp);

    int nIcl = nUniq;
    if (nUniq <= 1) {
        k_fill_i32<<<blocks_for(n), TPB, 0, s>>>(viClu, n, 1);
        k_first_centre<<<1, 1, 0, s>>>(ordrho, n, icl_tmp, hdr);
        nIcl = 1;
    } else {
        // ranks (ordrho must be a permutation), then at most ten passes
        int32_t *rank = sc.get<int32_t>(n);
        unsigned long long *stA = sc.get<unsigned long long>(n), *stB = sc.get<unsigned long long>(n);
        int *act = sc.get<int>(JUMP_MAX + 1);
        IRC_TRY(sc.err, "irc_assign_cluster_knn: propagation scratch");
        IRC_TRY(cudaMemsetAsync(rank, 0xff, sizeof(int32_t) * (size_t)n, s), "irc_assign_cluster_knn");
        k_rank<<<blocks_for(n), TPB, 0, s>>>(ordrho, n, rank, hdr);
        for (int pass = 0; pass < 10; ++pass) {
            IRC_TRY(cudaMemsetAsync(act, 0, sizeof(int) * (JUMP_MAX + 1), s), "irc_assign_cluster_knn");
            IRC_TRY(cudaMemsetAsync(hdr + 2, 0, sizeof(int), s), "irc_assign_cluster_knn");
            k_pass_state<<<blocks_for(n), TPB, 0, s>>>(ordrho, nneigh, rank, viClu, n, stA, act, hdr, hdr + 3);
            for (int round = 1; round <= JUMP_MAX; ++round) {
                const bool odd = round & 1;
                k_jump<<<blocks_for(n), TPB, 0, s>>>(odd ? stA : stB, odd ? stB : stA, n, act, round, hdr + 3,
                                                      odd ? 1 : 0);
                if (round % JUMP_BATCH == 0) {
                    int left = 0;
                    IRC_TRY(read_back(&left, act + round, 1, s), "irc_assign_cluster_knn: propagation");
                    if (left == 0) break;
                }
            }
            k_pass_finish<<<blocks_for(n), TPB, 0, s>>>(stA, stB, hdr + 3, ordrho, n, viClu, hdr + 2);
            int zeros = 0;
            IRC_TRY(read_back(&zeros, hdr + 2, 1, s), "irc_assign_cluster_knn: propagation");
            if (zeros == 0) break;
        }
    }
    counts[2] = nIcl;

    // dpclus_remove_count_
    int *ccnt = sc.get<int>(nIcl + 1), *keep = sc.get<int>(nIcl + 1), *newid = sc.get<int>(nIcl + 1);
    IRC_TRY(sc.err, "irc_assign_cluster_knn: count scratch");
    IRC_TRY(cudaMemsetAsync(ccnt, 0, sizeof(int) * (size_t)(nIcl + 1), s), "irc_assign_cluster_knn");
    const unsigned gh = blocks_for(n) < 152u * 4u ? blocks_for(n) : 152u * 4u;
    k_hist<<<gh, TPB, 0, s>>>(viClu, n, nIcl, ccnt);
    k_keep<<<blocks_for(nIcl + 1), TPB, 0, s>>>(ccnt, nIcl, min_count, keep);
    IRC_TRY(inclusive_sum(sc, keep, newid, nIcl + 1), "irc_assign_cluster_knn: keep scan");
    int nKeep = 0;
    IRC_TRY(read_back(&nKeep, newid + nIcl, 1, s), "irc_assign_cluster_knn: cluster count");
    if (nKeep < nIcl) k_remap<<<blocks_for(n), TPB, 0, s>>>(viClu, n, nIcl, keep, newid);
    k_centres<<<blocks_for(nIcl), TPB, 0, s>>>(icl_tmp, ccnt, nIcl, keep, newid, cap, icl, vnSpk_clu);
    counts[0] = nKeep;
    int err = 0;
    IRC_TRY(read_back(&err, hdr, 1, s), "irc_assign_cluster_knn");
    IRC_CHECK_LAUNCH("irc_assign_cluster_knn");
    if (err & ERR_ORDRHO_RANGE) {
        irc_host::set_error("irc_assign_cluster_knn: an ordrho entry is outside 1..nSpk");
        return IRC_E_INVAL;
    }
    if (err & ERR_ORDRHO_PERM) {
        irc_host::set_error("irc_assign_cluster_knn: ordrho is not a permutation of 1..nSpk");
        return IRC_E_INVAL;
    }
    if (err & ERR_NNEIGH_RANGE) {
        irc_host::set_error("irc_assign_cluster_knn: an nneigh entry of an unassigned spike is outside 1..nSpk");
        return IRC_E_INVAL;
    }
    if (nKeep > cap) {
        irc_host::set_error("irc_assign_cluster_knn: %d clusters, above cap = %lld", nKeep, (long long)cap);
        return IRC_E_INVAL;
    }
    return IRC_OK;
}
