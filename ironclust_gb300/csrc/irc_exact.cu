// irc_exact.cu -- EXACT-mode site kNN and the kNN-list delta.
//
// EXACT kNN: the true k nearest candidates (squared distance > 0, the irc2
// GPU convention) under the reference FP32 arithmetic, ordered by the key
// (d2 bits, index).  Two passes per query tile:
//   1. every thread keeps the minimum over a disjoint stripe of the linked
//      candidates (256 stripes); the k-th smallest stripe minimum tau bounds
//      the k-th neighbour distance from above (k distinct candidates lie at
//      or below it);
//   2. the stripes are rescanned and candidates with d2 <= tau are appended
//      to a per-query shared-memory list, which one warp sorts with a
//      bitonic network; the first k are the answer.
// A query whose list overflows (mass ties) is finished by a bounded
// fallback: k ordered scans, each taking the smallest key above the last.
//
// kNN-list delta: with the exact kNN list of every spike and rho for all of
// them, the nearest higher-rho spike is the first list entry whose rho
// exceeds the query's, whenever the list holds one (any closer higher-rho
// spike would rank earlier in the list).  Queries without one -- local
// density peaks -- go to a drift-window scan over all linked candidates.
#include <cstdio>
#include <mutex>

#include "irc_common.cuh"
#include "irc_plan.cuh"
#include "irc_scan.cuh"

namespace {

constexpr int kThreads = 256;     // = number of stripes
constexpr int kQB = 16;           // queries per CTA
constexpr int kCap = 256;         // list capacity per query
constexpr float kInfSentinel = IRC_SINGLE_INF_F;
constexpr int kQueueBlocks = 152 * 4;   // grid of the queue-draining kernels (8 warps per block)

__device__ __forceinline__ unsigned long long dkey(float d2, int idx)
{
    return ((unsigned long long)__float_as_uint(d2) << 32) | (unsigned)idx;
}

// Distance of candidate iB to QB staged queries (reference arithmetic).
template <int QB>
__device__ __forceinline__ void dist_qb(const float *__restrict__ fb, int nC, const float *sA,
                                        float (&acc)[QB])
{
#pragma unroll
    for (int q = 0; q < QB; ++q) acc[q] = 0.0f;
    for (int c = 0; c < nC; ++c) {
        const float bv = __ldg(fb + c);
        const float4 *a4 = reinterpret_cast<const float4 *>(sA + c * QB);
#pragma unroll
        for (int j = 0; j < QB / 4; ++j) {
            const float4 a = a4[j];
            acc[4 * j + 0] = irc::dterm(acc[4 * j + 0], bv, a.x);
            acc[4 * j + 1] = irc::dterm(acc[4 * j + 1], bv, a.y);
            acc[4 * j + 2] = irc::dterm(acc[4 * j + 2], bv, a.z);
            acc[4 * j + 3] = irc::dterm(acc[4 * j + 3], bv, a.w);
        }
    }
}

// Walk this thread's stripe (list positions p = t, t+256, ...) of the
// concatenated runs r0..r1-1, calling f(candidate index).
template <class Fn>
__device__ __forceinline__ void walk_stripe(const irc::PlanDev &p, int r0, int r1, int t, Fn f)
{
    int pos = 0;                                   // list position of the run start
    for (int r = r0; r < r1; ++r) {
        const int rs = __ldg(p.rs + r), rn = __ldg(p.rn + r);
        int first = (t - pos) % kThreads;
        if (first < 0) first += kThreads;
        for (int i = first; i < rn; i += kThreads) f(rs + i);
        pos += rn;
    }
}

// Warp-wide ascending bitonic sort of kCap 64-bit keys in shared memory.
__device__ __forceinline__ void warp_sort_keys(unsigned long long *keys, int lane)
{
    constexpr int PER = kCap / 32;
    unsigned long long v[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) v[i] = keys[lane * PER + i];   // element id = lane*PER + i
    // bitonic over element ids e in [0, kCap)
#pragma unroll
    for (int size = 2; size <= kCap; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= PER) {
                const int lstride = stride / PER;
#pragma unroll
                for (int i = 0; i < PER; ++i) {
                    const int e = lane * PER + i;
                    const unsigned long long o = __shfl_xor_sync(0xffffffffu, v[i], lstride);
                    const bool up = ((e & size) == 0);
                    const bool lower = ((e & stride) == 0);
                    const bool keep_min = (lower == up);
                    v[i] = keep_min ? (o < v[i] ? o : v[i]) : (o > v[i] ? o : v[i]);
                }
            } else {
#pragma unroll
                for (int i = 0; i < PER; ++i) {
                    const int j = i ^ stride;
                    if (j > i) {
                        const int e = lane * PER + i;
                        const bool up = ((e & size) == 0);
                        const unsigned long long a = v[i], b = v[j];
                        const bool swap = up ? (a > b) : (a < b);
                        v[i] = swap ? b : a;
                        v[j] = swap ? a : b;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < PER; ++i) keys[lane * PER + i] = v[i];
}

__global__ void __launch_bounds__(kThreads)
k_site_knn_exact(irc::PlanDev p, const float *__restrict__ F, int nC, int knn,
                 float *__restrict__ vrKnn, float *__restrict__ rho, int *__restrict__ miKnn,
                 float *__restrict__ d2Knn, int *__restrict__ ovf_count, int *__restrict__ ovf_list)
{
    __shared__ __align__(16) float sA[IRC_NC_MAX * kQB];
    __shared__ float sTau[kQB];
    __shared__ int sCnt[kQB];
    extern __shared__ __align__(16) unsigned char dyn[];
    unsigned long long *sList = reinterpret_cast<unsigned long long *>(dyn);   // [kQB][kCap]
    float *sMin = reinterpret_cast<float *>(sList + kQB * kCap);              // [kQB][kThreads]
    int chunk, qs, n;
    irc::tile_lookup<kQB>(p, blockIdx.x, chunk, qs, n);
    const int r0 = __ldg(p.roff + chunk), r1 = __ldg(p.roff + chunk + 1);
    irc::stage_queries<kQB>(F, nC, qs, n, sA);
    if (threadIdx.x < kQB) sCnt[threadIdx.x] = 0;
    __syncthreads();
    const int t = threadIdx.x;
    // pass 1: stripe minima
    float mn[kQB];
#pragma unroll
    for (int q = 0; q < kQB; ++q) mn[q] = __int_as_float(0x7f800000);
    walk_stripe(p, r0, r1, t, [&](int iB) {
        float acc[kQB];
        dist_qb<kQB>(F + (size_t)iB * nC, nC, sA, acc);
#pragma unroll
        for (int q = 0; q < kQB; ++q)
            if (acc[q] > 0.0f && acc[q] < mn[q]) mn[q] = acc[q];
    });
#pragma unroll
    for (int q = 0; q < kQB; ++q) sMin[q * kThreads + t] = mn[q];
    __syncthreads();
    // tau = k-th smallest stripe minimum (by value); +inf if fewer than k finite
    const int lane = t & 31, warp = t >> 5, nw = kThreads / 32;
    for (int q = warp; q < kQB; q += nw) {
        float *m = sMin + q * kThreads;
        float kth = __int_as_float(0x7f800000);
        for (int k = 0; k < knn; ++k) {
            unsigned long long best = ~0ull;
            for (int s = lane; s < kThreads; s += 32) {
                const unsigned long long key = dkey(m[s], s);
                best = key < best ? key : best;
            }
            best = irc::warp_min_u64(best);
            const int s = (int)(best & 0xffffffffu);
            kth = __uint_as_float((unsigned)(best >> 32));
            __syncwarp();
            if (lane == 0) m[s] = __int_as_float(0x7fffffff);      // NaN bits: sorts last
            __syncwarp();
            if (!(kth < __int_as_float(0x7f800000))) break;
        }
        if (lane == 0) sTau[q] = kth;
    }
    __syncthreads();
    // pass 2: collect d2 <= tau
    walk_stripe(p, r0, r1, t, [&](int iB) {
        float acc[kQB];
        dist_qb<kQB>(F + (size_t)iB * nC, nC, sA, acc);
#pragma unroll
        for (int q = 0; q < kQB; ++q)
            if (acc[q] > 0.0f && acc[q] <= sTau[q]) {
                const int slot = atomicAdd(&sCnt[q], 1);
                if (slot < kCap) sList[q * kCap + slot] = dkey(acc[q], iB);
            }
    });
    __syncthreads();
    for (int q = warp; q < n; q += nw) {
        const int cnt = sCnt[q];
        const size_t o = (size_t)(qs + q - p.q_base);
        if (cnt > kCap) {                          // overflow: finished by the fallback kernel
            if (lane == 0) { int i = atomicAdd(ovf_count, 1); ovf_list[i] = qs + q; }
            continue;
        }
        unsigned long long *L = sList + q * kCap;
        for (int i = cnt + lane; i < kCap; i += 32) L[i] = ~0ull;
        __syncwarp();
        warp_sort_keys(L, lane);
        __syncwarp();
        for (int k = lane; k < knn; k += 32) {
            const unsigned long long key = L[k];
            const bool ok = k < cnt;
            const float d2 = ok ? __uint_as_float((unsigned)(key >> 32)) : kInfSentinel;
            const int idx = ok ? (int)(key & 0xffffffffu) : qs + q;
            miKnn[(size_t)k + (size_t)knn * o] = idx + 1;
            if (d2Knn) d2Knn[(size_t)k + (size_t)knn * o] = d2;
            if (k == knn - 1) {
                const float v = irc::ref_sqrt_abs(d2);
                vrKnn[o] = v;
                if (rho) rho[o] = __fdiv_rn(1.0f, v);
            }
        }
        __syncwarp();
    }
}

// One CTA per queued query: k ordered scans of all linked candidates, each a
// block-wide minimum of the keys above the previous one.  Serves the rare
// queries whose candidate list overflowed (mass ties, or an unlucky spread of
// the tensor-core filter's list parts).
__global__ void __launch_bounds__(kThreads)
k_exact_overflow(irc::PlanDev p, const float *__restrict__ F, int nC, int knn,
                 const int *__restrict__ ovf_count, const int *__restrict__ ovf_list,
                 float *__restrict__ vrKnn, float *__restrict__ rho,
                 int *__restrict__ miKnn, float *__restrict__ d2Knn)
{
    __shared__ unsigned long long red[kThreads / 32];
    __shared__ unsigned long long sBest;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = *ovf_count;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        const int q = ovf_list[w];
        int lo = 0, hi = p.nChunks;
        while (hi - lo > 1) { int mid = (lo + hi) >> 1; if (__ldg(p.q0 + mid) <= q) lo = mid; else hi = mid; }
        const int r0 = __ldg(p.roff + lo), r1 = __ldg(p.roff + lo + 1);
        const float *a = F + (size_t)q * nC;
        const size_t o = (size_t)(q - p.q_base);
        unsigned long long prev = 0;
        bool have_prev = false;
        for (int k = 0; k < knn; ++k) {
            unsigned long long best = ~0ull;
            walk_stripe(p, r0, r1, threadIdx.x, [&](int iB) {
                const float *b = F + (size_t)iB * nC;
                float acc = 0.0f;
                for (int c = 0; c < nC; ++c) acc = irc::dterm(acc, __ldg(b + c), __ldg(a + c));
                if (!(acc > 0.0f) || !(acc < kInfSentinel)) return;
                const unsigned long long key = dkey(acc, iB);
                if ((!have_prev || key > prev) && key < best) best = key;
            });
            best = irc::warp_min_u64(best);
            if (lane == 0) red[warp] = best;
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned long long b = red[0];
                for (int i = 1; i < kThreads / 32; ++i) b = red[i] < b ? red[i] : b;
                sBest = b;
                const bool ok = b != ~0ull;
                const float d2 = ok ? __uint_as_float((unsigned)(b >> 32)) : kInfSentinel;
                const int idx = ok ? (int)(b & 0xffffffffu) : q;
                miKnn[(size_t)k + (size_t)knn * o] = idx + 1;
                if (d2Knn) d2Knn[(size_t)k + (size_t)knn * o] = d2;
                if (k == knn - 1) {
                    const float v = irc::ref_sqrt_abs(d2);
                    vrKnn[o] = v;
                    if (rho) rho[o] = __fdiv_rn(1.0f, v);
                }
            }
            __syncthreads();
            best = sBest;
            if (best != ~0ull) { prev = best; have_prev = true; }
        }
    }
}

// delta from the kNN list; queries without a higher-rho list entry are queued.
__global__ void k_delta_list(irc::PlanDev p, const float *__restrict__ R, int knn,
                             const int *__restrict__ miKnn, const float *__restrict__ d2Knn,
                             float *__restrict__ delta, int *__restrict__ nneigh,
                             int *__restrict__ fb_flag)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= p.n_out) return;
    const int q = o + p.q_base;
    const float rq = __ldg(R + q);
    const int *mi = miKnn + (size_t)knn * o;
    const float *dk = d2Knn + (size_t)knn * o;
    int miss = 1;
    for (int k = 0; k < knn; ++k) {
        const float d2 = __ldg(dk + k);
        if (!(d2 < kInfSentinel)) break;                 // list exhausted
        const int j = __ldg(mi + k) - 1;
        if (!(__ldg(R + j) <= rq)) {                     // reference mask: rb <= ra is excluded
            delta[o] = __fmul_rn(irc::ref_sqrt_abs(d2), rq);
            nneigh[o] = j + 1;
            miss = 0;
            break;
        }
    }
    fb_flag[o] = miss;
}

// One CTA per chunk: compact the chunk's flagged queries (in order) into the
// chunk's own segment of fb_list, then claim the (16-query tile, part) units
// of the fallback scan: unit = {chunk | part << 28, (first << 5) | count}.
constexpr int kParts = 8;        // most parts of one candidate window (part < 2^3: 3 bits at bit 28)
constexpr int kMinPart = 2048;   // fewest candidates of a part

__global__ void __launch_bounds__(kThreads)
k_delta_compact(irc::PlanDev p, const int *__restrict__ fb_flag, int *__restrict__ fb_list,
                int *__restrict__ n_items, int2 *__restrict__ items, unsigned long long *__restrict__ keys)
{
    __shared__ int wsum[kThreads / 32];
    __shared__ int running, base;
    const int chunk = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int q0 = __ldg(p.q0 + chunk), nq = __ldg(p.nq + chunk), seg = q0 - p.q_base;
    if (threadIdx.x == 0) running = 0;
    __syncthreads();
    for (int start = 0; start < nq; start += kThreads) {
        const int i = start + threadIdx.x;
        const int f = i < nq ? fb_flag[seg + i] : 0;
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        if (lane == 0) wsum[warp] = __popc(bal);
        __syncthreads();
        int off = running;
        for (int w = 0; w < warp; ++w) off += wsum[w];
        if (f) {
            fb_list[seg + off + __popc(bal & ((1u << lane) - 1u))] = q0 + i;
            keys[seg + i] = ~0ull;
        }
        __syncthreads();
        if (threadIdx.x == 0) for (int w = 0; w < kThreads / 32; ++w) running += wsum[w];
        __syncthreads();
    }
    const int total = running, ntile = (total + kQB - 1) / kQB;
    // a long candidate window is split into np parts of at least kMinPart
    const int np = min(kParts, max(1, __ldg(p.ncand + chunk) / kMinPart)), nunit = ntile * np;
    if (threadIdx.x == 0) base = nunit ? atomicAdd(n_items, nunit) : 0;
    __syncthreads();
    for (int j = threadIdx.x; j < nunit; j += kThreads) {
        const int t = j / np, part = j - t * np;
        items[base + j] = make_int2(chunk | (part << 28), ((t * kQB) << 5) | min(kQB, total - t * kQB));
    }
}

// Drift-window fallback for the queued queries, one unit per (16-query tile
// of a chunk, part of its candidate window; long windows have up to kParts
// parts of at least kMinPart candidates): a unit loads every candidate of its
// part once for the 16 queries, keeps per
// query the candidates whose rho exceeds the query's (the search_delta_drift
// mask), ties by (d2, index), and folds its best key into the query's key
// with a 64-bit atomicMin -- the minimum of the same keys in any order, so
// the split changes no result while giving the SMs kParts times more units
// (a probe holds ~1,000 fallback tiles per site, too few to fill 152 SMs
// when each scans a whole ~30K-candidate window).

__global__ void __launch_bounds__(kThreads)
k_delta_tiles(irc::PlanDev p, const float *__restrict__ F, const float *__restrict__ R, int nC,
              const uint8_t *__restrict__ row_dims, const int *__restrict__ n_items, const int2 *__restrict__ items,
              const int *__restrict__ fb_list, unsigned long long *__restrict__ keys)
{
    __shared__ __align__(16) float sA[IRC_NC_MAX * kQB];
    __shared__ float sRA[kQB];
    __shared__ int sQ[kQB];
    __shared__ unsigned long long red[kQB][kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int total = *n_items;
    for (int u = blockIdx.x; u < total; u += gridDim.x) {
        const int2 item = items[u];
        const int chunk = item.x & 0x0fffffff, part = item.x >> 28, first = item.y >> 5, n = item.y & 31;
        const int ntot = __ldg(p.ncand + chunk);
        const int np = min(kParts, max(1, ntot / kMinPart));
        const int r0 = __ldg(p.roff + chunk), r1 = __ldg(p.roff + chunk + 1);
        const int seg = __ldg(p.q0 + chunk) - p.q_base;
        // features that can be non-zero for this chunk's queries and candidates
        // (their site's width, irc_plan_set_site_dims): the rest add exactly 0
        const int nd = row_dims ? min(nC, (int)__ldg(row_dims + __ldg(p.q0 + chunk))) : nC;
        if (threadIdx.x < kQB) {
            const int q = fb_list[seg + first + min((int)threadIdx.x, n - 1)];
            sQ[threadIdx.x] = q;
            sRA[threadIdx.x] = __ldg(R + q);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nd * kQB; i += kThreads) {
            const int c = i / kQB, q = i - c * kQB;
            sA[i] = __ldg(F + (size_t)sQ[q] * nC + c);
        }
        __syncthreads();
        unsigned long long best[kQB];
#pragma unroll
        for (int q = 0; q < kQB; ++q) best[q] = ~0ull;
        const int per = (ntot + np - 1) / np, lo = part * per, hi = min(ntot, lo + per);
        int pos = 0;                                         // position of run r's first candidate
        for (int r = r0; r < r1 && pos < hi; ++r) {
            const int rs = __ldg(p.rs + r), rn = __ldg(p.rn + r);
            const int a = max(lo - pos, 0), b = min(hi - pos, rn);
            for (int i = a + (int)threadIdx.x; i < b; i += kThreads) {
                const int iB = rs + i;
                const float rb = __ldg(R + iB);
                unsigned live = 0;
#pragma unroll
                for (int q = 0; q < kQB; ++q)
                    if (!(rb <= sRA[q])) live |= 1u << q;
                if (!live) continue;
                float acc[kQB];
                dist_qb<kQB>(F + (size_t)iB * nC, nd, sA, acc);
#pragma unroll
                for (int q = 0; q < kQB; ++q)
                    if (((live >> q) & 1u) && acc[q] > 0.0f && acc[q] < kInfSentinel) {
                        const unsigned long long key = dkey(acc[q], iB);
                        best[q] = key < best[q] ? key : best[q];
                    }
            }
            pos += rn;
        }
#pragma unroll
        for (int q = 0; q < kQB; ++q) {
            const unsigned long long b = irc::warp_min_u64(best[q]);
            if (lane == 0) red[q][warp] = b;
        }
        __syncthreads();
        if (threadIdx.x < n) {
            unsigned long long b = red[threadIdx.x][0];
            for (int w = 1; w < kThreads / 32; ++w) b = red[threadIdx.x][w] < b ? red[threadIdx.x][w] : b;
            if (b != ~0ull) atomicMin(keys + (sQ[threadIdx.x] - p.q_base), b);
        }
        __syncthreads();
    }
}

// delta and nneigh of the queued queries from their keys (no candidate:
// sqrt(SINGLE_INF) .* rho and the query itself, as search_delta_drift_).
__global__ void k_delta_finish(irc::PlanDev p, const float *__restrict__ R, const int *__restrict__ n_items,
                               const int2 *__restrict__ items, const int *__restrict__ fb_list,
                               const unsigned long long *__restrict__ keys, float *__restrict__ delta,
                               int *__restrict__ nneigh)
{
    const int total = *n_items * kQB;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int2 item = items[t / kQB];
        const int j = t - (t / kQB) * kQB;
        const int chunk = item.x & 0x0fffffff, first = item.y >> 5, n = item.y & 31;
        if ((item.x >> 28) != 0 || j >= n) continue;        // each tile once (its part 0)
        const int qq = fb_list[__ldg(p.q0 + chunk) - p.q_base + first + j];
        const size_t o = (size_t)(qq - p.q_base);
        const unsigned long long b = keys[o];
        const bool ok = b != ~0ull;
        const float d2 = ok ? __uint_as_float((unsigned)(b >> 32)) : kInfSentinel;
        delta[o] = __fmul_rn(irc::ref_sqrt_abs(d2), __ldg(R + qq));
        nneigh[o] = (ok ? (int)(b & 0xffffffffu) : qq) + 1;
    }
}

}  // namespace

// Plan-owned scratch: two counters and two query lists of n_out entries.
static int irc_plan_scratch(irc_plan *pl, int **counters, int **list_a, int **list_b)
{
    *counters = pl->scratch;
    *list_a = pl->scratch + irc::kScratchLists;
    *list_b = pl->scratch + irc::kScratchLists + pl->dev.n_out;
    return IRC_OK;
}

int irc_site_knn_exact(irc_plan *pl, const float *F, int nC, int knn, float *vrKnn, float *rho,
                       int32_t *miKnn, float *d2Knn, cudaStream_t s)
{
    if (knn > kCap / 2) { irc_host::set_error("irc_site_knn(EXACT): knn %d > %d", knn, kCap / 2); return IRC_E_INVAL; }
    int *cnt, *la, *lb;
    int rc = irc_plan_scratch(pl, &cnt, &la, &lb);
    if (rc != IRC_OK) return rc;
    cudaError_t e = cudaMemsetAsync(cnt, 0, 2 * sizeof(int), s);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(EXACT): memset");
    const size_t smem = (size_t)kQB * kCap * 8 + (size_t)kQB * kThreads * 4;
    e = cudaFuncSetAttribute(k_site_knn_exact, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(EXACT): smem attribute");
    const int tiles = pl->ntiles[irc::tile_slot(kQB)];
    k_site_knn_exact<<<tiles, kThreads, smem, s>>>(pl->dev, F, nC, knn, vrKnn, rho, miKnn, d2Knn, cnt, la);
    IRC_CHECK_LAUNCH("irc_site_knn(EXACT)");
    // the overflow list is usually empty; size the grid for the worst case
    k_exact_overflow<<<kQueueBlocks, 256, 0, s>>>(
        pl->dev, F, nC, knn, cnt, la, vrKnn, rho, miKnn, d2Knn);
    IRC_CHECK_LAUNCH("irc_site_knn(EXACT) overflow");
    return IRC_OK;
}

int irc_site_delta_list(irc_plan *pl, const float *F, int nC, const float *R, int knn,
                        const int32_t *miKnn, const float *d2Knn, float *delta, int32_t *nneigh,
                        cudaStream_t s)
{
    int *cnt, *la, *lb;
    int rc = irc_plan_scratch(pl, &cnt, &la, &lb);
    if (rc != IRC_OK) return rc;
    // flags in list a, compacted queries in list b, (chunk, tile) items after them
    int *n_items = cnt + irc::kScratchItems;
    int2 *items = reinterpret_cast<int2 *>(lb + pl->dev.n_out);
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(
        lb + pl->dev.n_out + 16 * ((size_t)pl->dev.n_out / 16 + pl->dev.nChunks + 1));
    cudaError_t e = cudaMemsetAsync(n_items, 0, sizeof(int), s);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_delta: memset");
    const int n = pl->dev.n_out;
    k_delta_list<<<(n + 255) / 256, 256, 0, s>>>(pl->dev, R, knn, miKnn, d2Knn, delta, nneigh, la);
    IRC_CHECK_LAUNCH("irc_site_delta list");
    k_delta_compact<<<pl->dev.nChunks, kThreads, 0, s>>>(pl->dev, la, lb, n_items, items, keys);
    IRC_CHECK_LAUNCH("irc_site_delta compact");
    k_delta_tiles<<<kQueueBlocks, kThreads, 0, s>>>(pl->dev, F, R, nC, pl->row_dims, n_items, items, lb, keys);
    IRC_CHECK_LAUNCH("irc_site_delta tiles");
    k_delta_finish<<<kQueueBlocks, kThreads, 0, s>>>(pl->dev, R, n_items, items, lb, keys, delta, nneigh);
    IRC_CHECK_LAUNCH("irc_site_delta finish");
    return IRC_OK;
}

// Finish the queries the tensor-core kernel queued (list overflow) with the
// exact ordered-scan kernel; the queue is the plan's first scratch list.
int irc_exact_overflow_drain(irc_plan *pl, const float *F, int nC, int knn, float *vrKnn, float *rho,
                             int32_t *miKnn, float *d2Knn, cudaStream_t s)
{
    int *cnt, *la, *lb;
    irc_plan_scratch(pl, &cnt, &la, &lb);
    k_exact_overflow<<<kQueueBlocks, 256, 0, s>>>(pl->dev, F, nC, knn, cnt, la, vrKnn, rho, miKnn, d2Knn);
    IRC_CHECK_LAUNCH("irc_site_knn overflow drain");
    return IRC_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the EXACT site kNN (irc_site_knn_exact_noalloc).
//
// For callers that cannot call cudaMalloc: everything the kernels need
// besides the caller's inputs and outputs -- the device copy of the plan,
// the tile table, the overflow queue and its counter -- lives in the fixed
// array below, which every GPU that loads the library holds until the
// process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocWords = (size_t)2 << 20;     // 8 MiB of int32 words
static __device__ __align__(256) int32_t g_noalloc_scratch[kNoAllocWords];

// Device address of g_noalloc_scratch per device, looked up once per device
// with that device current (a host-side reference to the array is only a
// stand-in, not a device address).  The address belongs to the device's
// primary context: cudaDeviceReset destroys that context and the array with
// it, so a process that resets a device must not call the entry point on that
// device afterwards (the cached address would be stale).
constexpr int kMaxDevices = 64;
int32_t *g_noalloc_ptr[kMaxDevices];
std::mutex g_noalloc_mu;

int noalloc_scratch(int32_t **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn_exact_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) {
        irc_host::set_error("irc_site_knn_exact_noalloc: device %d out of range", dev);
        return IRC_E_INVAL;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn_exact_noalloc: cudaGetSymbolAddress");
        g_noalloc_ptr[dev] = (int32_t *)p;
    }
    *out = g_noalloc_ptr[dev];
    return IRC_OK;
}

// Word offsets of everything the entry point keeps in the fixed array, in
// order: the plan scratch words (queue counters), two query queues of n_out,
// q0 [nChunks], nq [nChunks], roff [nChunks+1], rs [nRuns], rn [nRuns] and
// the 16-query tile table [nChunks+1].  The size check and the pointers both
// come from here, so they cannot disagree.
struct NoAllocLayout {
    size_t q0, nq, roff, rs, rn, tile, total;
};

NoAllocLayout noalloc_layout(long long n_out, long long nChunks, long long nRuns)
{
    NoAllocLayout L;
    L.q0 = (size_t)irc::kScratchLists + 2 * (size_t)n_out;
    L.nq = L.q0 + (size_t)nChunks;
    L.roff = L.nq + (size_t)nChunks;
    L.rs = L.roff + (size_t)nChunks + 1;
    L.rn = L.rs + (size_t)nRuns;
    L.tile = L.rn + (size_t)nRuns;
    L.total = L.tile + (size_t)nChunks + 1;
    return L;
}

// tile_off[i] = sum_{j<i} ceil(nq[j] / QB), one block, chunked scan.
__global__ void k_noalloc_tiles(const int32_t *__restrict__ nq, int nChunks, int qb, int32_t *__restrict__ tile_off)
{
    __shared__ int32_t part[1024];
    const int t = threadIdx.x, nt = blockDim.x;
    const int per = (nChunks + nt - 1) / nt;
    const int lo = min(t * per, nChunks), hi = min(lo + per, nChunks);
    int32_t s = 0;
    for (int i = lo; i < hi; ++i) s += (nq[i] + qb - 1) / qb;
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        int32_t acc = 0;
        for (int i = 0; i < nt; ++i) { const int32_t v = part[i]; part[i] = acc; acc += v; }
    }
    __syncthreads();
    int32_t acc = part[t];
    for (int i = lo; i < hi; ++i) { tile_off[i] = acc; acc += (nq[i] + qb - 1) / qb; }
    if (hi == nChunks && lo < hi) tile_off[nChunks] = acc;
    if (nChunks == 0 && t == 0) tile_off[0] = 0;
}

}  // namespace

extern "C" int irc_site_knn_exact_noalloc(const float *F, int nC, const int32_t *q0, const int32_t *nq,
                                          const int32_t *roff, const int32_t *rs, const int32_t *rn, int nChunks,
                                          int q_base, int n_out, int nF, int knn, float *vrKnn, float *rho,
                                          int32_t *miKnn, float *d2Knn, void *stream)
{
    const char *me = "irc_site_knn_exact_noalloc";
    if (!F || !vrKnn || !miKnn) {
        irc_host::set_error("%s: null pointer", me);
        return IRC_E_INVAL;
    }
    if (nC > IRC_NC_MAX) { irc_host::set_error("%s: nC=%d > %d", me, nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || knn <= 0 || knn > kCap / 2) { irc_host::set_error("%s: bad nC=%d / knn=%d", me, nC, knn); return IRC_E_INVAL; }
    // the same checks as irc_plan_create (64-bit bounds)
    int rc = irc_host::check_plan(me, q0, nq, roff, rs, rn, nChunks, q_base, n_out, nF, nullptr, nullptr);
    if (rc != IRC_OK) return rc;
    const int nRuns = roff[nChunks];
    const NoAllocLayout L = noalloc_layout(n_out, nChunks, nRuns);
    if (L.total > kNoAllocWords) {
        irc_host::set_error("%s: plan needs %zu scratch words (4 + 2*n_out + 4*chunks + 2 + 2*runs), "
                            "the fixed array holds %zu", me, L.total, kNoAllocWords);
        return IRC_E_INVAL;
    }
    long long tiles = 0;
    for (int i = 0; i < nChunks; ++i) tiles += (nq[i] + kQB - 1) / kQB;
    int32_t *base = nullptr;
    rc = noalloc_scratch(&base);
    if (rc != IRC_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int32_t *d_q0 = base + L.q0, *d_nq = base + L.nq, *d_roff = base + L.roff;
    int32_t *d_rs = base + L.rs, *d_rn = base + L.rn, *d_tile = base + L.tile;
    cudaError_t e = cudaMemsetAsync(base, 0, irc::kScratchLists * sizeof(int32_t), s);    // counters start at zero
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_q0, q0, 4 * (size_t)nChunks, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_nq, nq, 4 * (size_t)nChunks, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_roff, roff, 4 * ((size_t)nChunks + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rs, rs, 4 * (size_t)nRuns, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rn, rn, 4 * (size_t)nRuns, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn_exact_noalloc: upload");
    k_noalloc_tiles<<<1, 1024, 0, s>>>(d_nq, nChunks, kQB, d_tile);
    IRC_CHECK_LAUNCH("irc_site_knn_exact_noalloc tiles");
    irc::PlanDev p;
    p.q0 = d_q0; p.nq = d_nq; p.roff = d_roff; p.rs = d_rs; p.rn = d_rn;
    p.roffr = d_roff; p.rsr = d_rs; p.rnr = d_rn;         // the EXACT kernels take any run split
    for (int k = 0; k < irc::kNumTileSizes; ++k) p.tile_off[k] = d_tile;     // only the 16-query table is read
    p.ncand = nullptr;                                    // read only by the delta kernels
    p.tc_toff = nullptr;                                  // read only by the tensor-core filter
    p.tc_tiles = nullptr;
    p.nChunks = nChunks; p.q_base = q_base; p.n_out = n_out; p.nF = nF; p.nRuns = nRuns;
    const size_t smem = (size_t)kQB * kCap * 8 + (size_t)kQB * kThreads * 4;
    e = cudaFuncSetAttribute(k_site_knn_exact, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn_exact_noalloc: smem attribute");
    int32_t *cnt = base, *queue = base + irc::kScratchLists;
    k_site_knn_exact<<<(unsigned)tiles, kThreads, smem, s>>>(p, F, nC, knn, vrKnn, rho, miKnn, d2Knn, cnt, queue);
    IRC_CHECK_LAUNCH("irc_site_knn_exact_noalloc");
    k_exact_overflow<<<kQueueBlocks, 256, 0, s>>>(p, F, nC, knn, cnt, queue, vrKnn, rho, miKnn, d2Knn);
    IRC_CHECK_LAUNCH("irc_site_knn_exact_noalloc overflow");
    return IRC_OK;
}
