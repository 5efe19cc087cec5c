// irc_tc.cu -- tensor-core (tcgen05) site kNN: BF16 distance filter, exact
// FP32 re-rank, FP64 at the k-th-neighbour boundary.
//
// Per CTA: 128 queries of one drift chunk (TMEM lanes) against every linked
// candidate, in 128-candidate tiles (TMEM columns, two accumulator
// buffers).  The BF16 operand rows (see irc_tc_host.cu) make every
// accumulator the approximate squared distance.  Warp roles: warp 0 issues
// TMA loads (4-stage ring), warp 1 owns TMEM and issues tcgen05.mma from one
// thread, warps 2-9 are the epilogue: two warps per TMEM lane quarter, each
// owning one half (64 columns) of every tile, so a query is served by two
// threads.  The candidate tiles are streamed twice:
//   pass 1  every thread folds its half-tiles into 64 per-column minima (one
//           FMNMX per pair, no branches); per query, the 64th smallest of the
//           128 minima of both halves is an upper bound tau on the 64th
//           nearest approximate distance (64 distinct candidates lie at or
//           below it);
//   pass 2  every thread marks the pairs at or below tau in a 32-bit mask
//           (one compare and one predicated OR per pair) and appends only the
//           marked candidates to its half-list in shared memory (~90 per
//           query on random data; 96 per half; an overflowing query is
//           finished by the exact fallback kernel).
// Every listed candidate is then re-ranked with the reference FP32
// arithmetic (exact), zero distances dropped, sorted by (distance, index)
// with a warp bitonic network; candidates within 16 ulps of the k-th
// distance are re-ordered by their FP64 distance.  The tensor cores
// recompute each tile in pass 2 because they are otherwise idle: the kernel
// is bound by the epilogue's instruction issue, not by the MMA.
#include <cuda.h>

#include "irc_common.cuh"
#include "irc_plan.cuh"
#include "irc_sm100.cuh"
#include "irc_tc.cuh"

namespace {

using irc_tc::BM;
using irc_tc::BN;
using irc_tc::KP;
constexpr int STAGES = 4;
constexpr int PARTS = 4;                          // epilogue warps per TMEM lane quarter
constexpr int PART = BN / PARTS;                  // columns of a tile per epilogue warp (32)
constexpr int CAPP = 64;                          // list capacity per query and part
constexpr int LROWP = CAPP + 1;                   // part-list row (u32), padded
constexpr int BROW = BN + 1;                      // per-column minima row (f32) during the threshold step
constexpr int EPI_WARPS = 4 * PARTS;
constexpr int EPI_THREADS = 32 * EPI_WARPS;
constexpr int THREADS = 32 * (2 + EPI_WARPS);
constexpr uint32_t TILE_BYTES = BN * KP * 2;      // 16 KB (A tile has the same size)
constexpr uint32_t TMEM_COLS = 2 * BN;
constexpr size_t LIST_BYTES = (size_t)LROWP * PARTS * BM * 4;
constexpr int WARP_KEYS = 64;                     // sorted re-rank keys kept per epilogue warp
constexpr size_t SMEM_BYTES = 1024 /*align slack*/ + TILE_BYTES * (1 + STAGES) + LIST_BYTES +
                              EPI_WARPS * WARP_KEYS * 8 + BM * 4 /*tau*/ + PARTS * BM * 4 /*counts*/ + 256;
static_assert(PART == 32, "one TMEM load of 32 columns per warp and tile");
static_assert((size_t)BROW * BM * 4 <= LIST_BYTES, "minima rows alias the list area");
static_assert(SMEM_BYTES <= 232448, "shared memory budget");

// Ascending bitonic sort of 32*PER keys held PER per lane (element e = lane*PER + i).
template <class T, int PER>
__device__ __forceinline__ void warp_bitonic(T (&v)[PER], int lane)
{
    constexpr int N = 32 * PER;
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= PER) {
                const int ls = stride / PER;
#pragma unroll
                for (int i = 0; i < PER; ++i) {
                    const int e = lane * PER + i;
                    const T o = __shfl_xor_sync(0xffffffffu, v[i], ls);
                    const bool up = (e & size) == 0, lower = (e & stride) == 0;
                    v[i] = (lower == up) ? (o < v[i] ? o : v[i]) : (o > v[i] ? o : v[i]);
                }
            } else {
#pragma unroll
                for (int i = 0; i < PER; ++i) {
                    const int j = i ^ stride;
                    if (j > i) {
                        const int e = lane * PER + i;
                        const bool up = (e & size) == 0;
                        const T a = v[i], b = v[j];
                        const bool sw = up ? (a > b) : (a < b);
                        v[i] = sw ? b : a;
                        v[j] = sw ? a : b;
                    }
                }
            }
        }
    }
}

__device__ __forceinline__ double dist2_f64(const float *__restrict__ b, const float *__restrict__ a, int nC)
{
    double acc = 0.0;
    for (int c = 0; c < nC; ++c) {
        const double d = (double)__ldg(b + c) - (double)__ldg(a + c);
        acc = __dadd_rn(acc, __dmul_rn(d, d));
    }
    return acc;
}

__device__ __forceinline__ void emit(int e, unsigned long long key, int q, int knn, size_t o, int *miKnn,
                                     float *d2Knn, float *vrKnn, float *rho)
{
    const bool have = key != ~0ull;
    const float d2 = have ? __uint_as_float((unsigned)(key >> 32)) : IRC_SINGLE_INF_F;
    const int idx = have ? (int)(key & 0xffffffffu) : q;
    miKnn[(size_t)e + (size_t)knn * o] = idx + 1;
    if (d2Knn) d2Knn[(size_t)e + (size_t)knn * o] = d2;
    if (e == knn - 1) {
        const float vk = irc::ref_sqrt_abs(d2);
        vrKnn[o] = vk;
        if (rho) rho[o] = __fdiv_rn(1.0f, vk);
    }
}

// Exact re-rank of the candidates listed for query q in its PARTS part-lists
// (lists[p*LROWP + i], i < cnt[p]), warp-cooperative.  Requires knn <= 32.
template <int PER>
__device__ __forceinline__ void rerank(const uint32_t *__restrict__ lists, const int (&cnt)[PARTS], int q,
                                       const float *__restrict__ F, int nC, int knn, size_t o,
                                       unsigned long long *ws, int lane, int *miKnn, float *d2Knn, float *vrKnn,
                                       float *rho)
{
    const float *a = F + (size_t)q * nC;
    int cL = 0;
#pragma unroll
    for (int p = 0; p < PARTS; ++p) cL += cnt[p];
    unsigned long long kv[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = i * 32 + lane;
        kv[i] = ~0ull;
        if (e < cL) {
            int p = 0, r = e;
#pragma unroll
            for (int u = 0; u < PARTS - 1; ++u)
                if (p == u && r >= cnt[u]) { r -= cnt[u]; p = u + 1; }
            const int idx = (int)lists[p * LROWP + r];
            const float *bb = F + (size_t)idx * nC;
            float acc = 0.0f;
            for (int c = 0; c < nC; ++c) acc = irc::dterm(acc, __ldg(bb + c), __ldg(a + c));
            if (acc > 0.0f && acc < IRC_SINGLE_INF_F)
                kv[i] = ((unsigned long long)__float_as_uint(acc) << 32) | (unsigned)idx;
        }
    }
    warp_bitonic<unsigned long long, PER>(kv, lane);
#pragma unroll
    for (int i = 0; i < PER; ++i)
        if (lane * PER + i < WARP_KEYS) ws[lane * PER + i] = kv[i];
    __syncwarp();
    // boundary band: keys within 16 ulps of the k-th distance, ordered by FP64
    const unsigned long long kk = ws[knn - 1];
    int lo = knn - 1, hi = knn;
    if (kk != ~0ull) {
        const float vk = __uint_as_float((unsigned)(kk >> 32));
        const float tol = vk * 0x1p-19f;
        unsigned mlo = 0xffffffffu, mhi = 0u;
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int e = lane * PER + i;
            if (e < WARP_KEYS && kv[i] != ~0ull && fabsf(__uint_as_float((unsigned)(kv[i] >> 32)) - vk) <= tol) {
                mlo = min(mlo, (unsigned)e);
                mhi = max(mhi, (unsigned)e + 1u);
            }
        }
        lo = (int)__reduce_min_sync(0xffffffffu, mlo);
        hi = (int)__reduce_max_sync(0xffffffffu, mhi);
    }
    const int nb = hi - lo;
    if (nb > 1 && nb <= 32) {
        // lanes j < nb hold band element lo + j; rank them by (FP64 distance, index)
        const unsigned long long kb = lane < nb ? ws[lo + lane] : ~0ull;
        const int ib = (int)(kb & 0xffffffffu);
        const double db = lane < nb ? dist2_f64(F + (size_t)ib * nC, a, nC) : 0.0;
        int rank = 0;
        for (int m = 0; m < nb; ++m) {
            const double dm = __shfl_sync(0xffffffffu, db, m);
            const int im = __shfl_sync(0xffffffffu, ib, m);
            rank += (dm < db || (dm == db && im < ib)) ? 1 : 0;
        }
        if (lane < nb && lo + rank < knn) emit(lo + rank, kb, q, knn, o, miKnn, d2Knn, vrKnn, rho);
        for (int e = lane; e < lo && e < knn; e += 32) emit(e, ws[e], q, knn, o, miKnn, d2Knn, vrKnn, rho);
    } else {
        for (int e = lane; e < knn; e += 32) emit(e, ws[e], q, knn, o, miKnn, d2Knn, vrKnn, rho);
    }
    __syncwarp();
}

__device__ __forceinline__ void epi_barrier() { asm volatile("bar.sync 1, %0;" ::"n"(EPI_THREADS) : "memory"); }

__global__ void __launch_bounds__(THREADS, 1)
k_knn_tc_bf16(const __grid_constant__ CUtensorMap tmQ, const __grid_constant__ CUtensorMap tmC, irc::PlanDev p,
              const float *__restrict__ F, int nC, int knn, float *__restrict__ vrKnn, float *__restrict__ rho,
              int *__restrict__ miKnn, float *__restrict__ d2Knn, int *__restrict__ scratch)
{
    extern __shared__ unsigned char smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *sA = base;
    uint8_t *sB = base + TILE_BYTES;
    uint32_t *lists = reinterpret_cast<uint32_t *>(sB + STAGES * TILE_BYTES);        // [BM][PARTS][LROWP]
    unsigned long long *wkeys = reinterpret_cast<unsigned long long *>(lists + (size_t)LROWP * PARTS * BM);
    float *sTau = reinterpret_cast<float *>(wkeys + EPI_WARPS * WARP_KEYS);          // [BM]
    int *sCnt = reinterpret_cast<int *>(sTau + BM);                                  // [BM][PARTS], -1 = overflow
    uint64_t *bars = reinterpret_cast<uint64_t *>(sCnt + PARTS * BM);
    uint64_t *full = bars, *empty = bars + STAGES, *a_full = bars + 2 * STAGES;
    uint64_t *acc_full = a_full + 1, *acc_empty = a_full + 3, *mma_done = a_full + 5;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(a_full + 6);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int chunk, qs, nq;
    irc::tile_lookup<BM>(p, blockIdx.x, chunk, qs, nq);
    const int r0 = __ldg(p.roff + chunk), r1 = __ldg(p.roff + chunk + 1);
    int ntiles = 0;
    for (int r = r0; r < r1; ++r) ntiles += (__ldg(p.rn + r) + BN - 1) / BN;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) { sm100::mbar_init(&full[s], 1); sm100::mbar_init(&empty[s], 1); }
        sm100::mbar_init(a_full, 1);
        for (int b = 0; b < 2; ++b) { sm100::mbar_init(&acc_full[b], 1); sm100::mbar_init(&acc_empty[b], EPI_WARPS); }
        sm100::mbar_init(mma_done, 1);
        *abort_flag = 0;
        sm100::fence_mbar_init();
    }
    if (warp == 1) sm100::tmem_alloc(tmem_slot, TMEM_COLS);
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ---------------- TMA producer: the tile sequence, twice ----------------
        if (lane == 0) {
            sm100::prefetch_tmap(&tmQ);
            sm100::prefetch_tmap(&tmC);
            sm100::mbar_arrive_expect_tx(a_full, TILE_BYTES);
            sm100::tma_load_2d(&tmQ, a_full, sA, 0, qs);
            int i = 0;
            bool ok = true;
            for (int pass = 0; pass < 2 && ok; ++pass)
                for (int r = r0; r < r1 && ok; ++r) {
                    const int rs = __ldg(p.rs + r), rn = __ldg(p.rn + r);
                    for (int t = 0; t < rn; t += BN, ++i) {
                        const int s = i % STAGES;
                        if (!(ok = sm100::mbar_wait(&empty[s], ((i / STAGES) & 1) ^ 1, abort_flag))) break;
                        sm100::mbar_arrive_expect_tx(&full[s], TILE_BYTES);
                        sm100::tma_load_2d(&tmC, &full[s], sB + (size_t)s * TILE_BYTES, 0, rs + t);
                    }
                }
            // every issued load has landed before the CTA exits
            for (int j = (i > STAGES ? i - STAGES : 0); j < i; ++j)
                sm100::mbar_wait(&full[j % STAGES], (j / STAGES) & 1, abort_flag);
            sm100::mbar_wait(a_full, 0, abort_flag);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            constexpr uint32_t idesc = sm100::idesc_make(BM, BN, 1, 1);   // bf16 x bf16 -> f32
            if (sm100::mbar_wait(a_full, 0, abort_flag)) {
                sm100::tc_fence_after();
                const uint64_t adesc = sm100::sdesc_sw128(sm100::smem_u32(sA));
                for (int i = 0; i < 2 * ntiles; ++i) {
                    const int s = i % STAGES, b = i & 1;
                    if (!sm100::mbar_wait(&acc_empty[b], ((i >> 1) & 1) ^ 1, abort_flag)) break;
                    if (!sm100::mbar_wait(&full[s], (i / STAGES) & 1, abort_flag)) break;
                    sm100::tc_fence_after();
                    const uint64_t bdesc = sm100::sdesc_sw128(sm100::smem_u32(sB + (size_t)s * TILE_BYTES));
#pragma unroll
                    for (int k = 0; k < KP / 16; ++k)
                        sm100::mma_f16(tmem + b * BN, adesc + 2 * k, bdesc + 2 * k, idesc, k > 0 ? 1u : 0u);
                    sm100::mma_commit(&empty[s]);
                    sm100::mma_commit(&acc_full[b]);
                }
            }
            // every MMA has completed before TMEM is released
            sm100::mma_commit(mma_done);
            sm100::mbar_wait(mma_done, 0, abort_flag);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: one (query, 32-column part) per thread ----------------
        const int ew = warp - 2;                      // 0..15
        const int quarter = warp & 3;                 // TMEM lane quarter this warp may access
        const int part = ew >> 2;                     // which 32 columns of every tile
        const int row = quarter * 32 + lane;
        const uint32_t tbase = tmem + ((uint32_t)(quarter * 32) << 16) + part * PART;
        bool ok = true;
        int i = 0;
        // pass 1: per-column minima of this part
        float bm[PART];
#pragma unroll
        for (int c = 0; c < PART; ++c) bm[c] = __int_as_float(0x7f800000);
        for (int r = r0; r < r1 && ok; ++r) {
            const int rn = __ldg(p.rn + r);
            for (int t = 0; t < rn; t += BN, ++i) {
                const int b = i & 1;
                if (!(ok = sm100::mbar_wait(&acc_full[b], (i >> 1) & 1, abort_flag))) break;
                sm100::tc_fence_after();
                const int lim = min(BN, rn - t) - part * PART;    // valid columns in this part
                if (lim > 0) {
                    float v[32];
                    sm100::tmem_ld32(tbase + b * BN, v);
                    if (lim >= 32) {
#pragma unroll
                        for (int j = 0; j < 32; ++j) bm[j] = fminf(bm[j], v[j]);
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            if (j < lim) bm[j] = fminf(bm[j], v[j]);
                    }
                }
                sm100::tc_fence_before();
                __syncwarp();
                if (lane == 0) sm100::mbar_arrive(&acc_empty[b]);
            }
        }
        // threshold: 64th smallest of the 128 column minima of every query
        {
            float *brow = reinterpret_cast<float *>(lists) + (size_t)row * BROW + part * PART;
#pragma unroll
            for (int c = 0; c < PART; ++c) brow[c] = fmaxf(bm[c], 0.0f);
            epi_barrier();
            for (int L = 0; L < 32 / PARTS; ++L) {
                const int rowL = quarter * 32 + part * (32 / PARTS) + L;
                const float *bl = reinterpret_cast<const float *>(lists) + (size_t)rowL * BROW;
                unsigned v4[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v4[u] = __float_as_uint(bl[u * 32 + lane]);
                warp_bitonic<unsigned, 4>(v4, lane);
                const unsigned kth = __shfl_sync(0xffffffffu, v4[63 % 4], 63 / 4);
                if (lane == 0) sTau[rowL] = __uint_as_float(kth);
            }
            epi_barrier();              // minima rows are read; the list area may be reused
        }
        const float tau = sTau[row];
        // pass 2: collect the candidates at or below tau
        uint32_t *lrow = lists + ((size_t)row * PARTS + part) * LROWP;
        int cnt = 0;
        bool ovf = false;
        for (int r = r0; r < r1 && ok; ++r) {
            const int rs = __ldg(p.rs + r), rn = __ldg(p.rn + r);
            for (int t = 0; t < rn; t += BN, ++i) {
                const int b = i & 1;
                if (!(ok = sm100::mbar_wait(&acc_full[b], (i >> 1) & 1, abort_flag))) break;
                sm100::tc_fence_after();
                const int lim = min(BN, rn - t) - part * PART;
                if (lim > 0) {
                    float v[32];
                    sm100::tmem_ld32(tbase + b * BN, v);
                    unsigned m = 0;
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (v[j] <= tau) m |= 1u << j;
                    if (lim < 32) m &= (1u << lim) - 1u;
                    if (cnt + __popc(m) > CAPP) { ovf = true; m = 0; }
                    const uint32_t c0 = (uint32_t)(rs + t + part * PART);
                    while (m) {
                        const int j = __ffs(m) - 1;
                        m &= m - 1u;
                        lrow[cnt++] = c0 + (uint32_t)j;
                    }
                }
                sm100::tc_fence_before();
                __syncwarp();
                if (lane == 0) sm100::mbar_arrive(&acc_empty[b]);
            }
        }
        sCnt[row * PARTS + part] = ovf ? -1 : cnt;
        epi_barrier();
        // exact re-rank: this warp serves 8 of its quarter's queries
        unsigned long long *ws = wkeys + (size_t)ew * WARP_KEYS;
        for (int L = 0; L < 32 / PARTS && ok; ++L) {
            const int rowL = quarter * 32 + part * (32 / PARTS) + L;
            if (rowL >= nq) break;
            const int q = qs + rowL;
            int c[PARTS];
            bool over = false, big = false;
#pragma unroll
            for (int u = 0; u < PARTS; ++u) { c[u] = sCnt[rowL * PARTS + u]; over |= c[u] < 0; }
            if (over) {                               // finished by the exact fallback kernel
                if (lane == 0) {
                    const int k = atomicAdd(scratch + 0, 1);
                    scratch[irc::kScratchLists + k] = q;
                }
                continue;
            }
            const int cL = c[0] + c[1] + c[2] + c[3];
            big = cL > 128;
            const uint32_t *lr = lists + (size_t)rowL * PARTS * LROWP;
            const size_t o = (size_t)(q - p.q_base);
            if (cL <= 64)
                rerank<2>(lr, c, q, F, nC, knn, o, ws, lane, miKnn, d2Knn, vrKnn, rho);
            else if (!big)
                rerank<4>(lr, c, q, F, nC, knn, o, ws, lane, miKnn, d2Knn, vrKnn, rho);
            else
                rerank<8>(lr, c, q, F, nC, knn, o, ws, lane, miKnn, d2Knn, vrKnn, rho);
        }
    }
    sm100::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        sm100::tc_fence_after();
        sm100::tmem_dealloc(tmem, TMEM_COLS);
    }
    if (threadIdx.x == 0 && *abort_flag) atomicExch(scratch + irc::kScratchErr, 1);
}

}  // namespace

namespace irc_tc {

int launch_knn_bf16(const CUtensorMap &mq, const CUtensorMap &mc, irc_plan *pl, const float *F, int nC, int knn,
                    float *vrKnn, float *rho, int32_t *miKnn, float *d2Knn, cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(k_knn_tc_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(BF16): smem attribute");
    const int tiles = pl->ntiles[irc::tile_slot(BM)];
    k_knn_tc_bf16<<<tiles, THREADS, SMEM_BYTES, s>>>(mq, mc, pl->dev, F, nC, knn, vrKnn, rho, miKnn, d2Knn,
                                                     pl->scratch);
    IRC_CHECK_LAUNCH("irc_site_knn(BF16)");
    return IRC_OK;
}

}  // namespace irc_tc
