// irc_tc.cu -- tensor-core (tcgen05) site kNN: BF16 distance filter, exact
// FP32 re-rank, FP64 at the k-th-neighbour boundary.
//
// A CTA serves one work item: up to four "slots", each a run of queries of
// one drift chunk (128, 64 or 32 rows), packed into the 128 TMEM lanes of
// one M=128 tile; every slot owns a share of the four 128-column TMEM
// accumulators and its own epilogue warps, and the slots' candidate tiles
// are issued round-robin so small chunks (a probe site has ~17 queries per
// chunk) share a CTA without waiting on each other.  Items are ordered by
// cost, largest first.  The BF16 (kind::f16) or FP8-e4m3 (kind::f8f6f4)
// operand rows of irc_tc_host.cu -- 128 bytes each, so both use the same
// swizzled layout and one MMA per 32 bytes -- make every accumulator the
// approximate squared distance (FP8: a fixed positive multiple of it).
// Warp roles: warp 0 issues
// TMA loads (4-stage ring of 128-candidate tiles, four 32-row query boxes),
// warp 1 owns TMEM and issues tcgen05.mma from one thread, warps 2-17 are
// the epilogue: four per TMEM lane quarter, each reading 32 columns of
// every tile of its slot.  Each slot's candidate tiles are streamed twice:
//   pass 1  every thread folds its columns into 32 per-column minima (one
//           FMNMX per pair, no branches); per query, the 64th smallest of the
//           128 minima (found by a bitwise search, rounded up by < 2^-11
//           relative) is an upper bound tau on the 64th nearest approximate
//           distance (64 distinct candidates lie at or below it);
//   pass 2  every thread marks the pairs at or below tau in a 32-bit mask
//           (one compare and one predicated OR per pair) and appends only the
//           marked candidates to its part-list in shared memory (~90 per
//           query on random data, 64 per part; an overflowing query is
//           finished by the exact fallback kernel).
// Every listed candidate is then re-ranked with the reference FP32
// arithmetic (exact), zero distances dropped, sorted by (distance, index)
// with a warp bitonic network; candidates within 16 ulps of the k-th
// distance are re-ordered by their FP64 distance.  The tensor cores
// recompute each tile in pass 2 because they are otherwise idle: the kernel
// is bound by the epilogue's instruction issue, not by the MMA.
#include <cuda.h>

#include <mutex>
#include <vector>

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
constexpr int THREADS = 32 * (2 + EPI_WARPS);
constexpr uint32_t TILE_BYTES = BN * KP * 2;      // 16 KB (A tile has the same size)
constexpr int NBUF = 4;                           // TMEM accumulator buffers, split among the slots
constexpr uint32_t TMEM_COLS = NBUF * BN;         // all 512 columns (one CTA per SM)
constexpr size_t LIST_BYTES = (size_t)LROWP * PARTS * BM * 4;
constexpr int WARP_KEYS = 64;                     // sorted re-rank keys kept per epilogue warp
constexpr int QROW4 = 16;                         // float4 of a staged query row (nC <= 64)
constexpr int TAU_LOW_BIT = 12;                   // threshold search stops at this bit (2^-11 relative)
constexpr size_t SMEM_BYTES = 1024 /*align slack*/ + TILE_BYTES * (1 + STAGES) + LIST_BYTES +
                              BM * 4 /*tau*/ + PARTS * BM * 4 /*counts*/ + 256;
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
    // streaming stores: the outputs are not read again by this kernel and
    // should not push the gathered feature rows out of L2
    __stcs(miKnn + (size_t)e + (size_t)knn * o, idx + 1);
    if (d2Knn) __stcs(d2Knn + (size_t)e + (size_t)knn * o, d2);
    if (e == knn - 1) {
        const float vk = irc::ref_sqrt_abs(d2);
        __stcs(vrKnn + o, vk);
        if (rho) __stcs(rho + o, __fdiv_rn(1.0f, vk));
    }
}

// 256-bit read-only load of 8 floats (32-byte aligned).
__device__ __forceinline__ void ld_nc_v8(const float *p, float (&v)[8])
{
    asm volatile("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                 : "l"(p));
}

// Exact re-rank of the cL candidates listed for query q (list[0 .. cL)),
// warp-cooperative; o = q - q_base.  Requires knn <= 32.  Candidate e is
// lane e % 32 of round e / 32, and every lane gathers its own rows.
template <int PER>
__device__ __forceinline__ void rerank(const uint32_t *__restrict__ list, int cL, bool complete, int q,
                                       const float *__restrict__ F, const float4 *__restrict__ Fp, int Dp4,
                                       float4 *__restrict__ qs, int nC, int knn, size_t o, unsigned long long *ws,
                                       int lane, int *miKnn, float *d2Knn, float *vrKnn, float *rho, int *scratch)
{
    const float *a = F + (size_t)q * nC;
    // the query row, staged once per warp (broadcast reads below)
    if (lane < Dp4) qs[lane] = __ldg(Fp + (size_t)q * Dp4 + lane);
    // exact FP32 distances with the reference arithmetic (d = b - a, fused
    // accumulate in feature order)
    const int nbatch = (cL + 31) / 32;                // <= PER (checked by the caller)
    unsigned long long kv[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) kv[i] = ~0ull;
    __syncwarp();
#pragma unroll
    for (int bi = 0; bi < PER; ++bi) {
        if (bi >= nbatch) break;
        const int e = bi * 32 + lane;
        if (e < cL) {
            const int idx = (int)__ldg(list + e);
            // whole 32-byte sectors: rows are padded to a multiple of 8 floats
            const float *bs = reinterpret_cast<const float *>(Fp + (size_t)idx * Dp4);
            float acc = 0.0f;
#pragma unroll 2
            for (int c8 = 0; c8 < Dp4 / 2; ++c8) {
                float bv[8];
                ld_nc_v8(bs + 8 * c8, bv);
                const float4 a0 = qs[2 * c8], a1 = qs[2 * c8 + 1];
                const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const int c = 8 * c8;
                acc = irc::dterm(acc, bv[0], av[0]);
#pragma unroll
                for (int u = 1; u < 8; ++u)
                    if (c + u < nC) acc = irc::dterm(acc, bv[u], av[u]);
            }
            if (acc > 0.0f && acc < IRC_SINGLE_INF_F)
                kv[bi] = ((unsigned long long)__float_as_uint(acc) << 32) | (unsigned)idx;
        }
    }
    // A list cut by tau that holds fewer than knn + 16 positive distances
    // (exact copies of the query, at distance 0 and excluded like the
    // reference's d > 0 test, crowded the threshold) may miss nearer
    // distinct candidates: such a query goes to the exact fallback.
    if (!complete) {
        unsigned nv = 0;
#pragma unroll
        for (int i = 0; i < PER; ++i) nv += kv[i] != ~0ull;
        if (__reduce_add_sync(0xffffffffu, nv) < (unsigned)(knn + 16)) {
            if (lane == 0) {
                const int k = atomicAdd(scratch + 0, 1);
                scratch[irc::kScratchLists + k] = q;
            }
            return;
        }
    }
    // ws[0 .. WARP_KEYS) <- the WARP_KEYS smallest keys, ascending.  With
    // more than 64 keys, select first: a bitwise search (stopped at
    // TAU_LOW_BIT, rounded up) bounds the k-th distance from above, and the
    // keys at or below that bound plus 2^-16 relative -- the band below
    // lies inside it -- are compacted into ws and sorted alone.  They are
    // the first positions of the full sort, so the result is the same; if
    // more than WARP_KEYS pass, the full sort runs.
    bool sorted = false;
    if (PER > 2) {
        unsigned ans = 0;
#pragma unroll 1
        for (int b = 30; b >= TAU_LOW_BIT; --b) {
            const unsigned t = ans | (1u << b);
            unsigned c = 0;
#pragma unroll
            for (int i = 0; i < PER; ++i) c += (unsigned)((unsigned)(kv[i] >> 32) < t);
            if (__reduce_add_sync(0xffffffffu, c) < (unsigned)knn) ans = t;
        }
        const unsigned ub = ans | ((1u << TAU_LOW_BIT) - 1u);
        const unsigned tb = ub >= 0x7f800000u ? 0x7f800000u
                                              : __float_as_uint(__uint_as_float(ub) * (1.0f + 0x1p-16f));
        int n = 0;
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const bool pr = (unsigned)(kv[i] >> 32) <= tb;          // never an empty slot (~0)
            const unsigned bal = __ballot_sync(0xffffffffu, pr);
            const int pos = n + __popc(bal & ((1u << lane) - 1u));
            if (pr && pos < WARP_KEYS) ws[pos] = kv[i];
            n += __popc(bal);
        }
        __syncwarp();
        if (n <= WARP_KEYS) {
            unsigned long long v2[2];
#pragma unroll
            for (int i = 0; i < 2; ++i) v2[i] = lane * 2 + i < n ? ws[lane * 2 + i] : ~0ull;
            __syncwarp();
            warp_bitonic<unsigned long long, 2>(v2, lane);
#pragma unroll
            for (int i = 0; i < 2; ++i) ws[lane * 2 + i] = v2[i];
            sorted = true;
        }
    }
    if (!sorted) {
        warp_bitonic<unsigned long long, PER>(kv, lane);
#pragma unroll
        for (int i = 0; i < PER; ++i)
            if (lane * PER + i < WARP_KEYS) ws[lane * PER + i] = kv[i];
    }
    __syncwarp();
    // boundary band: keys within 16 ulps of the k-th distance, ordered by FP64
    const unsigned long long kk = ws[knn - 1];
    int lo = knn - 1, hi = knn;
    if (kk != ~0ull) {
        const float vk = __uint_as_float((unsigned)(kk >> 32));
        const float tol = vk * 0x1p-19f;
        unsigned mlo = 0xffffffffu, mhi = 0u;
#pragma unroll
        for (int i = 0; i < WARP_KEYS / 32; ++i) {
            const int e = lane + 32 * i;
            const unsigned long long k = ws[e];
            if (k != ~0ull && fabsf(__uint_as_float((unsigned)(k >> 32)) - vk) <= tol) {
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

__device__ __forceinline__ void slot_barrier(int slot, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(1 + slot), "r"(nthreads) : "memory");
}

// Cursor over the candidate tiles of one chunk: run r (absolute index), offset t.
struct TileCursor {
    // run bounds of the current run (rs, rn) and of the next one (ns, nn),
    // loaded one run ahead so the loads are in flight while the current
    // run's tiles are issued
    int r, r0, r1, t, rs, rn, ns, nn;
    __device__ __forceinline__ int after(int x) const { return x + 1 < r1 ? x + 1 : r0; }
    __device__ __forceinline__ void reset(const irc::PlanDev &p, int chunk)
    {
        r0 = __ldg(p.roff + chunk);
        r1 = __ldg(p.roff + chunk + 1);
        r = r0;
        t = 0;
        rs = __ldg(p.rs + r);
        rn = __ldg(p.rn + r);
        const int n1 = after(r);
        ns = __ldg(p.rs + n1);
        nn = __ldg(p.rn + n1);
    }
    // current tile: first candidate row and valid column count; then advance
    __device__ __forceinline__ void next(const irc::PlanDev &p, int &row0, int &ncol)
    {
        row0 = rs + t;
        ncol = min(BN, rn - t);
        t += BN;
        if (t >= rn) {                                // next run; wraps for the second pass
            t = 0;
            r = after(r);
            rs = ns;
            rn = nn;
            const int n1 = after(r);
            ns = __ldg(p.rs + n1);
            nn = __ldg(p.rn + n1);
        }
    }
};

__device__ __forceinline__ int chunk_tiles(const irc::PlanDev &p, int chunk)
{
    if (chunk < 0) return 0;
    int n = 0;
    for (int r = __ldg(p.roff + chunk); r < __ldg(p.roff + chunk + 1); ++r) n += (__ldg(p.rn + r) + BN - 1) / BN;
    return n;
}

// Epilogue of one warp: lane quarter `quarter` (the TMEM lanes it may read),
// 32 columns `part` of every tile of its slot.  Each slot's epilogue warps
// synchronise only among themselves (named barrier 1 + slot).
__device__ __forceinline__ void epilogue(const irc::PlanDev &p, const irc_tc::TcItem &it, const int (&nt)[4], int qps,
                                         int bps, uint32_t tmem, uint32_t *lists, float *sTau, int *sCnt,
                                         uint64_t *acc_full, uint64_t *acc_empty, volatile int *abort_flag,
                                         const irc_tc::ListOut &lo, int *scratch, int warp, int lane)
{
    const int ew = warp - 2;                      // 0..15
    const int quarter = warp & 3;                 // TMEM lane quarter this warp may access
    const int part = ew >> 2;                     // which 32 columns of every tile
    const int s = quarter / qps;                  // slot of this lane quarter
    const int qrow = (quarter % qps) * 32;        // first row of this quarter inside its slot
    const int nq_s = it.chunk[s] >= 0 ? it.nq[s] : 0;
    const int nts = nt[s];
    const int slot_threads = 32 * PARTS * qps;
    const int row = quarter * 32 + lane;
    const uint32_t tbase = tmem + ((uint32_t)(quarter * 32) << 16) + part * PART;
    const bool active = qrow < nq_s;              // warp-uniform: any valid query in this quarter
    bool ok = true;
    TileCursor cur;
    if (nts) cur.reset(p, it.chunk[s]);

    // pass 1: per-column minima of this part
    float bm[PART];
#pragma unroll
    for (int c = 0; c < PART; ++c) bm[c] = __int_as_float(0x7f800000);
    int bj = 0, use = 0;                          // tile j of this slot: buffer s*bps + bj, use count
    for (int j = 0; j < nts && ok; ++j) {
        const int b = s * bps + bj;
        const uint32_t par = use & 1;
        if (++bj == bps) { bj = 0; ++use; }
        int row0, ncol;
        cur.next(p, row0, ncol);
        if (!(ok = sm100::mbar_wait(&acc_full[b], par, abort_flag))) break;
        sm100::tc_fence_after();
        const int lim = ncol - part * PART;                   // valid columns in this part
        if (active && lim > 0) {
            float v[32];
            sm100::tmem_ld32(tbase + b * BN, v);
            if (lim >= 32) {
#pragma unroll
                for (int jj = 0; jj < 32; ++jj) bm[jj] = fminf(bm[jj], v[jj]);
            } else {
#pragma unroll
                for (int jj = 0; jj < 32; ++jj)
                    if (jj < lim) bm[jj] = fminf(bm[jj], v[jj]);
            }
        }
        sm100::tc_fence_before();
        __syncwarp();
        if (lane == 0) sm100::mbar_arrive(&acc_empty[b]);
    }
    // threshold: 64th smallest of the 128 column minima of every query; the
    // minima rows of a quarter alias that quarter's own list rows
    float *qarea = reinterpret_cast<float *>(lists + (size_t)quarter * 32 * PARTS * LROWP);
    {
        float *brow = qarea + lane * BROW + part * PART;
#pragma unroll
        for (int c = 0; c < PART; ++c) brow[c] = fmaxf(bm[c], 0.0f);
        slot_barrier(s, slot_threads);
        // The warp's 8 rows at once (independent chains): a bitwise search,
        // from the top, of the largest t with fewer than 64 minima below it,
        // i.e. of the 64th smallest minimum, on the non-negative float bit
        // patterns.  It stops at TAU_LOW_BIT and rounds up, so tau is an
        // upper bound of the 64th smallest within 2^-11 of it (a few more
        // candidates listed, never fewer).
        constexpr int RL = 32 / PARTS;
        unsigned v4[RL][4], ans[RL];
#pragma unroll
        for (int L = 0; L < RL; ++L) {
            const float *bl = qarea + (part * RL + L) * BROW;
#pragma unroll
            for (int u = 0; u < 4; ++u) v4[L][u] = __float_as_uint(bl[u * 32 + lane]);
            ans[L] = 0u;
        }
#pragma unroll 1
        for (int b = 30; b >= TAU_LOW_BIT; --b) {
#pragma unroll
            for (int L = 0; L < RL; ++L) {
                const unsigned t = ans[L] | (1u << b);
                const unsigned c = (unsigned)(v4[L][0] < t) + (unsigned)(v4[L][1] < t) + (unsigned)(v4[L][2] < t) +
                                   (unsigned)(v4[L][3] < t);
                if (__reduce_add_sync(0xffffffffu, c) < 64u) ans[L] = t;
            }
        }
        if (lane < RL) {
            unsigned a = ans[0];
#pragma unroll
            for (int L = 1; L < RL; ++L)
                if (lane == L) a = ans[L];
            sTau[quarter * 32 + part * RL + lane] = __uint_as_float(min(a | ((1u << TAU_LOW_BIT) - 1u), 0x7f800000u));
        }
        slot_barrier(s, slot_threads);     // minima rows are read; the list rows may be written
    }
    const float tau = sTau[row];
    // pass 2: collect the candidates at or below tau
    uint32_t *lrow = lists + ((size_t)row * PARTS + part) * LROWP;
    int cnt = 0;
    bool ovf = false;
    for (int j = nts; j < 2 * nts && ok; ++j) {
        const int b = s * bps + bj;
        const uint32_t par = use & 1;
        if (++bj == bps) { bj = 0; ++use; }
        int row0, ncol;
        cur.next(p, row0, ncol);
        if (!(ok = sm100::mbar_wait(&acc_full[b], par, abort_flag))) break;
        sm100::tc_fence_after();
        const int lim = ncol - part * PART;
        if (active && lim > 0) {
            float v[32];
            sm100::tmem_ld32(tbase + b * BN, v);
            // four independent partial masks: short dependency chains
            unsigned mq[4] = {0u, 0u, 0u, 0u};
#pragma unroll
            for (int jj = 0; jj < 32; ++jj)
                if (v[jj] <= tau) mq[jj & 3] |= 1u << jj;
            unsigned m = (mq[0] | mq[1]) | (mq[2] | mq[3]);
            if (lim < 32) m &= (1u << lim) - 1u;
            if (cnt + __popc(m) > CAPP) { ovf = true; m = 0; }
            const uint32_t c0 = (uint32_t)(row0 + part * PART);
            while (m) {
                const int jj = __ffs(m) - 1;
                m &= m - 1u;
                lrow[cnt++] = c0 + (uint32_t)jj;
            }
        }
        sm100::tc_fence_before();
        __syncwarp();
        if (lane == 0) sm100::mbar_arrive(&acc_empty[b]);
    }
    sCnt[row * PARTS + part] = ovf ? -1 : cnt;
    slot_barrier(s, slot_threads);
    // Hand the lists to the re-rank kernel: this warp packs 8 of its
    // quarter's queries (query L in lane L) into one bump allocation and
    // records (offset, length) per query; an overflowed part-list, a list
    // longer than LIST_MAX or a full list area sends the query to the exact
    // fallback instead.
    if (!__all_sync(0xffffffffu, ok)) return;
    constexpr int RL = 32 / PARTS;
    int cL = -1;                                  // -1: no query in this lane, -2: to the fallback
    if (lane < RL && qrow + part * RL + lane < nq_s) {
        const int rowL = quarter * 32 + part * RL + lane;
        int t = 0;
        bool over = false;
#pragma unroll
        for (int u = 0; u < PARTS; ++u) {
            const int c = sCnt[rowL * PARTS + u];
            over |= c < 0;
            t += c;
        }
        cL = (over || t > irc_tc::LIST_MAX) ? -2 : t;
    }
    const unsigned len = cL > 0 ? (unsigned)cL : 0u;
    unsigned incl = len;
#pragma unroll
    for (int d = 1; d < RL; d <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    const unsigned total = __shfl_sync(0xffffffffu, incl, RL - 1);
    unsigned base = 0;
    if (lane == 0 && total) base = atomicAdd(lo.count, total);
    base = __shfl_sync(0xffffffffu, base, 0);
    const bool fits = (unsigned long long)base + total <= (unsigned long long)lo.cap;
    if (lane < RL && cL != -1) {
        const int q = it.qs[s] + qrow + part * RL + lane;
        if (cL == -2 || !fits) {
            const int k = atomicAdd(scratch + 0, 1);
            scratch[irc::kScratchLists + k] = q;
        } else {
            // bit 30: the list holds every candidate of the chunk (nothing was cut by tau)
            const int complete = cL == __ldg(p.ncand + it.chunk[s]) ? (1 << 30) : 0;
            lo.qinfo[q - p.q_base] = make_int2((int)(base + incl - len), cL | complete);
        }
    }
    if (!fits) return;
#pragma unroll 1
    for (int L = 0; L < RL; ++L) {
        const int n = __shfl_sync(0xffffffffu, cL, L);
        const unsigned off = base + __shfl_sync(0xffffffffu, incl - len, L);
        if (n <= 0) continue;                     // warp-uniform
        const int rowL = quarter * 32 + part * RL + L;
        const int c0 = sCnt[rowL * PARTS + 0], c1 = sCnt[rowL * PARTS + 1], c2 = sCnt[rowL * PARTS + 2];
        const uint32_t *lr = lists + (size_t)rowL * PARTS * LROWP;
        for (int e = lane; e < n; e += 32) {
            int pp = 0, r = e;
            if (r >= c0) {
                r -= c0;
                pp = 1;
                if (r >= c1) {
                    r -= c1;
                    pp = 2;
                    if (r >= c2) { r -= c2; pp = 3; }
                }
            }
            lo.lists[off + e] = lr[pp * LROWP + r];
        }
    }
}

// TMA producer (one thread): the four 32-row query boxes, then the slots'
// candidate tiles round-robin, each slot's sequence twice (both passes).
template <int NS>
__device__ __forceinline__ void produce(const CUtensorMap &tmQ, const CUtensorMap &tmC, const irc::PlanDev &p,
                                        const irc_tc::TcItem &it, const int (&nt)[4], uint8_t *sA, uint8_t *sB,
                                        uint64_t *full, uint64_t *empty, uint64_t *a_full, volatile int *abort_flag)
{
    constexpr int QPS = 4 / NS;
    sm100::prefetch_tmap(&tmQ);
    sm100::prefetch_tmap(&tmC);
    sm100::mbar_arrive_expect_tx(a_full, TILE_BYTES);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int s = q / QPS;
        const int row0 = it.chunk[s] >= 0 ? it.qs[s] + (q % QPS) * 32 : 0;
        sm100::tma_load_2d(&tmQ, a_full, sA + q * (TILE_BYTES / 4), 0, row0);
    }
    TileCursor cur[NS];
    int n2[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        n2[s] = 2 * nt[s];
        if (nt[s]) cur[s].reset(p, it.chunk[s]);
    }
    int i = 0;
    bool ok = true;
    for (int k = 0; ok; ++k) {
        bool any = false;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            if (ok && k < n2[s]) {
                any = true;
                int row0, ncol;
                cur[s].next(p, row0, ncol);
                const int st = i % STAGES;
                if ((ok = sm100::mbar_wait(&empty[st], ((i / STAGES) & 1) ^ 1, abort_flag))) {
                    sm100::mbar_arrive_expect_tx(&full[st], TILE_BYTES);
                    sm100::tma_load_2d(&tmC, &full[st], sB + (size_t)st * TILE_BYTES, 0, row0);
                    ++i;
                }
            }
        }
        if (!any) break;
    }
    // every issued load has landed before the CTA exits
    for (int j = (i > STAGES ? i - STAGES : 0); j < i; ++j)
        sm100::mbar_wait(&full[j % STAGES], (j / STAGES) & 1, abort_flag);
    sm100::mbar_wait(a_full, 0, abort_flag);
}

// MMA issuer (one thread), in the producer's order; slot s's tile k goes to
// accumulator s*BPS + k % BPS.
template <int NS, bool FP8>
__device__ __forceinline__ void issue(const int (&nt)[4], int nk, uint32_t tmem, uint8_t *sA, uint8_t *sB, uint64_t *full,
                                      uint64_t *empty, uint64_t *a_full, uint64_t *acc_full, uint64_t *acc_empty,
                                      uint64_t *mma_done, volatile int *abort_flag)
{
    constexpr int BPS = NBUF / NS;
    // bf16 x bf16 (kind::f16, K = 16) or e4m3 x e4m3 (kind::f8f6f4, K = 32) -> f32;
    // either way one MMA consumes 32 bytes of every 128-byte operand row
    constexpr uint32_t idesc = FP8 ? sm100::idesc_make(BM, BN, 0, 0) : sm100::idesc_make(BM, BN, 1, 1);
    if (sm100::mbar_wait(a_full, 0, abort_flag)) {
        sm100::tc_fence_after();
        const uint64_t adesc = sm100::sdesc_sw128(sm100::smem_u32(sA));
        int n2[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) n2[s] = 2 * nt[s];
        int i = 0;
        bool ok = true;
        for (int k = 0; ok; ++k) {
            bool any = false;
#pragma unroll
            for (int s = 0; s < NS; ++s) {
                if (ok && k < n2[s]) {
                    any = true;
                    const int b = s * BPS + k % BPS, u = k / BPS, st = i % STAGES;
                    ok = sm100::mbar_wait(&acc_empty[b], (u & 1) ^ 1, abort_flag) &&
                         sm100::mbar_wait(&full[st], (i / STAGES) & 1, abort_flag);
                    if (ok) {
                        sm100::tc_fence_after();
                        const uint64_t bdesc = sm100::sdesc_sw128(sm100::smem_u32(sB + (size_t)st * TILE_BYTES));
#pragma unroll
                        for (int kk = 0; kk < KP / 16; ++kk)
                            if (kk >= nk)
                                break;                    // the rest of every operand row is zero
                            else if (FP8)
                                sm100::mma_f8(tmem + b * BN, adesc + 2 * kk, bdesc + 2 * kk, idesc, kk > 0 ? 1u : 0u);
                            else
                                sm100::mma_f16(tmem + b * BN, adesc + 2 * kk, bdesc + 2 * kk, idesc, kk > 0 ? 1u : 0u);
                        sm100::mma_commit(&empty[st]);
                        sm100::mma_commit(&acc_full[b]);
                        ++i;
                    }
                }
            }
            if (!any) break;
        }
    }
    // every MMA has completed before TMEM is released
    sm100::mma_commit(mma_done);
    sm100::mbar_wait(mma_done, 0, abort_flag);
}

template <bool FP8>
__global__ void __launch_bounds__(THREADS, 1)
k_knn_tc(const __grid_constant__ CUtensorMap tmQ, const __grid_constant__ CUtensorMap tmC, irc::PlanDev p,
              const irc_tc::TcItem *__restrict__ items, int nk, irc_tc::ListOut lo, int *__restrict__ scratch)
{
    extern __shared__ unsigned char smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *sA = base;
    uint8_t *sB = base + TILE_BYTES;
    uint32_t *lists = reinterpret_cast<uint32_t *>(sB + STAGES * TILE_BYTES);        // [BM][PARTS][LROWP]
    float *sTau = reinterpret_cast<float *>(lists + (size_t)LROWP * PARTS * BM);     // [BM]
    int *sCnt = reinterpret_cast<int *>(sTau + BM);                                  // [BM][PARTS], -1 = overflow
    uint64_t *bars = reinterpret_cast<uint64_t *>(sCnt + PARTS * BM);
    uint64_t *full = bars, *empty = bars + STAGES, *a_full = bars + 2 * STAGES;
    uint64_t *acc_full = a_full + 1, *acc_empty = acc_full + NBUF, *mma_done = acc_empty + NBUF;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const irc_tc::TcItem it = items[blockIdx.x];
    const int nslot = it.nslot, qps = 4 / nslot, bps = NBUF / nslot;
    int nt[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) nt[s] = s < nslot ? chunk_tiles(p, it.chunk[s]) : 0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) { sm100::mbar_init(&full[s], 1); sm100::mbar_init(&empty[s], 1); }
        sm100::mbar_init(a_full, 1);
        for (int b = 0; b < NBUF; ++b) {
            sm100::mbar_init(&acc_full[b], 1);
            sm100::mbar_init(&acc_empty[b], PARTS * qps);      // the owning slot's epilogue warps
        }
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
        if (lane == 0) {
            if (nslot == 1) produce<1>(tmQ, tmC, p, it, nt, sA, sB, full, empty, a_full, abort_flag);
            else if (nslot == 2) produce<2>(tmQ, tmC, p, it, nt, sA, sB, full, empty, a_full, abort_flag);
            else produce<4>(tmQ, tmC, p, it, nt, sA, sB, full, empty, a_full, abort_flag);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            if (nslot == 1) issue<1, FP8>(nt, nk, tmem, sA, sB, full, empty, a_full, acc_full, acc_empty, mma_done, abort_flag);
            else if (nslot == 2) issue<2, FP8>(nt, nk, tmem, sA, sB, full, empty, a_full, acc_full, acc_empty, mma_done, abort_flag);
            else issue<4, FP8>(nt, nk, tmem, sA, sB, full, empty, a_full, acc_full, acc_empty, mma_done, abort_flag);
        }
        __syncwarp();
    } else {
        epilogue(p, it, nt, qps, bps, tmem, lists, sTau, sCnt, acc_full, acc_empty, abort_flag, lo, scratch, warp,
                 lane);
    }
    sm100::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        sm100::tc_fence_after();
        sm100::tmem_dealloc(tmem, TMEM_COLS);
    }
    if (threadIdx.x == 0 && *abort_flag) atomicExch(scratch + irc::kScratchErr, 1);
}

// Exact re-rank kernel: one warp per query of the plan, in query order (the
// queries of a chunk share their candidate rows, which stay in L1/L2 for the
// block's warps); queries without a list (qinfo.x < 0) belong to the exact
// fallback or to no chunk.
constexpr int RR_WARPS = 8;

__global__ void __launch_bounds__(32 * RR_WARPS, 4)
k_rerank(const int2 *__restrict__ qinfo, const uint32_t *__restrict__ lists, int n_out, int q_base,
         const float *__restrict__ F, const float4 *__restrict__ Fp, int nC, int knn, float *__restrict__ vrKnn,
         float *__restrict__ rho, int *__restrict__ miKnn, float *__restrict__ d2Knn, int *__restrict__ scratch)
{
    __shared__ unsigned long long wkeys[RR_WARPS * WARP_KEYS];
    __shared__ float4 qrows[RR_WARPS * QROW4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int o = blockIdx.x * RR_WARPS + warp;
    if (o >= n_out) return;
    const int2 qi = __ldg(qinfo + o);
    if (qi.x < 0) return;
    const int Dp4 = irc_tc::fp_row4(nC);
    const uint32_t *lst = lists + (unsigned)qi.x;
    const int cL = qi.y & 0x3fffffff, q = q_base + o;
    const bool complete = (qi.y >> 30) & 1;
    unsigned long long *ws = wkeys + warp * WARP_KEYS;
    float4 *qs = qrows + warp * QROW4;
    if (cL <= 64)
        rerank<2>(lst, cL, complete, q, F, Fp, Dp4, qs, nC, knn, (size_t)o, ws, lane, miKnn, d2Knn, vrKnn, rho,
                  scratch);
    else if (cL <= 128)
        rerank<4>(lst, cL, complete, q, F, Fp, Dp4, qs, nC, knn, (size_t)o, ws, lane, miKnn, d2Knn, vrKnn, rho,
                  scratch);
    else
        rerank<8>(lst, cL, complete, q, F, Fp, Dp4, qs, nC, knn, (size_t)o, ws, lane, miKnn, d2Knn, vrKnn, rho,
                  scratch);
}

}  // namespace

namespace irc_tc {

// Kernel timing (irc_profile_begin / irc_profile_end): three events per
// tensor-core call -- before the filter, between filter and re-rank, after
// the re-rank -- in a table created by irc_profile_begin.
static std::mutex g_prof_mu;
static std::vector<cudaEvent_t> g_prof_ev;
static int g_prof_used = 0, g_prof_on = 0;

static cudaEvent_t *profile_slot()
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (!g_prof_on || 3 * (g_prof_used + 1) > (int)g_prof_ev.size()) return nullptr;
    return &g_prof_ev[3 * g_prof_used++];
}

int launch_knn_tc(bool fp8, const CUtensorMap &mq, const CUtensorMap &mc, irc_plan *pl, const float *F,
                  const float4 *Fp, int nC, int knn, float *vrKnn, float *rho, int32_t *miKnn, float *d2Knn,
                  const ListOut &lo, cudaStream_t s)
{
    auto kern = fp8 ? k_knn_tc<true> : k_knn_tc<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(tensor core): smem attribute");
    const int n_out = pl->dev.n_out;
    e = cudaMemsetAsync(lo.qinfo, 0xff, (size_t)n_out * sizeof(int2), s);          // (-1, -1): no list
    if (e == cudaSuccess) e = cudaMemsetAsync(lo.count, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(tensor core): memset");
    // MMAs per tile: only the 32-byte K slices that hold data (nC features
    // plus 6 BF16 / 12 FP8 norm entries); the rest of each row is zero
    const int used = fp8 ? nC + 12 : 2 * (nC + 6);
    const int nk = (used + 31) / 32;
    cudaEvent_t *ev = profile_slot();
    if (ev) cudaEventRecord(ev[0], s);
    kern<<<pl->n_tc_items, THREADS, SMEM_BYTES, s>>>(mq, mc, pl->dev, pl->tc_items, nk, lo, pl->scratch);
    IRC_CHECK_LAUNCH("irc_site_knn(tensor core)");
    if (ev) cudaEventRecord(ev[1], s);
    k_rerank<<<(n_out + RR_WARPS - 1) / RR_WARPS, 32 * RR_WARPS, 0, s>>>(
        lo.qinfo, lo.lists, n_out, pl->dev.q_base, F, Fp, nC, knn, vrKnn, rho, miKnn, d2Knn, pl->scratch);
    IRC_CHECK_LAUNCH("irc_site_knn(tensor core) re-rank");
    if (ev) cudaEventRecord(ev[2], s);
    return IRC_OK;
}

}  // namespace irc_tc

extern "C" {

int irc_profile_begin(int max_calls)
{
    using namespace irc_tc;
    if (max_calls <= 0 || max_calls > 65536) {
        irc_host::set_error("irc_profile_begin: max_calls must be in 1..65536");
        return IRC_E_INVAL;
    }
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (cudaEvent_t e : g_prof_ev) cudaEventDestroy(e);
    g_prof_ev.clear();
    for (int i = 0; i < 3 * max_calls; ++i) {
        cudaEvent_t e;
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) {
            for (cudaEvent_t x : g_prof_ev) cudaEventDestroy(x);
            g_prof_ev.clear();
            return irc_host::cuda_status(r, "irc_profile_begin");
        }
        g_prof_ev.push_back(e);
    }
    g_prof_used = 0;
    g_prof_on = 1;
    return IRC_OK;
}

int irc_profile_end(float *filter_ms, float *rerank_ms, int *calls)
{
    using namespace irc_tc;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    float a = 0.0f, b = 0.0f;
    for (int i = 0; i < g_prof_used; ++i) {
        float x = 0.0f, y = 0.0f;
        cudaError_t r = cudaEventSynchronize(g_prof_ev[3 * i + 2]);
        if (r == cudaSuccess) r = cudaEventElapsedTime(&x, g_prof_ev[3 * i], g_prof_ev[3 * i + 1]);
        if (r == cudaSuccess) r = cudaEventElapsedTime(&y, g_prof_ev[3 * i + 1], g_prof_ev[3 * i + 2]);
        if (r != cudaSuccess) {
            g_prof_on = 0;
            return irc_host::cuda_status(r, "irc_profile_end");
        }
        a += x;
        b += y;
    }
    if (filter_ms) *filter_ms = a;
    if (rerank_ms) *rerank_ms = b;
    if (calls) *calls = g_prof_used;
    for (cudaEvent_t e : g_prof_ev) cudaEventDestroy(e);
    g_prof_ev.clear();
    g_prof_used = 0;
    g_prof_on = 0;
    return IRC_OK;
}

}  // extern "C"
