// irc_tc.cu -- tensor-core (tcgen05) site kNN: BF16 distance filter, exact
// FP32 re-rank, FP64 at the k-th-neighbour boundary.
//
// A work item is up to four "slots", each a run of queries of one drift
// chunk (128, 64 or 32 rows), packed into the 128 TMEM lanes of one M=128
// tile; every slot owns a share of the TMEM accumulators and its own epilogue
// warps, and the slots' candidate tiles are issued round-robin so small
// chunks (a probe site has ~17 queries per chunk) share a CTA without waiting
// on each other.  The filter is persistent: one launch per packing class
// (one-, two- or four-slot items), one CTA per SM, each CTA taking items from
// the class's work queue (an atomic head over the items, ordered by cost,
// largest first) until it is empty.  Barrier phases, stage and accumulator
// counters run on across a CTA's items; the query tile is double-buffered,
// so the next item's tiles load and its first MMAs run while the epilogue
// still finishes the item before.
// The BF16 (kind::f16) or FP8-e4m3 (kind::f8f6f4) operand rows of
// irc_tc_host.cu -- 128 bytes each, so both use the same swizzled layout and
// one MMA per 32 bytes -- make every accumulator the approximate squared
// distance (FP8: a fixed positive multiple of it).
//
// A slot streams its chunk's 128-candidate tiles (a per-chunk tile table in
// the plan) in units: items of one or two slots use 256-wide units (two
// tiles, loaded by two TMA boxes into one stage, one N = 256 MMA per K slice,
// two 256-column accumulators) -- the issue cost of an MMA is the same at
// N = 256 as at 128, so this halves it per pair -- unless the plan asks for
// 128-wide units (irc_plan_tc_units), and four-slot items 128-wide units
// (four accumulators, one per slot).  Warp roles: warp 0 claims items and
// issues TMA loads (a 3- or 4-stage ring, four 32-row query boxes per item),
// warp 1 owns TMEM and issues tcgen05.mma from one thread, warps 2-17 are the
// epilogue: four per TMEM lane quarter, warp w of a quarter reading columns
// 32w .. 32w + 31 of every 128-tile.  Each slot's units are streamed twice:
//   pass 1  every thread folds its columns into 32 per-column minima (the two
//           tiles of a wide unit with one three-input min); per query, the
//           r-th smallest of the 128 minima (r = 48 for BF16, 64 for FP8; a
//           bitwise search, rounded up by < 2^-11 relative, < 2^-7 for
//           slots of at most 16 tiles) is an upper bound
//           tau on the r-th nearest approximate distance (r distinct
//           candidates lie at or below it, against knn <= 32);
//   pass 2  the candidates at or below tau are appended to the query's list
//           in shared memory (~55-70 per query on random data, at most 192; an
//           overflowing query is finished by the exact fallback kernel).  In
//           the BF16 wide units the thresholds are folded into the MMA: each
//           query's -tau goes into three spare K columns of its operand row,
//           against 1s in the candidate rows, so the accumulators are
//           d2 - tau and a hit is a sign bit (one funnel shift per pair);
//           elsewhere every pair is compared with tau in the epilogue.
// The minima partition is the same at both widths, so results never depend
// on the width or the work layout.  Every listed candidate is then re-ranked
// with the reference FP32 arithmetic (exact), zero distances dropped, sorted
// by (distance, index) with a warp bitonic network; candidates within 16 ulps
// of the k-th distance are re-ordered by their FP64 distance.  The kernel is
// bound by its epilogue (TMEM loads, fold, compare, list appends), not by the
// tensor pipe.
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>
#include <type_traits>
#include <vector>

#include "irc_common.cuh"
#include "irc_plan.cuh"
#include "irc_sm100.cuh"
#include "irc_tc.cuh"

// Poll limit of the filter's pipeline waits (irc_set_wait_limit); the
// drains of a CTA's own copies and MMAs keep the full bound.
__constant__ uint32_t c_wait_polls = 1u << 22;

namespace {

using irc_tc::BM;
using irc_tc::KP;
constexpr int PARTS = 4;                          // epilogue warps per TMEM lane quarter
constexpr int PART = 32;                          // columns of a 128-tile per epilogue warp (one minimum each)
constexpr int BROW = 128 + 1;                     // minima row of a query (f32, 4 parts x 32) in the threshold step
constexpr int EPI_WARPS = 4 * PARTS;
constexpr int THREADS = 32 * (2 + EPI_WARPS);
constexpr uint32_t A_BYTES = BM * KP * 2;         // the query tile: 128 rows x 128 bytes
constexpr uint32_t HALF_BYTES = 128 * KP * 2;     // one 128-candidate tile
constexpr uint32_t TMEM_COLS = 512;               // all TMEM columns (one CTA per SM)
constexpr int LISTCAP = 192;                      // candidate-list capacity per query (the four warps' hits pooled)
constexpr int LROW = LISTCAP + 1;                 // list row (u32), padded
constexpr size_t LIST_BYTES = (size_t)LROW * BM * 4;
constexpr int WARP_KEYS = 64;                     // sorted re-rank keys kept per epilogue warp
constexpr int QROW4 = 16;                         // float4 of a staged query row (nC <= 64)
constexpr int TAU_LOW_BIT = 12;                   // threshold search stops at this bit (2^-11 relative)
// The threshold is the tau_rank-th smallest per-column minimum: tau_rank
// distinct candidates lie at or below it, a margin over knn (<= 32) for the
// rounding of the filter.  A list it cut must hold at least knn +
// crowd_margin positive distances (exact copies of the query, at distance 0,
// take places in it), else the query goes to the exact fallback.  BF16:
// measured against FP64, rank 48 keeps the kNN recall at 1.0 with the same
// rho / delta error as rank 64 on the 400k-spike drift site, a 1M-spike
// sample of the probe batch and the test sites, with 20% less re-rank work;
// rank 40 missed one neighbour on a 20k-spike site with exact duplicates (its
// BF16 distance error, ~2^-8 |a| / d relative, crossed the gap between the
// 30th and 40th neighbour), rank 44 did not.  FP8 (3 mantissa bits) keeps
// rank 64.
__host__ __device__ constexpr int tau_rank(bool fp8) { return fp8 ? 64 : 48; }
__host__ __device__ constexpr int crowd_margin(bool fp8) { return fp8 ? 16 : 8; }
static_assert(tau_rank(false) >= irc_tc::KNN_MAX + crowd_margin(false), "rank covers knn plus the margin");
static_assert(tau_rank(true) >= irc_tc::KNN_MAX + crowd_margin(true), "rank covers knn plus the margin");
static_assert((size_t)BROW * BM * 4 <= LIST_BYTES, "minima rows alias the list area");
static_assert(LISTCAP <= irc_tc::LIST_MAX, "the re-rank takes every list the filter hands over");

// Shapes of the filter for a unit width BN (MMA N): 256 for items of one or
// two slots (two 256-column accumulators; the MMA issue cost per instruction
// is the same at N = 256 as at 128, so the wider unit halves it per pair), 128
// for four-slot items (one accumulator per slot).
template <int BN>
struct Tile {
    static_assert(BN == 128 || BN == 256, "unit width");
    static constexpr int NBUF = TMEM_COLS / BN;   // accumulator buffers, split among the slots
    static constexpr int STAGES = BN == 256 ? 3 : 4;
    static constexpr uint32_t STAGE_BYTES = BN * KP * 2;
    // two query tiles (the next item's loads while this one's MMAs run)
    static constexpr size_t SMEM_BYTES = 1024 /*align slack*/ + 2 * A_BYTES + (size_t)STAGE_BYTES * STAGES +
                                         LIST_BYTES + BM * 4 /*tau*/ + BM * 4 /*counts*/ + 256 /*barriers*/;
    static_assert(SMEM_BYTES <= 232448, "shared memory budget");
};

// Work units of a slot per pass over its chunk's sequence of 128-candidate
// tiles (nts of them).  BN = 128: one tile per unit; BN = 256: tiles 2u and
// 2u + 1 in unit u, loaded by two TMA boxes into the halves of one 256-row
// stage (the second absent when the count is odd).  Either way epilogue warp
// w of a lane quarter reads columns 32w .. 32w + 31 of every 128-tile, and
// per-column minimum i of that warp covers column 32w + i of every tile, so
// the minima, the threshold and the candidate lists do not depend on the
// width, nor on the work layout.
template <int BN>
__device__ __forceinline__ int units_per_pass(int nts)
{
    return BN == 256 ? (nts + 1) >> 1 : nts;
}

// A wait of the filter's pipeline (see sm100::mbar_wait), bounded by the
// poll limit set with irc_set_wait_limit.  It starts with try_wait (no
// non-blocking probes): a probing warp would take issue slots from the
// epilogue warps sharing its scheduler.  A limit below 64 polls makes every
// poll a non-blocking test instead, so such a limit gives up at the first
// phase that is not already complete (how the tests force the timeout path).
__device__ __forceinline__ bool pipe_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag)
{
    const uint32_t lim = c_wait_polls;
    return sm100::mbar_wait(bar, parity, abort_flag, lim, lim < 64u ? lim : 0u);
}

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

__device__ __forceinline__ double dist2_f64(const float *__restrict__ b, const float *__restrict__ a, int nd)
{
    double acc = 0.0;
    for (int c = 0; c < nd; ++c) {
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
// lane e % 32 of round e / 32, and every lane gathers its own rows.  nC is
// the row stride of F; nd <= nC the features that can be non-zero for this
// query and its candidates (the width of their site): the rest are zero in
// both rows and add exactly 0 to every distance, so they are skipped.
template <int PER>
__device__ __forceinline__ void rerank(const uint32_t *__restrict__ list, int cL, bool complete, int q,
                                       const float *__restrict__ F, const float4 *__restrict__ Fp, int Dp4,
                                       float4 *__restrict__ qs, int nC, int nd, int knn, size_t o,
                                       unsigned long long *ws, int lane, int margin, int *miKnn, float *d2Knn,
                                       float *vrKnn, float *rho, int *scratch)
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
            const int full = nd >> 3, tail = nd & 7;   // whole groups of 8 features, then the rest
#pragma unroll 2
            for (int c8 = 0; c8 < full; ++c8) {
                float bv[8];
                ld_nc_v8(bs + 8 * c8, bv);
                const float4 a0 = qs[2 * c8], a1 = qs[2 * c8 + 1];
                const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
                for (int u = 0; u < 8; ++u) acc = irc::dterm(acc, bv[u], av[u]);
            }
            if (tail) {
                float bv[8];
                ld_nc_v8(bs + 8 * full, bv);
                const float4 a0 = qs[2 * full], a1 = qs[2 * full + 1];
                const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (u < tail) acc = irc::dterm(acc, bv[u], av[u]);
            }
            if (acc > 0.0f && acc < IRC_SINGLE_INF_F)
                kv[bi] = ((unsigned long long)__float_as_uint(acc) << 32) | (unsigned)idx;
        }
    }
    // A list cut by tau that holds fewer than knn + margin positive distances
    // (exact copies of the query, at distance 0 and excluded like the
    // reference's d > 0 test, crowded the threshold) may miss nearer
    // distinct candidates: such a query goes to the exact fallback.
    if (!complete) {
        unsigned nv = 0;
#pragma unroll
        for (int i = 0; i < PER; ++i) nv += kv[i] != ~0ull;
        if (__reduce_add_sync(0xffffffffu, nv) < (unsigned)(knn + margin)) {
            if (lane == 0) {
                const int k = atomicAdd(scratch + 0, 1);
                scratch[irc::kScratchLists + k] = q;
            }
            return;
        }
    }
    // ws[0 .. WARP_KEYS) <- the smallest keys, ascending, selection first:
    // a bitwise search (stopped at TAU_LOW_BIT,
    // rounded up) bounds the k-th distance from above, and the keys at or
    // below that bound plus 2^-16 relative -- the band below lies inside it
    // -- are compacted into ws and sorted alone, one per lane when at most 32
    // pass (the usual case: about knn of them), else two per lane.  They are
    // the first positions of the full sort, so the result is the same; if
    // more than WARP_KEYS pass, the full sort runs.
    bool sorted = false;
    if (PER >= 2) {
        // the bits above the highest one in which the keys' distances differ
        // are common to all of them, hence the answer's: start below them
        unsigned lo = 0xffffffffu, hi = 0u;
#pragma unroll
        for (int i = 0; i < PER; ++i)
            if (kv[i] != ~0ull) {
                lo = min(lo, (unsigned)(kv[i] >> 32));
                hi = max(hi, (unsigned)(kv[i] >> 32));
            }
        lo = __reduce_min_sync(0xffffffffu, lo);
        hi = __reduce_max_sync(0xffffffffu, hi);
        unsigned ans = 0;
        int top = 30;
        if (lo <= hi) {                           // some key: distances are below 2^31 as bit patterns
            const unsigned x = lo ^ hi;
            top = x ? 31 - __clz(x) : TAU_LOW_BIT;
            ans = top < 31 ? lo & ~((2u << top) - 1u) : 0u;
            top = min(top, 30);
        }
#pragma unroll 1
        for (int b = top; b >= TAU_LOW_BIT; --b) {
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
        if (n <= 32) {                            // the common case: ~knn keys, one per lane
            unsigned long long v1[1] = {lane < n ? ws[lane] : ~0ull};
            __syncwarp();
            warp_bitonic<unsigned long long, 1>(v1, lane);
            ws[lane] = v1[0];
            ws[32 + lane] = ~0ull;
            sorted = true;
        } else if (n <= WARP_KEYS) {
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
        const double db = lane < nb ? dist2_f64(F + (size_t)ib * nC, a, nd) : 0.0;
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

constexpr int TILE = 128;

__device__ __forceinline__ int chunk_tiles(const irc::PlanDev &p, int chunk)
{
    if (chunk < 0) return 0;
    int n = 0;
    for (int r = __ldg(p.roff + chunk); r < __ldg(p.roff + chunk + 1); ++r) n += (__ldg(p.rn + r) + TILE - 1) / TILE;
    return n;
}

// Pass 1 of one warp and 128-tile (BN = 128): fold its 32 columns (taddr:
// the first) into the per-column minima; lim = valid columns of the 32.
__device__ __forceinline__ void fold32(uint32_t taddr, int lim, float (&bm)[PART])
{
    uint32_t x[16], y[16];
    sm100::tmem_ld16_nowait(taddr, x);
    sm100::tmem_ld16_nowait(taddr + 16, y);
    sm100::tmem_wait_ld(x, y);
    if (lim >= 32) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            bm[i] = fminf(bm[i], __uint_as_float(x[i]));
            bm[16 + i] = fminf(bm[16 + i], __uint_as_float(y[i]));
        }
    } else {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            if (i < lim) bm[i] = fminf(bm[i], __uint_as_float(x[i]));
            if (16 + i < lim) bm[16 + i] = fminf(bm[16 + i], __uint_as_float(y[i]));
        }
    }
}

// Pass 1 of one warp and 256-wide unit: its 32 columns of both 128-tiles
// (ta, tb: the first column of each; la, lb: valid columns) folded into the
// same minima with three-input mins.
__device__ __forceinline__ void fold2x32(uint32_t ta, int la, uint32_t tb, int lb, float (&bm)[PART])
{
    const float inf = __int_as_float(0x7f800000);
#pragma unroll
    for (int r = 0; r < 2; ++r) {                 // minima 16r .. 16r + 15
        uint32_t x[16], y[16];
        sm100::tmem_ld16_nowait(ta + 16 * r, x);
        sm100::tmem_ld16_nowait(tb + 16 * r, y);
        sm100::tmem_wait_ld(x, y);
        if (la >= 32 && lb >= 32) {
#pragma unroll
            for (int i = 0; i < 16; ++i)
                bm[16 * r + i] = sm100::fmin3(bm[16 * r + i], __uint_as_float(x[i]), __uint_as_float(y[i]));
        } else {
#pragma unroll
            for (int i = 0; i < 16; ++i)
                bm[16 * r + i] = sm100::fmin3(bm[16 * r + i], 16 * r + i < la ? __uint_as_float(x[i]) : inf,
                                              16 * r + i < lb ? __uint_as_float(y[i]) : inf);
        }
    }
}

__device__ __forceinline__ unsigned lim_mask(int lim)
{
    return lim >= 32 ? 0xffffffffu : lim <= 0 ? 0u : (1u << lim) - 1u;
}

// Pass 2 of one warp and 128-tile: the mask of its 32 columns at or below
// tau, limited to the lim valid columns.
__device__ __forceinline__ unsigned mark32(uint32_t taddr, int lim, float tau)
{
    uint32_t x[16], y[16];
    sm100::tmem_ld16_nowait(taddr, x);
    sm100::tmem_ld16_nowait(taddr + 16, y);
    sm100::tmem_wait_ld(x, y);
    // four independent partial masks: short dependency chains
    unsigned a0 = 0u, a1 = 0u, a2 = 0u, a3 = 0u;
#pragma unroll
    for (int i = 0; i < 16; i += 2) {
        if (__uint_as_float(x[i]) <= tau) a0 |= 1u << i;
        if (__uint_as_float(x[i + 1]) <= tau) a1 |= 1u << (i + 1);
        if (__uint_as_float(y[i]) <= tau) a2 |= 1u << (16 + i);
        if (__uint_as_float(y[i + 1]) <= tau) a3 |= 1u << (17 + i);
    }
    return ((a0 | a1) | (a2 | a3)) & lim_mask(lim);
}

// Bit c of the result = sign bit of v[c], one funnel shift per value in two
// independent chains.
__device__ __forceinline__ unsigned signs16(const uint32_t (&v)[16])
{
    unsigned c0 = 0u, c1 = 0u;                    // values 0-7, 8-15
#pragma unroll
    for (int i = 7; i >= 0; --i) {
        c0 = __funnelshift_l(v[i], c0, 1);
        c1 = __funnelshift_l(v[8 + i], c1, 1);
    }
    return c0 | (c1 << 8);
}

// Pass 2 with the threshold folded into the MMA (accumulators d2 - tau) of
// one warp and 256-wide unit: the masks of its 32 columns of each tile with a
// negative accumulator, limited to the valid columns.
__device__ __forceinline__ void mark2x32_signs(uint32_t ta, int la, uint32_t tb, int lb, unsigned &ma, unsigned &mb)
{
    unsigned a[2], b[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {                 // columns 16r .. 16r + 15 of both tiles
        uint32_t x[16], y[16];
        sm100::tmem_ld16_nowait(ta + 16 * r, x);
        sm100::tmem_ld16_nowait(tb + 16 * r, y);
        sm100::tmem_wait_ld(x, y);
        a[r] = signs16(x);
        b[r] = signs16(y);
    }
    ma = (a[0] | (a[1] << 16)) & lim_mask(la);
    mb = (b[0] | (b[1] << 16)) & lim_mask(lb);
}

// The pass-2 threshold of query row `row` into the query tile in shared
// memory: -tau' split exactly into three BF16 terms at K positions tau_k ..
// tau_k + 2, against 1, 1, 1 in every candidate row, so the pass-2
// accumulators are d2 - tau'.  tau' = tau (1 + 2^-10), capped at 1e30: the
// small margin keeps every candidate at or below tau negative whatever the
// rounding of the extra terms.  The tile is 128-byte swizzled: the 16-byte
// piece c of row r sits at piece c ^ (r % 8).
__device__ __forceinline__ void put_tau(uint8_t *sA, int row, int tau_k, float tau)
{
    const float x = -fminf(tau * (1.0f + 0x1p-10f), 1e30f);
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    const __nv_bfloat16 m = __float2bfloat16_rn(r1);
    const __nv_bfloat16 l = __float2bfloat16_rn(r1 - __bfloat162float(m));
    const __nv_bfloat16 v[3] = {h, m, l};
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        const int k = tau_k + t;
        __nv_bfloat16 *dst = reinterpret_cast<__nv_bfloat16 *>(sA + (size_t)row * 128 +
                                                               (((k >> 3) ^ (row & 7)) << 4) + (k & 7) * 2);
        *dst = v[t];
    }
}

// Append the hits of a 32-column mask (columns c0 + bit) to the query's
// pooled list (its four epilogue warps share it): one shared-memory atomic
// reserves the room; entries past LISTCAP are dropped, and a count past it
// sends the query to the exact fallback.
__device__ __forceinline__ void append_hits(uint32_t *lrow, int *cnt, unsigned m, uint32_t c0)
{
    int e = atomicAdd(cnt, __popc(m));
    while (m) {
        const int jj = __ffs(m) - 1;
        m &= m - 1u;
        if (e < LISTCAP) lrow[e] = c0 + (uint32_t)jj;
        ++e;
    }
}

// Named barrier 1 + slot over the slot's epilogue warps that also returns the
// AND of v over them: every warp of the slot gets the same answer, so they
// leave the item loop together (a warp that left alone would leave the others
// waiting at the slot's next barrier).
__device__ __forceinline__ bool slot_barrier_and(int slot, int nthreads, bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + slot), "r"(nthreads)
        : "memory");
    return r != 0;
}

// The handoff of one item's lists to the re-rank kernel: this warp packs 8 of
// its quarter's queries (query L in lane L) into one bump allocation and
// records (offset, length) per query; a list past LISTCAP or a full list area
// sends the query to the exact fallback instead.
__device__ __forceinline__ void hand_off(const irc::PlanDev &p, const irc_tc::TcItem &it, int s, int quarter, int part,
                                         int qrow, int nq_s, const uint32_t *lists, const int *sCnt,
                                         const irc_tc::ListOut &lo, int *scratch, int lane)
{
    constexpr int RL = 32 / PARTS;
    int cL = -1;                                  // -1: no query in this lane, -2: to the fallback
    if (lane < RL && qrow + part * RL + lane < nq_s) {
        const int t = sCnt[quarter * 32 + part * RL + lane];
        cL = t > LISTCAP ? -2 : t;
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
        const uint32_t *lr = lists + (size_t)(quarter * 32 + part * RL + L) * LROW;
        for (int e = lane; e < n; e += 32) lo.lists[off + e] = lr[e];
    }
}

// Shared state of a persistent filter CTA: the item ring (the producer claims
// items from the launch's work queue and publishes their indices), the
// double-buffered query tile and the mbarriers of every stage.
struct Shared {
    uint8_t *sA;                                  // two query tiles, A_BYTES each
    uint8_t *sB;                                  // candidate stages
    uint32_t *lists;                              // [BM][LROW]
    float *sTau;                                  // [BM]
    int *sCnt;                                    // [BM] list counts
    uint64_t *full, *empty;                       // [STAGES] candidate stages loaded / consumed
    uint64_t *a_full, *a_empty;                   // [2] query tile loaded / its item's MMAs done
    uint64_t *acc_full, *acc_empty;               // [NBUF] accumulator written / read
    uint64_t *tau_ready;                          // [4] a slot's thresholds are in its query tile
    uint64_t *item_full, *item_empty;             // [2] item index published / read by every consumer
    uint64_t *mma_done;
    int *item_idx;                                // [2]
    uint32_t *tmem_slot;
    volatile int *abort_flag;
};

// Epilogue of one warp: lane quarter `quarter` (the TMEM lanes it may read)
// and part `part` (columns 32 * part .. 32 * part + 31 of every 128-tile of
// its slot), over the items the CTA takes.  Each slot's epilogue warps
// synchronise only among themselves (named barrier 1 + slot).  Unit g of a
// slot (counted over all its items, both passes) goes to accumulator
// s * BPS + g % BPS, whose barriers are in phase g / BPS.
template <int BN, int NS, bool TAU>
__device__ __forceinline__ void epilogue(const irc::PlanDev &p, const irc_tc::TcItem *__restrict__ items, int rank,
                                         uint32_t tmem, int tau_k, const Shared &sh, const irc_tc::ListOut &lo,
                                         int *scratch, int warp, int lane)
{
    using T = Tile<BN>;
    constexpr int QPS = 4 / NS;                   // lane quarters per slot
    constexpr int BPS = T::NBUF / NS;             // accumulator buffers per slot
    const int ew = warp - 2;                      // 0..15
    const int quarter = warp & 3;                 // TMEM lane quarter this warp may access
    const int part = ew >> 2;                     // its 32 columns of every 128-tile
    const int s = quarter / QPS;                  // slot of this lane quarter
    const int qrow = (quarter % QPS) * 32;        // first row of this quarter inside its slot
    const int slot_threads = 32 * PARTS * QPS;
    const int row = quarter * 32 + lane;
    const uint32_t tbase = tmem + ((uint32_t)(quarter * 32) << 16) + part * PART;
    // the minima rows of a quarter alias that quarter's own list rows
    float *qarea = reinterpret_cast<float *>(sh.lists + (size_t)quarter * 32 * LROW);
    uint32_t *lrow = sh.lists + (size_t)row * LROW;
    unsigned g0 = 0;                              // this slot's units of the earlier items
    for (int seq = 0;; ++seq) {
        const int r = seq & 1;
        bool ok = pipe_wait(&sh.item_full[r], (seq >> 1) & 1, sh.abort_flag);
        if (!slot_barrier_and(s, slot_threads, ok)) break;
        const int idx = sh.item_idx[r];
        __syncwarp();
        if (lane == 0) sm100::mbar_arrive(&sh.item_empty[r]);
        if (idx < 0) break;                       // the queue is empty
        const irc_tc::TcItem it = items[idx];
        const int nq_s = it.chunk[s] >= 0 ? it.nq[s] : 0;
        const int nts = chunk_tiles(p, it.chunk[s]);
        const bool active = qrow < nq_s;          // warp-uniform: any valid query in this quarter
        const int U = units_per_pass<BN>(nts);
        // the slot's tile list: unit u is tile u (BN = 128) or tiles 2u, 2u + 1
        // (BN = 256; the second is (0, 0) past the end of an odd count)
        const int2 *tl = nts ? p.tc_tiles + __ldg(p.tc_toff + it.chunk[s]) : p.tc_tiles;

        // Unit k of the two passes: (first row, columns) of its tile(s), loaded
        // one unit ahead of its use.
        auto load_unit = [&](int k) -> int4 {
            const int u = k < U ? k : k - U;
            if constexpr (BN == 256) {
                return __ldg(reinterpret_cast<const int4 *>(tl) + u);
            } else {
                const int2 v = __ldg(tl + u);
                return make_int4(v.x, v.y, 0, 0);
            }
        };
        int4 cu = U ? load_unit(0) : make_int4(0, 0, 0, 0);
        // this warp's columns of the unit: first rows ra, rb and valid counts
        // na, nb of its 32 columns in each tile (none: <= 0)
        auto unit = [&](int k, int &ra, int &na, int &rb, int &nb) {
            const int4 nx = load_unit(k + 1 < 2 * U ? k + 1 : k);
            ra = cu.x;
            na = cu.y - part * PART;
            rb = cu.z;
            nb = cu.w - part * PART;
            cu = nx;
        };

        // pass 1: per-column minima of this warp's columns
        float bm[PART];
#pragma unroll
        for (int c = 0; c < PART; ++c) bm[c] = __int_as_float(0x7f800000);
        for (int k = 0; k < U && ok; ++k) {
            int ra, na, rb, nb;
            unit(k, ra, na, rb, nb);
            const unsigned g = g0 + (unsigned)k;
            const int b = s * BPS + (int)(g % BPS);
            if (!(ok = pipe_wait(&sh.acc_full[b], (g / BPS) & 1, sh.abort_flag))) break;
            sm100::tc_fence_after();
            if (active) {
                if constexpr (BN == 256) {
                    // either tile may be the short one (the first when it ends a run)
                    if (na > 0 || nb > 0) fold2x32(tbase + b * BN, na, tbase + b * BN + 128, nb, bm);
                } else {
                    if (na > 0) fold32(tbase + b * BN, na, bm);
                }
            }
            sm100::tc_fence_before();
            __syncwarp();
            if (lane == 0) sm100::mbar_arrive(&sh.acc_empty[b]);
        }
        // threshold: rank-th smallest of the 128 column minima of every query
        {
            float *brow = qarea + lane * BROW + part * PART;
#pragma unroll
            for (int c = 0; c < PART; ++c) brow[c] = fmaxf(bm[c], 0.0f);
            if (part == 0) sh.sCnt[row] = 0;      // list counts of pass 2 (ordered by the barriers below)
            slot_barrier(s, slot_threads);
            // The warp's 8 rows at once (independent chains): a bitwise
            // search, from the top, of the largest t with fewer than rank
            // minima below it, i.e. of the rank-th smallest minimum, on the
            // non-negative float bit patterns.  It stops at bit lowb and
            // rounds up, so tau is an upper bound of the rank-th smallest
            // within 2^-(lowb - 1) relative of it (a few more candidates
            // listed, never fewer).  The search is a fixed cost per item,
            // the extra candidates a cost per tile: slots of at most 16
            // tiles stop 4 bits earlier (2^-7), longer ones search to 2^-11.
            constexpr int RL = 32 / PARTS;
            unsigned v4[RL][4], ans[RL];
#pragma unroll
            for (int L = 0; L < RL; ++L) {
                const float *bl = qarea + (part * RL + L) * BROW;
#pragma unroll
                for (int u = 0; u < 4; ++u) v4[L][u] = __float_as_uint(bl[u * 32 + lane]);
                ans[L] = 0u;
            }
            const int lowb = nts <= 16 ? TAU_LOW_BIT + 4 : TAU_LOW_BIT;   // uniform over the slot
#pragma unroll 1
            for (int b = 30; b >= lowb; --b) {
#pragma unroll
                for (int L = 0; L < RL; ++L) {
                    const unsigned t = ans[L] | (1u << b);
                    const unsigned c = (unsigned)(v4[L][0] < t) + (unsigned)(v4[L][1] < t) +
                                       (unsigned)(v4[L][2] < t) + (unsigned)(v4[L][3] < t);
                    if (__reduce_add_sync(0xffffffffu, c) < (unsigned)rank) ans[L] = t;
                }
            }
            if (lane < RL) {
                unsigned a = ans[0];
#pragma unroll
                for (int L = 1; L < RL; ++L)
                    if (lane == L) a = ans[L];
                sh.sTau[quarter * 32 + part * RL + lane] =
                    __uint_as_float(min(a | ((1u << lowb) - 1u), 0x7f800000u));
            }
            slot_barrier(s, slot_threads);        // minima rows are read; the list rows may be written
        }
        const float tau = sh.sTau[row];
        if (TAU && part == 0 && U > 0) {
            // the thresholds into the item's query tile; visible to the tensor
            // core (async proxy) before the MMA thread, released by tau_ready,
            // issues the slot's pass-2 MMAs (one phase per item with units)
            put_tau(sh.sA + (size_t)r * A_BYTES, row, tau_k, tau);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) sm100::mbar_arrive(&sh.tau_ready[s]);
        }
        // pass 2: collect the candidates at or below tau
        for (int k = U; k < 2 * U && ok; ++k) {
            int ra, na, rb, nb;
            unit(k, ra, na, rb, nb);
            const unsigned g = g0 + (unsigned)k;
            const int b = s * BPS + (int)(g % BPS);
            if (!(ok = pipe_wait(&sh.acc_full[b], (g / BPS) & 1, sh.abort_flag))) break;
            sm100::tc_fence_after();
            if (active && (na > 0 || nb > 0)) {
                unsigned ma = 0u, mb = 0u;
                if constexpr (BN == 256 && TAU) {
                    mark2x32_signs(tbase + b * BN, na, tbase + b * BN + 128, nb, ma, mb);
                } else {
                    if (na > 0) ma = mark32(tbase + b * BN, na, tau);
                    if (BN == 256 && nb > 0) mb = mark32(tbase + b * BN + 128, nb, tau);
                }
                if (ma) append_hits(lrow, sh.sCnt + row, ma, (uint32_t)(ra + part * PART));
                if (mb) append_hits(lrow, sh.sCnt + row, mb, (uint32_t)(rb + part * PART));
            }
            sm100::tc_fence_before();
            __syncwarp();
            if (lane == 0) sm100::mbar_arrive(&sh.acc_empty[b]);
        }
        slot_barrier(s, slot_threads);
        if (__all_sync(0xffffffffu, ok)) hand_off(p, it, s, quarter, part, qrow, nq_s, sh.lists, sh.sCnt, lo, scratch, lane);
        g0 += 2u * (unsigned)U;
        // every warp of the slot is done with this item's lists before the
        // next item's minima overwrite them; after a timed-out wait all stop
        if (!slot_barrier_and(s, slot_threads, ok && !*sh.abort_flag)) break;
    }
}

// TMA producer (one thread): claims items from the launch's work queue and
// publishes their indices (a two-entry ring), loads each item's four 32-row
// query boxes into the free query tile, then the slots' units round-robin,
// each slot's sequence twice (both passes).  A unit's 128-candidate tiles land
// in consecutive 128-row halves of its stage.  Stage and tile counters run on
// across items, so the ring never drains between them.
template <int BN, int NS>
__device__ __forceinline__ void produce(const CUtensorMap &tmQ, const CUtensorMap &tmC, const irc::PlanDev &p,
                                        const irc_tc::TcItem *__restrict__ items, int n_items, unsigned *queue,
                                        const Shared &sh)
{
    using T = Tile<BN>;
    constexpr int QPS = 4 / NS;
    sm100::prefetch_tmap(&tmQ);
    sm100::prefetch_tmap(&tmC);
    int i = 0, n_a = 0;                           // candidate stages and query tiles loaded
    bool ok = true;
    for (int seq = 0; ok; ++seq) {
        const int r = seq & 1;
        const unsigned claim = atomicAdd(queue, 1u);
        const int idx = claim < (unsigned)n_items ? (int)claim : -1;
        if (!(ok = pipe_wait(&sh.item_empty[r], ((seq >> 1) & 1) ^ 1, sh.abort_flag))) break;
        sh.item_idx[r] = idx;
        sm100::mbar_arrive(&sh.item_full[r]);     // release: the index is visible to the waiters
        if (idx < 0) break;
        const irc_tc::TcItem it = items[idx];
        const int2 *tl[NS];
        int U[NS], nt[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            nt[s] = chunk_tiles(p, it.chunk[s]);
            U[s] = units_per_pass<BN>(nt[s]);
            tl[s] = nt[s] ? p.tc_tiles + __ldg(p.tc_toff + it.chunk[s]) : p.tc_tiles;
        }
        // the query tile of item seq - 2 is free once that item's MMAs are done
        if (!(ok = pipe_wait(&sh.a_empty[r], ((seq >> 1) & 1) ^ 1, sh.abort_flag))) break;
        uint8_t *sA = sh.sA + (size_t)r * A_BYTES;
        sm100::mbar_arrive_expect_tx(&sh.a_full[r], A_BYTES);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int s = q / QPS;
            const int row0 = it.chunk[s] >= 0 ? it.qs[s] + (q % QPS) * 32 : 0;
            sm100::tma_load_2d(&tmQ, &sh.a_full[r], sA + q * (A_BYTES / 4), 0, row0);
        }
        ++n_a;
        for (int k = 0; ok; ++k) {
            bool any = false;
#pragma unroll
            for (int s = 0; s < NS; ++s) {
                if (ok && k < 2 * U[s]) {
                    any = true;
                    const int u = k % U[s];
                    const int st = i % T::STAGES;
                    if ((ok = pipe_wait(&sh.empty[st], ((i / T::STAGES) & 1) ^ 1, sh.abort_flag))) {
                        uint8_t *dst = sh.sB + (size_t)st * T::STAGE_BYTES;
                        const int nh = BN == 256 && 2 * u + 1 < nt[s] ? 2 : 1;   // 128-tiles of the unit
                        sm100::mbar_arrive_expect_tx(&sh.full[st], nh * HALF_BYTES);
                        for (int h = 0; h < nh; ++h) {
                            const int row0 = __ldg(tl[s] + (BN == 256 ? 2 * u + h : u)).x;
                            sm100::tma_load_2d(&tmC, &sh.full[st], dst + h * HALF_BYTES, 0, row0);
                        }
                        ++i;
                    }
                }
            }
            if (!any) break;
        }
    }
    // every issued load has landed before the CTA exits
    for (int j = (i > T::STAGES ? i - T::STAGES : 0); j < i; ++j)
        sm100::mbar_drain(&sh.full[j % T::STAGES], (j / T::STAGES) & 1);
    for (int j = (n_a > 2 ? n_a - 2 : 0); j < n_a; ++j) sm100::mbar_drain(&sh.a_full[j & 1], (j >> 1) & 1);
}

// MMA issuer (one thread), in the producer's order; unit g of slot s (counted
// over the CTA's items) goes to accumulator s*BPS + g % BPS and is issued once
// every epilogue warp of the slot released unit g - BPS of that buffer.  With
// TAU the slot's first pass-2 unit of an item also waits until its epilogue
// wrote the thresholds into the query tile (tau_ready[s], one phase per item
// in which the slot has units).  After an item's last MMA a commit frees its
// query tile.
template <int BN, int NS, bool FP8, bool TAU>
__device__ __forceinline__ void issue(const irc::PlanDev &p, const irc_tc::TcItem *__restrict__ items, int nk,
                                      uint32_t tmem, const Shared &sh)
{
    using T = Tile<BN>;
    constexpr int BPS = T::NBUF / NS;
    // bf16 x bf16 (kind::f16, K = 16) or e4m3 x e4m3 (kind::f8f6f4, K = 32) -> f32;
    // either way one MMA consumes 32 bytes of every 128-byte operand row
    constexpr uint32_t idesc = FP8 ? sm100::idesc_make(BM, BN, 0, 0) : sm100::idesc_make(BM, BN, 1, 1);
    unsigned g0[NS], taus[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) g0[s] = taus[s] = 0;
    int i = 0;
    bool ok = true;
    for (int seq = 0; ok; ++seq) {
        const int r = seq & 1;
        if (!(ok = pipe_wait(&sh.item_full[r], (seq >> 1) & 1, sh.abort_flag))) break;
        const int idx = sh.item_idx[r];
        sm100::mbar_arrive(&sh.item_empty[r]);
        if (idx < 0) break;
        const irc_tc::TcItem it = items[idx];
        int U[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) U[s] = units_per_pass<BN>(chunk_tiles(p, it.chunk[s]));
        if (!(ok = pipe_wait(&sh.a_full[r], (seq >> 1) & 1, sh.abort_flag))) break;
        sm100::tc_fence_after();
        const uint64_t adesc = sm100::sdesc_sw128(sm100::smem_u32(sh.sA + (size_t)r * A_BYTES));
        for (int k = 0; ok; ++k) {
            bool any = false;
#pragma unroll
            for (int s = 0; s < NS; ++s) {
                if (ok && k < 2 * U[s]) {
                    any = true;
                    const unsigned g = g0[s] + (unsigned)k, use = g / BPS;
                    const int b = s * BPS + (int)(g % BPS), st = i % T::STAGES;
                    ok = (use == 0 || pipe_wait(&sh.acc_empty[b], (use - 1) & 1, sh.abort_flag)) &&
                         pipe_wait(&sh.full[st], (i / T::STAGES) & 1, sh.abort_flag) &&
                         // the slot's thresholds are in the query tile before its pass 2
                         (!TAU || k != U[s] || pipe_wait(&sh.tau_ready[s], taus[s] & 1, sh.abort_flag));
                    if (ok) {
                        sm100::tc_fence_after();
                        const uint64_t bdesc =
                            sm100::sdesc_sw128(sm100::smem_u32(sh.sB + (size_t)st * T::STAGE_BYTES));
#pragma unroll
                        for (int kk = 0; kk < KP / 16; ++kk)
                            if (kk >= nk)
                                break;                    // the rest of every operand row is zero
                            else if (FP8)
                                sm100::mma_f8(tmem + b * BN, adesc + 2 * kk, bdesc + 2 * kk, idesc, kk > 0 ? 1u : 0u);
                            else
                                sm100::mma_f16(tmem + b * BN, adesc + 2 * kk, bdesc + 2 * kk, idesc, kk > 0 ? 1u : 0u);
                        sm100::mma_commit(&sh.empty[st]);
                        sm100::mma_commit(&sh.acc_full[b]);
                        ++i;
                    }
                }
            }
            if (!any) break;
        }
        if (!ok) break;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            g0[s] += 2u * (unsigned)U[s];
            taus[s] += U[s] > 0 ? 1u : 0u;
        }
        sm100::mma_commit(&sh.a_empty[r]);        // this item's MMAs done: its query tile may be replaced
    }
    // every MMA has completed before TMEM is released
    sm100::mma_commit(sh.mma_done);
    sm100::mbar_drain(sh.mma_done, 0);
}

// The filter over the work items of one packing class (NS slots per item:
// one or two at BN = 256, four at BN = 128), persistent: each CTA takes items
// from the class's work queue (queue: its head, items cost-ordered) until it
// is empty.  TAU: pass 2 reads the signs of d2 - tau (the thresholds written
// into the query tile at K position tau_k), else it compares d2 with tau in
// the epilogue.
template <bool FP8, int BN, bool TAU, int NS>
__global__ void __launch_bounds__(THREADS, 1)
k_knn_tc(const __grid_constant__ CUtensorMap tmQ, const __grid_constant__ CUtensorMap tmC, irc::PlanDev p,
         const irc_tc::TcItem *__restrict__ items, int n_items, unsigned *queue, int nk, int tau_k, irc_tc::ListOut lo,
         int *__restrict__ scratch)
{
    using T = Tile<BN>;
    constexpr int QPS = 4 / NS;
    extern __shared__ unsigned char smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    Shared sh;
    sh.sA = base;
    sh.sB = base + 2 * A_BYTES;
    sh.lists = reinterpret_cast<uint32_t *>(sh.sB + T::STAGES * T::STAGE_BYTES);   // [BM][LROW]
    sh.sTau = reinterpret_cast<float *>(sh.lists + (size_t)LROW * BM);
    sh.sCnt = reinterpret_cast<int *>(sh.sTau + BM);
    uint64_t *bars = reinterpret_cast<uint64_t *>(sh.sCnt + BM);
    sh.full = bars;
    sh.empty = sh.full + T::STAGES;
    sh.a_full = sh.empty + T::STAGES;
    sh.a_empty = sh.a_full + 2;
    sh.acc_full = sh.a_empty + 2;
    sh.acc_empty = sh.acc_full + T::NBUF;
    sh.tau_ready = sh.acc_empty + T::NBUF;
    sh.item_full = sh.tau_ready + 4;
    sh.item_empty = sh.item_full + 2;
    sh.mma_done = sh.item_empty + 2;
    sh.item_idx = reinterpret_cast<int *>(sh.mma_done + 1);
    sh.tmem_slot = reinterpret_cast<uint32_t *>(sh.item_idx + 2);
    sh.abort_flag = reinterpret_cast<volatile int *>(sh.tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < T::STAGES; ++s) { sm100::mbar_init(&sh.full[s], 1); sm100::mbar_init(&sh.empty[s], 1); }
        for (int r = 0; r < 2; ++r) {
            sm100::mbar_init(&sh.a_full[r], 1);
            sm100::mbar_init(&sh.a_empty[r], 1);
            sm100::mbar_init(&sh.item_full[r], 1);
            sm100::mbar_init(&sh.item_empty[r], 1 + EPI_WARPS);   // the MMA thread and every epilogue warp
        }
        for (int b = 0; b < T::NBUF; ++b) {
            sm100::mbar_init(&sh.acc_full[b], 1);
            sm100::mbar_init(&sh.acc_empty[b], PARTS * QPS);       // the slot's epilogue warps
        }
        sm100::mbar_init(sh.mma_done, 1);
        for (int s = 0; s < 4; ++s) sm100::mbar_init(&sh.tau_ready[s], QPS);   // the slot's quarters' writers
        *sh.abort_flag = 0;
        sm100::fence_mbar_init();
    }
    if (warp == 1) sm100::tmem_alloc(sh.tmem_slot, TMEM_COLS);
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    const uint32_t tmem = *sh.tmem_slot;

    if (warp == 0) {
        if (lane == 0) produce<BN, NS>(tmQ, tmC, p, items, n_items, queue, sh);
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) issue<BN, NS, FP8, TAU>(p, items, nk, tmem, sh);
        __syncwarp();
    } else {
        epilogue<BN, NS, TAU>(p, items, tau_rank(FP8), tmem, tau_k, sh, lo, scratch, warp, lane);
    }
    sm100::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        sm100::tc_fence_after();
        sm100::tmem_dealloc(tmem, TMEM_COLS);
    }
    if (threadIdx.x == 0 && *sh.abort_flag) atomicExch(scratch + irc::kScratchErr, 1);
}

// Exact re-rank kernel: one warp per query of the plan, in query order (the
// queries of a chunk share their candidate rows, which stay in L1/L2 for the
// block's warps); queries without a list (qinfo.x < 0) belong to the exact
// fallback or to no chunk.
constexpr int RR_WARPS = 8;

__global__ void __launch_bounds__(32 * RR_WARPS, 4)
k_rerank(const int2 *__restrict__ qinfo, const uint32_t *__restrict__ lists, int n_out, int q_base,
         const float *__restrict__ F, const float4 *__restrict__ Fp, int nC, const uint8_t *__restrict__ row_dims,
         int knn, float *__restrict__ vrKnn, float *__restrict__ rho, int *__restrict__ miKnn,
         float *__restrict__ d2Knn, int margin, int *__restrict__ scratch)
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
    const int nd = row_dims ? min(nC, (int)__ldg(row_dims + q)) : nC;
    const bool complete = (qi.y >> 30) & 1;
    unsigned long long *ws = wkeys + warp * WARP_KEYS;
    float4 *qs = qrows + warp * QROW4;
    if (cL <= 64)
        rerank<2>(lst, cL, complete, q, F, Fp, Dp4, qs, nC, nd, knn, (size_t)o, ws, lane, margin, miKnn, d2Knn, vrKnn, rho,
                  scratch);
    else if (cL <= 128)
        rerank<4>(lst, cL, complete, q, F, Fp, Dp4, qs, nC, nd, knn, (size_t)o, ws, lane, margin, miKnn, d2Knn, vrKnn, rho,
                  scratch);
    else
        rerank<8>(lst, cL, complete, q, F, Fp, Dp4, qs, nC, nd, knn, (size_t)o, ws, lane, margin, miKnn, d2Knn, vrKnn, rho,
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

template <bool FP8, int BN, bool TAU, int NS>
static int launch_filter(const CUtensorMap &mq, const CUtensorMap &mc, irc_plan *pl, const irc_tc::TcItem *items,
                         int n_items, unsigned *queue, int nk, int tau_k, const ListOut &lo, cudaStream_t s)
{
    if (n_items <= 0) return IRC_OK;
    auto kern = k_knn_tc<FP8, BN, TAU, NS>;
    const int smem = (int)Tile<BN>::SMEM_BYTES;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, pl->device);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(tensor core): launch attributes");
    // persistent: one CTA per SM (shared memory and TMEM allow one), each
    // taking items from the queue until it is empty
    const int grid = n_items < sms ? n_items : sms;
    kern<<<grid, THREADS, smem, s>>>(mq, mc, pl->dev, items, n_items, queue, nk, tau_k, lo, pl->scratch);
    IRC_CHECK_LAUNCH("irc_site_knn(tensor core)");
    return IRC_OK;
}

int launch_knn_tc(bool fp8, const CUtensorMap &mq, const CUtensorMap &mc, irc_plan *pl, const float *F,
                  const float4 *Fp, int nC, int knn, float *vrKnn, float *rho, int32_t *miKnn, float *d2Knn,
                  const ListOut &lo, cudaStream_t s)
{
    const int n_out = pl->dev.n_out;
    cudaError_t e = cudaMemsetAsync(lo.qinfo, 0xff, (size_t)n_out * sizeof(int2), s);   // (-1, -1): no list
    if (e == cudaSuccess) e = cudaMemsetAsync(lo.count, 0, 4 * sizeof(unsigned), s);     // count, queue heads
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(tensor core): memset");
    // BF16: the pass-2 thresholds go into K positions nC + 6 .. nC + 8 of the
    // query rows when they fit (else, and for FP8, pass 2 compares in the
    // epilogue).  MMAs per unit: only the 32-byte K slices that hold data
    // (nC features, 6 BF16 / 12 FP8 norm entries, the threshold terms).
    const int tau_k = (!fp8 && nC + 9 <= KP) ? nC + 6 : -1;
    const int used = fp8 ? nC + 12 : 2 * (nC + (tau_k >= 0 ? 9 : 6));
    const int nk = (used + 31) / 32;
    cudaEvent_t *ev = profile_slot();
    if (ev) cudaEventRecord(ev[0], s);
    // one persistent launch per packing class: one-slot and two-slot items on
    // 256-candidate units (or 128, irc_plan_tc_units), then four-slot items
    // on 128.  The threshold goes into the MMA only on 256-wide units; the
    // narrower ones compare in the epilogue.  Four-slot items (small chunks)
    // keep the compare: their CTAs are short, and waiting for the thresholds
    // before the pass-2 MMAs would put the threshold step on their critical
    // path.  Neither the width nor the packing changes the results.
    const int n1 = pl->n_tc_one, n2 = pl->n_tc_wide - pl->n_tc_one, n4 = pl->n_tc_items - pl->n_tc_wide;
    const irc_tc::TcItem *it1 = pl->tc_items, *it2 = it1 + n1, *it4 = it2 + n2;
    const bool narrow = pl->tc_wide_bn == 128;
    using yes = std::true_type;
    using no = std::false_type;
    auto run = [&](auto tau_c) {
        constexpr bool T = decltype(tau_c)::value;
        int r;
        if (narrow)
            r = fp8 ? launch_filter<true, 128, false, 1>(mq, mc, pl, it1, n1, lo.count + 1, nk, tau_k, lo, s)
                    : launch_filter<false, 128, false, 1>(mq, mc, pl, it1, n1, lo.count + 1, nk, tau_k, lo, s);
        else
            r = fp8 ? launch_filter<true, 256, false, 1>(mq, mc, pl, it1, n1, lo.count + 1, nk, tau_k, lo, s)
                    : launch_filter<false, 256, T, 1>(mq, mc, pl, it1, n1, lo.count + 1, nk, tau_k, lo, s);
        if (r != IRC_OK) return r;
        if (narrow)
            r = fp8 ? launch_filter<true, 128, false, 2>(mq, mc, pl, it2, n2, lo.count + 2, nk, tau_k, lo, s)
                    : launch_filter<false, 128, false, 2>(mq, mc, pl, it2, n2, lo.count + 2, nk, tau_k, lo, s);
        else
            r = fp8 ? launch_filter<true, 256, false, 2>(mq, mc, pl, it2, n2, lo.count + 2, nk, tau_k, lo, s)
                    : launch_filter<false, 256, T, 2>(mq, mc, pl, it2, n2, lo.count + 2, nk, tau_k, lo, s);
        if (r != IRC_OK) return r;
        return fp8 ? launch_filter<true, 128, false, 4>(mq, mc, pl, it4, n4, lo.count + 3, nk, tau_k, lo, s)
                   : launch_filter<false, 128, false, 4>(mq, mc, pl, it4, n4, lo.count + 3, nk, tau_k, lo, s);
    };
    const int rc = tau_k >= 0 ? run(yes{}) : run(no{});
    if (rc != IRC_OK) return rc;
    if (ev) cudaEventRecord(ev[1], s);
    k_rerank<<<(n_out + RR_WARPS - 1) / RR_WARPS, 32 * RR_WARPS, 0, s>>>(
        lo.qinfo, lo.lists, n_out, pl->dev.q_base, F, Fp, nC, pl->row_dims, knn, vrKnn, rho, miKnn, d2Knn,
        crowd_margin(fp8), pl->scratch);
    IRC_CHECK_LAUNCH("irc_site_knn(tensor core) re-rank");
    if (ev) cudaEventRecord(ev[2], s);
    return IRC_OK;
}

}  // namespace irc_tc

extern "C" {

int irc_set_wait_limit(int polls)
{
    const uint32_t v = polls > 0 ? (uint32_t)polls : (1u << 22);
    cudaError_t e = cudaMemcpyToSymbol(c_wait_polls, &v, sizeof(v));
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_set_wait_limit");
    return IRC_OK;
}

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
