// irc_plan.cuh -- device-resident launch plan of one site (internal).
#pragma once
#include "irc_common.cuh"

namespace irc {

// Plan scratch words: [0] overflow-queue count, [1] delta-fallback count,
// [2] device error word (a bounded wait gave up), [3] unused; the two query
// lists of n_out entries follow.
constexpr int kScratchErr = 2;
constexpr int kScratchItems = 3;      // count of delta-fallback (chunk, tile) items
constexpr int kScratchLists = 4;

// Query-tile sizes for which a plan precomputes its tile tables.
constexpr int kTileSizes[] = {8, 16, 32, 64, 128};
constexpr int kNumTileSizes = 5;

__host__ __device__ constexpr int tile_slot(int qb)
{
    return qb == 8 ? 0 : qb == 16 ? 1 : qb == 32 ? 2 : qb == 64 ? 3 : 4;
}

// Work item of the tensor-core kNN: up to four slots packed into one 128-row
// tile; slot s covers queries [qs[s], qs[s]+nq[s]) of chunk[s] (chunk < 0:
// empty) and 128/nslot rows of the tile.
struct TcItem {
    int nslot;
    int chunk[4];
    int qs[4];
    int nq[4];
    int pad[3];
};
static_assert(sizeof(TcItem) == 64, "TcItem is 16 words");

// Plain device pointers into one allocation owned by irc_plan.
// roff/rs/rn: every chunk's candidate set as maximal contiguous row intervals
// (adjacent linked runs merged); roffr/rsr/rnr: the runs exactly as the
// reference passes them (IBB/NBB), which the REF kernels' bins depend on.
struct PlanDev {
    const int32_t *q0, *nq, *roff, *rs, *rn;
    const int32_t *roffr, *rsr, *rnr;
    const int32_t *tile_off[kNumTileSizes];   // [nChunks+1] prefix sums of ceil(nq/QB)
    const int32_t *ncand;                     // [nChunks] candidates of each chunk (sum of its runs)
    // 128-candidate tiles of every chunk's intervals for the tensor-core
    // filter: tile j of chunk c is tc_tiles[tc_toff[c] + j] = (first row,
    // columns); each chunk's list is padded to an even length with (0, 0),
    // so a 256-wide unit is one aligned int4.  Null in plans without it.
    const int32_t *tc_toff;                   // [nChunks+1]
    const int2 *tc_tiles;
    int nChunks, q_base, n_out, nF, nRuns;
};

// Map a flat tile id to (chunk, first query, query count) for tile size QB.
template <int QB>
__device__ __forceinline__ void tile_lookup(const PlanDev &p, int tile, int &chunk, int &qs, int &n)
{
    const int32_t *to = p.tile_off[tile_slot(QB)];
    int lo = 0, hi = p.nChunks;            // find chunk with to[chunk] <= tile < to[chunk+1]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (__ldg(to + mid) <= tile) lo = mid; else hi = mid;
    }
    chunk = lo;
    const int qt = tile - __ldg(to + lo);
    qs = __ldg(p.q0 + lo) + qt * QB;
    n = min(QB, __ldg(p.nq + lo) - qt * QB);
}

}  // namespace irc

struct irc_plan {
    irc::PlanDev dev;
    void *dmem;                            // single device allocation behind dev
    int32_t *scratch;                      // inside dmem: 4 words + 2 x n_out query lists
    const irc::TcItem *tc_items;           // tensor-core work items: inside dmem, or tc_items_buf
    int n_tc_items;
    int n_tc_one;                          // items [0, n_tc_one) have one slot, [n_tc_one, n_tc_wide) two
    int n_tc_wide;                         // (both on 256-candidate units), the rest four (128-candidate units)
    int tc_wide_bn;                        // unit width of the one- and two-slot items: 256 (0 = default) or 128
    uint8_t *row_dims;                     // [nF] features of each row's site (irc_plan_set_site_dims) or null
    void *tc_items_buf;                    // items of irc_plan_tc_layout, when called
    void *tc_buf;                          // tensor-core operand rows (2 x nF x tc_row_bytes) and the
                                           // padded FP32 rows of the re-rank, allocated lazily
    size_t tc_row_bytes;
    size_t tc_bytes;                       // allocated size of tc_buf
    int tc_external;                       // tc_buf belongs to the caller (irc_plan_set_tc_buffer)
    int n_row_iv;                          // rows of F the plan reads: n_row_iv intervals
    int row_iv[2 * 8];                     // [lo, hi) pairs, ascending (at most 8; else one hull)
    int ntiles[irc::kNumTileSizes];        // host copy of tile counts
    int max_nq;                            // largest query chunk
    long long pairs;                       // (query, candidate) pairs of the plan
    int device;
    // host copies (for the per-chunk drop-in emulation and validation)
    int32_t *h_q0, *h_nq, *h_roff, *h_rs, *h_rn;
};
