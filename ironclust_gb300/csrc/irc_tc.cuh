// irc_tc.cuh -- shared constants of the tensor-core kNN (internal).
#pragma once
#include <cuda.h>

#include "irc_plan.cuh"

namespace irc_tc {

constexpr int BM = 128;          // queries per CTA (TMEM lanes)
constexpr int KP = 64;           // padded feature dimension (bf16 elements, one 128-byte row)
constexpr int KNN_MAX = 32;      // largest knn served (candidate lists hold >= 64 for the re-rank)
constexpr int LIST_MAX = 256;    // longest candidate list re-ranked (else: the exact fallback)
constexpr int LIST_AVG = 128;    // list area per plan: LIST_AVG entries per query
using TcItem = irc::TcItem;

// The re-rank's FP32 copy of a feature row, zero-padded to a multiple of 8
// floats (32 bytes) so that it is read with whole-sector 256-bit loads:
// width in float4.
inline __host__ __device__ int fp_row4(int nC) { return 2 * ((nC + 7) / 8); }

// Candidate lists handed from the filter kernel to the re-rank kernel:
// qinfo[o] = (offset into lists, length) of query q_base + o, or (-1, -1);
// lists packed by a bump allocator (count) of cap entries.
struct ListOut {
    int2 *qinfo;
    uint32_t *lists;
    unsigned *count;             // count[0]: list entries used; count[1..3]: work-queue heads of the
    unsigned cap;                // filter's one-, two- and four-slot launches
};

// Entries of the list area of a plan with n_out queries (offsets are int32).
inline size_t list_cap(long long n_out)
{
    const size_t c = (size_t)n_out * LIST_AVG, m = (size_t)0x7fffff00;
    return c < m ? c : m;
}

// Bytes of the list area of a plan with n_out queries (qinfo, the count and
// the filter's three work-queue counters in one 256-byte block, lists).
inline size_t list_area_bytes(long long n_out)
{
    return (((size_t)n_out * 8 + 255) & ~(size_t)255) + 256 + list_cap(n_out) * 4;
}

inline ListOut list_area(void *base, long long n_out)
{
    ListOut lo;
    char *b = (char *)base;
    lo.qinfo = (int2 *)b;
    b += ((size_t)n_out * 8 + 255) & ~(size_t)255;
    lo.count = (unsigned *)b;
    lo.lists = (uint32_t *)(b + 256);
    lo.cap = (unsigned)list_cap(n_out);
    return lo;
}

// The filter (one persistent launch per packing class: items of one or two
// slots on 256-candidate units, four-slot items on 128-candidate units; mc is
// the candidate-row map with 128-row boxes) and the re-rank, on stream s.
int launch_knn_tc(bool fp8, const CUtensorMap &mq, const CUtensorMap &mc, irc_plan *pl, const float *F,
                  const float4 *Fp, int nC, int knn, float *vrKnn, float *rho, int32_t *miKnn, float *d2Knn,
                  const ListOut &lo, cudaStream_t s);

}  // namespace irc_tc
