// irc_tc.cuh -- shared constants of the tensor-core kNN (internal).
#pragma once
#include <cuda.h>

#include "irc_plan.cuh"

namespace irc_tc {

constexpr int BM = 128;          // queries per CTA (TMEM lanes)
constexpr int BN = 128;          // candidates per tile (TMEM columns)
constexpr int KP = 64;           // padded feature dimension (bf16 elements, one 128-byte row)
constexpr int KNN_MAX = 32;      // largest knn served (candidate lists hold >= 64 for the re-rank)
using TcItem = irc::TcItem;

int launch_knn_tc(bool fp8, const CUtensorMap &mq, const CUtensorMap &mc, irc_plan *pl, const float *F,
                  const float4 *Fp, int nC, int knn, float *vrKnn, float *rho, int32_t *miKnn, float *d2Knn,
                  cudaStream_t s);

}  // namespace irc_tc
