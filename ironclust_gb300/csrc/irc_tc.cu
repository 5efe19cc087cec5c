// irc_tc.cu -- tensor-core (tcgen05) site kNN: BF16 distance filter + exact
// FP32 re-rank.
//
// Distances as a contraction.  Every spike is stored twice in BF16, padded to
// K = 64 (one 128-byte swizzle row):
//     query row     [ -2*a_1 .. -2*a_D,  na_h, na_m, na_l,  1, 1, 1,  0 ... ]
//     candidate row [    b_1 ..    b_D,     1,    1,    1, nb_h, nb_m, nb_l, 0 ... ]
// where a, b are the BF16-rounded features and na = |a|^2 (FP32, from the
// rounded values) split exactly into three BF16 terms.  One tcgen05 MMA over
// K = 64 then yields |a|^2 + |b|^2 - 2 a.b = |a - b|^2 of the rounded
// features in FP32 straight in TMEM, so the epilogue is one compare per pair.
//
// Per CTA: 128 queries of one drift chunk (TMEM lanes) against every linked
// candidate, streamed in 128-candidate tiles (TMEM columns, two accumulator
// buffers).  Warp roles: warp 0 issues TMA loads (4-stage ring), warp 1
// allocates TMEM and issues the MMAs from one thread, warps 2-5 (one per TMEM
// lane quarter) run the epilogue: each thread owns one query, keeps a
// threshold tau and appends candidates below it to a shared-memory list;
// when a list fills up the warp sorts it cooperatively (bitonic, 4 keys per
// lane), keeps the best 64 and lowers tau to the 64th.  At the end the 64
// approximate nearest candidates of every query are re-ranked with the
// reference FP32 arithmetic (exact), zero distances dropped, and the first
// knn written out in (distance, index) order.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstring>

#include "irc_common.cuh"
#include "irc_plan.cuh"
#include "irc_sm100.cuh"

namespace {

constexpr int BM = 128;                       // queries per CTA
constexpr int BN = 128;                       // candidates per tile
constexpr int KP = 64;                        // padded feature dimension (bf16)
constexpr int STAGES = 4;
constexpr int CAP = 128;                      // per-query list capacity
constexpr int KEEP = 64;                      // approximate candidates kept per query
constexpr int EPI_WARPS = 4;
constexpr int THREADS = 32 * (2 + EPI_WARPS);
constexpr uint32_t TILE_BYTES = BN * KP * 2;  // 16 KB (A tile has the same size)
constexpr uint32_t TMEM_COLS = 2 * BN;
constexpr int LSTRIDE = CAP + 1;             // list row stride (u64), padded against bank conflicts
constexpr size_t SMEM_BYTES = 1024 /*align slack*/ + TILE_BYTES * (1 + STAGES) + (size_t)LSTRIDE * BM * 8 + 256;
constexpr int KNN_MAX = 32;

__device__ __forceinline__ unsigned long long akey(float v, int idx)
{
    return ((unsigned long long)__float_as_uint(fmaxf(v, 0.0f)) << 32) | (unsigned)idx;
}

// Ascending bitonic sort of 32*PER 64-bit keys held PER per lane (element
// e = lane*PER + i).
template <int PER>
__device__ __forceinline__ void warp_bitonic(unsigned long long (&v)[PER], int lane)
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
                    const unsigned long long o = __shfl_xor_sync(0xffffffffu, v[i], ls);
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
                        const unsigned long long a = v[i], b = v[j];
                        const bool sw = up ? (a > b) : (a < b);
                        v[i] = sw ? b : a;
                        v[j] = sw ? a : b;
                    }
                }
            }
        }
    }
}

// Sort the list of query row `row` (lane L of this warp), keep the best KEEP,
// lower that lane's tau to the KEEP-th key.  Warp-uniform.
__device__ __forceinline__ void compact_row(unsigned long long *keys, int row, int L, int lane, int &cnt,
                                            float &tau)
{
    const int cL = __shfl_sync(0xffffffffu, cnt, L);
    unsigned long long v[CAP / 32];
#pragma unroll
    for (int i = 0; i < CAP / 32; ++i) {
        const int e = i * 32 + lane;                     // any assignment: the input is unsorted
        v[i] = e < cL ? keys[(size_t)row * LSTRIDE + e] : ~0ull;
    }
    warp_bitonic<CAP / 32>(v, lane);
#pragma unroll
    for (int i = 0; i < CAP / 32; ++i) {
        const int e = lane * (CAP / 32) + i;
        if (e < KEEP) keys[(size_t)row * LSTRIDE + e] = v[i];
    }
    // element KEEP-1 sits in lane (KEEP-1)/PER, slot (KEEP-1)%PER
    constexpr int PER = CAP / 32;
    const unsigned long long kth = __shfl_sync(0xffffffffu, v[(KEEP - 1) % PER], (KEEP - 1) / PER);
    if (lane == L) {
        if (cL >= KEEP) tau = __uint_as_float((unsigned)(kth >> 32));
        cnt = cL < KEEP ? cL : KEEP;
    }
    __syncwarp();
}

__global__ void __launch_bounds__(THREADS, 1)
k_knn_tc_bf16(const __grid_constant__ CUtensorMap tmQ, const __grid_constant__ CUtensorMap tmC, irc::PlanDev p,
              const float *__restrict__ F, int nC, int knn, float *__restrict__ vrKnn, float *__restrict__ rho,
              int *__restrict__ miKnn, float *__restrict__ d2Knn, int *__restrict__ err)
{
    extern __shared__ unsigned char smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *sA = base;
    uint8_t *sB = base + TILE_BYTES;
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(sB + STAGES * TILE_BYTES);   // [BM][LSTRIDE]
    uint64_t *bars = reinterpret_cast<uint64_t *>(keys + (size_t)LSTRIDE * BM);
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
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            sm100::prefetch_tmap(&tmQ);
            sm100::prefetch_tmap(&tmC);
            sm100::mbar_arrive_expect_tx(a_full, TILE_BYTES);
            sm100::tma_load_2d(&tmQ, a_full, sA, 0, qs);
            int i = 0;
            bool ok = true;
            for (int r = r0; r < r1 && ok; ++r) {
                const int rs = __ldg(p.rs + r), rn = __ldg(p.rn + r);
                for (int t = 0; t < rn && ok; t += BN, ++i) {
                    const int s = i % STAGES;
                    const uint32_t ph = (i / STAGES) & 1;
                    if (!(ok = sm100::mbar_wait(&empty[s], ph ^ 1, abort_flag))) break;
                    sm100::mbar_arrive_expect_tx(&full[s], TILE_BYTES);
                    sm100::tma_load_2d(&tmC, &full[s], sB + (size_t)s * TILE_BYTES, 0, rs + t);
                }
            }
            // drain: every issued load has landed before the CTA exits
            for (int j = (i > STAGES ? i - STAGES : 0); j < i; ++j)
                sm100::mbar_wait(&full[j % STAGES], (j / STAGES) & 1, abort_flag);
            sm100::mbar_wait(a_full, 0, abort_flag);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            constexpr uint32_t idesc = sm100::idesc_make(BM, BN, 1, 1);   // bf16 x bf16 -> f32
            int issued = 0;
            if (sm100::mbar_wait(a_full, 0, abort_flag)) {
                sm100::tc_fence_after();
                const uint64_t adesc = sm100::sdesc_sw128(sm100::smem_u32(sA));
                for (int i = 0; i < ntiles; ++i) {
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
                    ++issued;
                }
            }
            // every MMA has completed before TMEM is released
            sm100::mma_commit(mma_done);
            sm100::mbar_wait(mma_done, 0, abort_flag);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: one query per thread ----------------
        const int quarter = warp & 3;
        const int row = quarter * 32 + lane;
        const uint32_t tlane = (uint32_t)(quarter * 32) << 16;
        float tau = __int_as_float(0x7f800000);
        int cnt = 0;
        int i = 0;
        bool ok = true;
        for (int r = r0; r < r1 && ok; ++r) {
            const int rs = __ldg(p.rs + r), rn = __ldg(p.rn + r);
            for (int t = 0; t < rn; t += BN, ++i) {
                const int b = i & 1;
                if (!(ok = sm100::mbar_wait(&acc_full[b], (i >> 1) & 1, abort_flag))) break;
                sm100::tc_fence_after();
                const int nvalid = min(BN, rn - t);
                const int cand0 = rs + t;
                for (int cc = 0; cc < nvalid; cc += 32) {
                    unsigned need = __ballot_sync(0xffffffffu, cnt > CAP - 32);
                    while (need) {
                        const int L = __ffs(need) - 1;
                        compact_row(keys, quarter * 32 + L, L, lane, cnt, tau);
                        need &= need - 1;
                    }
                    float v[32];
                    sm100::tmem_ld32(tmem + tlane + b * BN + cc, v);
                    const int lim = min(32, nvalid - cc);
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (j < lim && v[j] < tau) {
                            keys[(size_t)row * LSTRIDE + cnt] = akey(v[j], cand0 + cc + j);
                            ++cnt;
                        }
                    __syncwarp();
                }
                sm100::tc_fence_before();
                __syncwarp();
                if (lane == 0) sm100::mbar_arrive(&acc_empty[b]);
            }
        }
        // final sort of every list
        for (int L = 0; L < 32; ++L) compact_row(keys, quarter * 32 + L, L, lane, cnt, tau);
        // exact FP32 re-rank of the kept candidates, one query per warp step
        for (int L = 0; L < 32 && ok; ++L) {
            const int rowL = quarter * 32 + L;
            if (rowL >= nq) break;
            const int q = qs + rowL;
            const int cL = __shfl_sync(0xffffffffu, cnt, L);
            const float *a = F + (size_t)q * nC;
            unsigned long long kv[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int e = lane * 2 + u;
                kv[u] = ~0ull;
                if (e < cL) {
                    const int idx = (int)(keys[(size_t)rowL * LSTRIDE + e] & 0xffffffffu);
                    const float *bb = F + (size_t)idx * nC;
                    float acc = 0.0f;
                    for (int c = 0; c < nC; ++c) acc = irc::dterm(acc, __ldg(bb + c), __ldg(a + c));
                    if (acc > 0.0f && acc < IRC_SINGLE_INF_F)
                        kv[u] = ((unsigned long long)__float_as_uint(acc) << 32) | (unsigned)idx;
                }
            }
            warp_bitonic<2>(kv, lane);
            const size_t o = (size_t)(q - p.q_base);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int e = lane * 2 + u;
                if (e < knn) {
                    const bool have = kv[u] != ~0ull;
                    const float d2 = have ? __uint_as_float((unsigned)(kv[u] >> 32)) : IRC_SINGLE_INF_F;
                    const int idx = have ? (int)(kv[u] & 0xffffffffu) : q;
                    miKnn[(size_t)e + (size_t)knn * o] = idx + 1;
                    if (d2Knn) d2Knn[(size_t)e + (size_t)knn * o] = d2;
                    if (e == knn - 1) {
                        const float vk = irc::ref_sqrt_abs(d2);
                        vrKnn[o] = vk;
                        if (rho) rho[o] = __fdiv_rn(1.0f, vk);
                    }
                }
            }
        }
    }
    sm100::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        sm100::tc_fence_after();
        sm100::tmem_dealloc(tmem, TMEM_COLS);
    }
    if (threadIdx.x == 0 && *abort_flag) atomicExch(err, 1);
}

// F (f32 [nF x nC]) -> query / candidate BF16 rows of 64 (see file comment).
__global__ void k_prep_bf16(const float *__restrict__ F, int nF, int nC, uint4 *__restrict__ Fq,
                            uint4 *__restrict__ Fc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nF) return;
    const float *a = F + (size_t)i * nC;
    float na = 0.0f;
    for (int k = 0; k < nC; ++k) {
        const float f = __bfloat162float(__float2bfloat16_rn(__ldg(a + k)));
        na = __fmaf_rn(f, f, na);
    }
    const __nv_bfloat16 h = __float2bfloat16_rn(na);
    const float rem1 = na - __bfloat162float(h);
    const __nv_bfloat16 m = __float2bfloat16_rn(rem1);
    const __nv_bfloat16 l = __float2bfloat16_rn(rem1 - __bfloat162float(m));
    const __nv_bfloat16 one = __float2bfloat16_rn(1.0f), zero = __float2bfloat16_rn(0.0f);
#pragma unroll 1
    for (int j = 0; j < KP / 8; ++j) {
        __align__(16) __nv_bfloat16 wq[8], wc[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int k = j * 8 + e;
            __nv_bfloat16 vq = zero, vc = zero;
            if (k < nC) {
                const __nv_bfloat16 bf = __float2bfloat16_rn(__ldg(a + k));
                vc = bf;
                vq = __float2bfloat16_rn(-2.0f * __bfloat162float(bf));
            } else if (k < nC + 3) {
                vq = (k == nC) ? h : (k == nC + 1) ? m : l;
                vc = one;
            } else if (k < nC + 6) {
                vq = one;
                vc = (k == nC + 3) ? h : (k == nC + 4) ? m : l;
            }
            wq[e] = vq;
            wc[e] = vc;
        }
        Fq[(size_t)i * (KP / 8) + j] = *reinterpret_cast<uint4 *>(wq);
        Fc[(size_t)i * (KP / 8) + j] = *reinterpret_cast<uint4 *>(wc);
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(ptr);
    }
    return fn;
}

// Tensor map over a [rows x 64] BF16 matrix, 128-row boxes, 128-byte swizzle.
int make_map(CUtensorMap *m, void *base, int rows, CUtensorMapDataType dt, int elem_bytes, int inner)
{
    EncodeTiledFn enc = encode_fn();
    if (!enc) { irc_host::set_error("cuTensorMapEncodeTiled unavailable"); return IRC_E_CUDA; }
    cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)inner * elem_bytes};
    cuuint32_t box[2] = {(cuuint32_t)inner, (cuuint32_t)BN};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(m, dt, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { irc_host::set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return IRC_E_CUDA; }
    return IRC_OK;
}

}  // namespace

// Plan-owned tensor-core operand buffers (allocated on the first tensor-core call).
int irc_plan_tc_buffers(irc_plan *pl, void **fq, void **fc, size_t row_bytes);

int irc_site_knn_tc(irc_plan *pl, const float *F, int nC, int knn, int mode, float *vrKnn, float *rho,
                    int32_t *miKnn, float *d2Knn, cudaStream_t s)
{
    if (mode != IRC_MODE_BF16) {
        irc_host::set_error("irc_site_knn: FP8 tensor-core mode not available");
        return IRC_E_UNSUPPORTED;
    }
    if (nC + 6 > KP) { irc_host::set_error("irc_site_knn(BF16): nC=%d > %d", nC, KP - 6); return IRC_E_NC; }
    if (knn > KNN_MAX) { irc_host::set_error("irc_site_knn(BF16): knn %d > %d", knn, KNN_MAX); return IRC_E_INVAL; }
    const int nF = pl->dev.nF;
    void *fq, *fc;
    int rc = irc_plan_tc_buffers(pl, &fq, &fc, KP * 2);
    if (rc != IRC_OK) return rc;
    k_prep_bf16<<<(nF + 255) / 256, 256, 0, s>>>(F, nF, nC, (uint4 *)fq, (uint4 *)fc);
    IRC_CHECK_LAUNCH("irc_site_knn(BF16) prep");
    CUtensorMap mq, mc;
    if ((rc = make_map(&mq, fq, nF, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, KP)) != IRC_OK) return rc;
    if ((rc = make_map(&mc, fc, nF, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, KP)) != IRC_OK) return rc;
    cudaError_t e = cudaFuncSetAttribute(k_knn_tc_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(BF16): smem attribute");
    const int tiles = pl->ntiles[irc::tile_slot(BM)];
    k_knn_tc_bf16<<<tiles, THREADS, SMEM_BYTES, s>>>(mq, mc, pl->dev, F, nC, knn, vrKnn, rho, miKnn, d2Knn,
                                                     pl->scratch + irc::kScratchErr);
    IRC_CHECK_LAUNCH("irc_site_knn(BF16)");
    return IRC_OK;
}
