// irc_tc_host.cu -- operand preparation and launch of the tensor-core kNN.
//
// Operand rows.  Every spike is stored twice in BF16, padded to K = 64 (one
// 128-byte swizzle row):
//     query row     [ -2*a_1 .. -2*a_D,  na_h, na_m, na_l,  1, 1, 1,  0, 0, 0,  0 ... ]
//     candidate row [    b_1 ..    b_D,     1,    1,    1, nb_h, nb_m, nb_l, 1, 1, 1, 0 ... ]
// where a, b are the BF16-rounded features and na = |a|^2 (FP32, from the
// rounded values) split exactly into three BF16 terms, so one K = 64
// contraction yields |a|^2 + |b|^2 - 2 a.b = |a - b|^2 of the rounded
// features, accumulated in FP32.  The filter's second pass writes a query's
// threshold, -tau split into three BF16 terms, into the three zeros of its
// row in shared memory (irc_tc.cu): its accumulators are then d2 - tau.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include "irc_common.cuh"
#include "irc_plan.cuh"
#include "irc_tc.cuh"

namespace {

// F (f32 [nF x nC]) -> query / candidate BF16 rows of 64.
// Centring of the tensor-core operands.  Distances do not change when every
// feature vector is shifted by the same reference point, but the rounding
// error of the BF16 / FP8 contraction grows with the operands' magnitude, and
// drift can carry features far from the origin.  The operand rows are built
// from F - ref with ref = the column means of a strided sample of at most
// 64K of the plan's query rows (fixed summation order, so the rows are the
// same on every call); the exact re-rank keeps reading the unshifted
// features.
constexpr int kMeanBlocks = 256;

__global__ void k_colsum_part(const float *__restrict__ F, int nC, int stride, int nS, float *__restrict__ part)
{
    __shared__ float red[4][64];
    const int c = threadIdx.x & 63, lane_r = threadIdx.x >> 6;   // 64 columns x 4 row lanes
    const int per = (nS + gridDim.x - 1) / gridDim.x;
    const int k0 = blockIdx.x * per, k1 = min(nS, k0 + per);
    float acc = 0.0f;
    if (c < nC)
        for (int k = k0 + lane_r; k < k1; k += 4) acc += __ldg(F + (size_t)k * stride * nC + c);
    red[lane_r][c] = acc;
    __syncthreads();
    if (threadIdx.x < 64)
        part[(size_t)blockIdx.x * 64 + c] = ((red[0][c] + red[1][c]) + red[2][c]) + red[3][c];
}

__global__ void k_colsum_final(const float *__restrict__ part, int nb, int nC, int nS, float *__restrict__ ref)
{
    const int c = threadIdx.x;
    if (c >= nC) return;
    double acc = 0.0;
    for (int b = 0; b < nb; ++b) acc += (double)part[(size_t)b * 64 + c];
    ref[c] = nS > 0 ? (float)(acc / (double)nS) : 0.0f;
}

// |F| maximum (bits of a non-negative float, so integer max == float max).
__global__ void k_absmax(const float *__restrict__ F, size_t n, int nC, const float *__restrict__ ref,
                         unsigned *__restrict__ out)
{
    unsigned m = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        m = max(m, __float_as_uint(fabsf(__ldg(F + i) - __ldg(ref + i % nC))));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__device__ __forceinline__ unsigned char to_e4m3(float x)
{
    return (unsigned char)__nv_cvt_float_to_fp8(x, __NV_SATFINITE, __NV_E4M3);
}

__device__ __forceinline__ float from_e4m3(unsigned char v)
{
    const __half_raw h = __nv_cvt_fp8_to_halfraw((__nv_fp8_storage_t)v, __NV_E4M3);
    return __half2float(__half(h));
}

// FP8 rows of 128 e4m3 values (K = 128, 128 bytes).  With x = e4m3(s*a),
// y = e4m3(s*b) and s = 32 / max|F| (so |x| <= 32 and -2x is exact):
//     query row     [ -2x_1 .. -2x_D, nx_0 .. nx_5, 2^e_0 .. 2^e_5, 0 ... ]
//     candidate row [    y_1 ..  y_D, 2^e_0 .. 2^e_5, ny_0 .. ny_5, 0 ... ]
// where |x|^2 = sum_t nx_t * 2^e_t (e = 8, 4, 0, -4, -8, -9: each e4m3 piece
// takes the next 4 bits of the remainder), so the contraction is
// s^2 |a - b|^2 of the rounded features -- a positive multiple, which the
// filter only compares.
constexpr int kFp8Pieces = 6;
__device__ __forceinline__ int piece_exp(int t) { return t < 5 ? 8 - 4 * t : -9; }

// Operand preparation, one warp per 32 consecutive rows of a row interval.
// The rows (contiguous in F) are read coalesced into shared memory with an
// odd row stride (nC | 1 words), so lane r working on row r has no bank
// conflicts; every lane builds its row's query and candidate operand rows
// (BF16: above the file; FP8: above) and stages them in shared memory in
// 16-byte pieces XOR-swizzled by row; the warp then writes its 32 rows of
// every output -- the re-rank's FP32 rows padded to Dp4 float4 too -- with
// contiguous stores.
constexpr int kPrepWarps = 4;

size_t prep_smem(int nC)
{
    return (size_t)kPrepWarps * (2 * 32 * 128 + 32 * (size_t)(nC | 1) * 4) + 64 * 4;
}

template <bool FP8>
__global__ void __launch_bounds__(32 * kPrepWarps)
k_prep(const float *__restrict__ F, int lo, int n, int nC, const float *__restrict__ ref,
       const unsigned *__restrict__ amax, uint4 *__restrict__ Fq, uint4 *__restrict__ Fc, float *__restrict__ Fp,
       int Dp4, int q_lo, int q_hi)
{
    extern __shared__ __align__(16) unsigned char prep_sm[];
    const int nCs = nC | 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint4 *sq = reinterpret_cast<uint4 *>(prep_sm) + (size_t)warp * 2 * 32 * 8;     // [32 rows][8], swizzled
    uint4 *sc = sq + 32 * 8;
    float *sref = reinterpret_cast<float *>(prep_sm + (size_t)kPrepWarps * 2 * 32 * 128);
    float *w = sref + 64 + (size_t)warp * 32 * nCs;
    for (int k = threadIdx.x; k < nC; k += blockDim.x) sref[k] = __ldg(ref + k);
    __syncthreads();
    const long long r0 = (long long)lo + ((long long)blockIdx.x * kPrepWarps + warp) * 32;
    if (r0 >= (long long)lo + n) return;
    const int nr = (int)min(32LL, (long long)lo + n - r0);
    const float *src = F + (size_t)r0 * nC;
    for (int t = lane; t < nr * nC; t += 32) {
        const int r = t / nC;
        w[r * nCs + (t - r * nC)] = __ldg(src + t);
    }
    __syncwarp();
    const int W = 4 * Dp4;
    float *dst = Fp + (size_t)r0 * W;
    for (int t = lane; t < nr * W; t += 32) {
        const int r = t / W, c = t - r * W;
        dst[t] = c < nC ? w[r * nCs + c] : 0.0f;
    }
    if (lane < nr) {
        const float *a = w + lane * nCs;
        uint4 *oq = sq + lane * 8, *oc = sc + lane * 8;
        const int sw = lane & 7;
        if (!FP8) {
            float na = 0.0f;
            for (int k = 0; k < nC; ++k) {
                const float f = __bfloat162float(__float2bfloat16_rn(a[k] - sref[k]));
                na = __fmaf_rn(f, f, na);
            }
            const __nv_bfloat16 h = __float2bfloat16_rn(na);
            const float rem1 = na - __bfloat162float(h);
            const __nv_bfloat16 m = __float2bfloat16_rn(rem1);
            const __nv_bfloat16 l = __float2bfloat16_rn(rem1 - __bfloat162float(m));
            const __nv_bfloat16 one = __float2bfloat16_rn(1.0f), zero = __float2bfloat16_rn(0.0f);
#pragma unroll 1
            for (int j = 0; j < irc_tc::KP / 8; ++j) {
                __align__(16) __nv_bfloat16 wq[8], wc[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int k = j * 8 + e;
                    __nv_bfloat16 vq = zero, vc = zero;
                    if (k < nC) {
                        const __nv_bfloat16 bf = __float2bfloat16_rn(a[k] - sref[k]);
                        vc = bf;
                        vq = __float2bfloat16_rn(-2.0f * __bfloat162float(bf));
                    } else if (k < nC + 3) {
                        vq = (k == nC) ? h : (k == nC + 1) ? m : l;
                        vc = one;
                    } else if (k < nC + 6) {
                        vq = one;
                        vc = (k == nC + 3) ? h : (k == nC + 4) ? m : l;
                    } else if (k < nC + 9) {
                        vc = one;                  // against the query's pass-2 threshold terms
                    }
                    wq[e] = vq;
                    wc[e] = vc;
                }
                oq[j ^ sw] = *reinterpret_cast<uint4 *>(wq);
                oc[j ^ sw] = *reinterpret_cast<uint4 *>(wc);
            }
        } else {
            const float am = __uint_as_float(*amax);
            const float scl = am > 0.0f ? 32.0f / am : 1.0f;
            float nx = 0.0f;
            for (int k = 0; k < nC; ++k) {
                const float x = from_e4m3(to_e4m3(scl * (a[k] - sref[k])));
                nx = __fmaf_rn(x, x, nx);
            }
            unsigned char pc[kFp8Pieces], pf[kFp8Pieces];
            float rem = nx;
#pragma unroll
            for (int t = 0; t < kFp8Pieces; ++t) {
                const float f = ldexpf(1.0f, piece_exp(t));
                pc[t] = to_e4m3(rem / f);
                pf[t] = to_e4m3(f);
                rem -= from_e4m3(pc[t]) * f;
            }
#pragma unroll 1
            for (int j = 0; j < 128 / 16; ++j) {
                __align__(16) unsigned char wq[16], wc[16];
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const int k = j * 16 + e;
                    unsigned char vq = 0, vc = 0;
                    if (k < nC) {
                        const unsigned char y = to_e4m3(scl * (a[k] - sref[k]));
                        vc = y;
                        vq = to_e4m3(-2.0f * from_e4m3(y));
                    } else if (k < nC + kFp8Pieces) {
                        vq = pc[k - nC];
                        vc = pf[k - nC];
                    } else if (k < nC + 2 * kFp8Pieces) {
                        vq = pf[k - nC - kFp8Pieces];
                        vc = pc[k - nC - kFp8Pieces];
                    }
                    wq[e] = vq;
                    wc[e] = vc;
                }
                oq[j ^ sw] = *reinterpret_cast<uint4 *>(wq);
                oc[j ^ sw] = *reinterpret_cast<uint4 *>(wc);
            }
        }
    }
    __syncwarp();
    // query rows (the plan's own queries, q_lo .. q_hi-1) are only read as query operands
    uint4 *gq = Fq + (size_t)r0 * 8, *gc = Fc + (size_t)r0 * 8;
    for (int t = lane; t < nr * 8; t += 32) {
        const int r = t >> 3, j = t & 7;
        if (r0 + r >= q_lo && r0 + r < q_hi) gq[t] = sq[r * 8 + (j ^ (r & 7))];
        gc[t] = sc[r * 8 + (j ^ (r & 7))];
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

// Tensor map over [rows x 128 bytes] operand rows (64 BF16 or 128 e4m3 values),
// box_rows-row boxes, 128-byte swizzle.
int make_map(CUtensorMap *m, void *base, int rows, int box_rows, bool fp8)
{
    EncodeTiledFn enc = encode_fn();
    if (!enc) { irc_host::set_error("cuTensorMapEncodeTiled unavailable"); return IRC_E_CUDA; }
    const int inner = fp8 ? 128 : irc_tc::KP;
    cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)128};
    cuuint32_t box[2] = {(cuuint32_t)inner, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(m, fp8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims,
                     strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { irc_host::set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return IRC_E_CUDA; }
    return IRC_OK;
}

}  // namespace

// Plan-owned tensor-core operand buffers (irc_site.cu) and the exact
// fallback for queries whose candidate list overflowed (irc_exact.cu).
int irc_plan_tc_buffers(irc_plan *pl, void **fq, void **fc, void **fp, void **extra, size_t row_bytes,
                        size_t fp_row_bytes, size_t extra_bytes);
int irc_exact_overflow_drain(irc_plan *pl, const float *F, int nC, int knn, float *vrKnn, float *rho,
                             int32_t *miKnn, float *d2Knn, cudaStream_t s);

int irc_site_knn_tc(irc_plan *pl, const float *F, int nC, int knn, int mode, float *vrKnn, float *rho,
                    int32_t *miKnn, float *d2Knn, cudaStream_t s)
{
    const bool fp8 = mode == IRC_MODE_FP8;
    if (nC + (fp8 ? 2 * kFp8Pieces : 6) > (fp8 ? 128 : irc_tc::KP)) {
        irc_host::set_error("irc_site_knn(tensor core): nC=%d too large", nC);
        return IRC_E_NC;
    }
    if (knn > irc_tc::KNN_MAX) { irc_host::set_error("irc_site_knn(BF16): knn %d > %d", knn, irc_tc::KNN_MAX); return IRC_E_INVAL; }
    const int nF = pl->dev.nF;
    void *fq, *fc, *fp, *ex;
    const int Dp4 = irc_tc::fp_row4(nC);                               // padded FP32 row, float4
    const size_t part_bytes = sizeof(float) * kMeanBlocks * 64;
    int rc = irc_plan_tc_buffers(pl, &fq, &fc, &fp, &ex, irc_tc::KP * 2, (size_t)Dp4 * 16,
                                 part_bytes + 256 + irc_tc::list_area_bytes(pl->dev.n_out));
    float *part = (float *)ex;
    float *ref = (float *)((char *)ex + part_bytes);
    const irc_tc::ListOut lo = irc_tc::list_area((char *)ex + part_bytes + 256, pl->dev.n_out);
    if (rc != IRC_OK) return rc;
    cudaError_t e = cudaMemsetAsync(pl->scratch, 0, sizeof(int), s);       // overflow-queue count
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(BF16): memset");
    const int nQ = pl->dev.n_out;                                     // the query rows q_base ..
    const int stride = nQ > 65536 ? (nQ + 65535) / 65536 : 1;
    const int nS = (nQ + stride - 1) / stride;                        // sampled: q_base + k * stride
    k_colsum_part<<<kMeanBlocks, 256, 0, s>>>(F + (size_t)pl->dev.q_base * nC, nC, stride, nS, part);
    k_colsum_final<<<1, 64, 0, s>>>(part, kMeanBlocks, nC, nS, ref);
    IRC_CHECK_LAUNCH("irc_site_knn(tensor core) centre");
    // operand rows for the rows the plan reads (its row intervals)
    unsigned *amax = reinterpret_cast<unsigned *>(pl->scratch + 1);       // free word of the plan scratch
    if (fp8) {
        e = cudaMemsetAsync(amax, 0, sizeof(unsigned), s);
        if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(FP8): memset");
        for (int v = 0; v < pl->n_row_iv; ++v) {
            const int lo = pl->row_iv[2 * v], n = pl->row_iv[2 * v + 1] - lo;
            k_absmax<<<152 * 4, 256, 0, s>>>(F + (size_t)lo * nC, (size_t)n * nC, nC, ref, amax);
        }
        IRC_CHECK_LAUNCH("irc_site_knn(FP8) absmax");
    }
    const size_t psm = prep_smem(nC);
    auto prep = fp8 ? k_prep<true> : k_prep<false>;
    e = cudaFuncSetAttribute(prep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn(tensor core): prep smem attribute");
    for (int v = 0; v < pl->n_row_iv; ++v) {
        const int lo = pl->row_iv[2 * v], n = pl->row_iv[2 * v + 1] - lo;
        const int rows_per_block = 32 * kPrepWarps;
        prep<<<(n + rows_per_block - 1) / rows_per_block, 32 * kPrepWarps, psm, s>>>(
            F, lo, n, nC, ref, amax, (uint4 *)fq, (uint4 *)fc, (float *)fp, Dp4, pl->dev.q_base,
            pl->dev.q_base + pl->dev.n_out);
    }
    IRC_CHECK_LAUNCH("irc_site_knn(tensor core) prep");
    CUtensorMap mq, mc;
    if ((rc = make_map(&mq, fq, nF, 32, fp8)) != IRC_OK) return rc;       // 32 query rows per lane quarter
    if ((rc = make_map(&mc, fc, nF, 128, fp8)) != IRC_OK) return rc;     // 128-row candidate tiles
    rc = irc_tc::launch_knn_tc(fp8, mq, mc, pl, F, (const float4 *)fp, nC, knn, vrKnn, rho, miKnn, d2Knn, lo, s);
    if (rc != IRC_OK) return rc;
    return irc_exact_overflow_drain(pl, F, nC, knn, vrKnn, rho, miKnn, d2Knn, s);
}
