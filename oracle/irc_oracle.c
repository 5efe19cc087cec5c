/*
 * irc_oracle.c -- CPU oracle for the IronClust clustering hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this file; only the tests, the smoke check and the CPU-baseline leg of
 * the benchmark use it, as the checker.
 *
 * Three groups of functions live here:
 *
 *  1. Restatements of the five reference CUDA kernels, one CPU loop nest per
 *     kernel, following the per-thread scan order of the shipped sources so
 *     that every float bit and every index matches:
 *       orc_search_min_drift     matlab/search_min_drift.cu:24-94
 *       orc_search_delta_drift   matlab/search_delta_drift.cu:24-106
 *       orc_cuda_knn_index       matlab/cuda_knn_index.cu:27-111
 *       orc_cuda_delta_knn       matlab/cuda_delta_knn.cu:19-87
 *       orc_rho_drift            matlab/irc_cuda_rho_drift.cu:28-108
 *       orc_delta_drift          matlab/irc_cuda_delta_drift.cu:28-131
 *       orc_cuda_knn / orc_cuda_knn_full / orc_cuda_knn_ib
 *                                matlab/cuda_knn.cu, cuda_knn_full.cu, cuda_knn_ib.cu
 *       orc_cuda_rho / orc_cuda_delta
 *                                matlab/irc_cuda_rho.cu, irc_cuda_delta.cu
 *     The kernels accumulate squared distances as `dist += d*d` with
 *     d = b - a in feature order; nvcc contracts that into one fused
 *     multiply-add per feature, which fmaf() restates.  This file must be
 *     compiled with -ffp-contract=off so the C compiler adds no contraction of
 *     its own.
 *
 *  2. The MATLAB post-processing the host applies to those outputs:
 *       orc_post_sort_knn   `sort` (stable, NaN last) + first knn rows,
 *                           matlab/irc2.m:3784-3787
 *       orc_post_min        `min` along columns (first index, NaN skipped),
 *                           matlab/irc2.m:3855-3857
 *
 *  3. Independent references:
 *       orc_exact_knn_f64 / orc_exact_delta_f64
 *            true k nearest neighbours / nearest higher-rho spike in double
 *            precision over the same drift-linked candidate runs, ties broken
 *            by (distance, index);
 *       orc_knn_cpu / orc_delta_cpu
 *            the reference's CPU path (irc2 with fGpu=0): knn_cpu_
 *            (matlab/irc2.m:4244-4263, pdist2 'Smallest', self included) and
 *            delta_cpu_ (matlab/irc2.m:3981-3994, expansion form, rho mask,
 *            no zero-distance exclusion).  pdist2 and MATLAB's single BLAS
 *            are closed, so their rounding is restated, not pinned.
 *
 * Array conventions follow MATLAB: features are column-major [nC x n]
 * (the nC features of a spike are contiguous), 2-D outputs are
 * column-major, returned indices are 1-based.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_SINGLE_INF ((float)3.402E+38)

/* plan: per query chunk i, queries [q0[i], q0[i]+nq[i]) and candidate runs
 * roff[i]..roff[i+1]-1 into (rs, rn): run start (0-based) and run length. */

/* ------------------------------------------------------------------------ */
/* 1. kernel restatements                                                    */
/* ------------------------------------------------------------------------ */

static inline float dist2_fma(const float *b, const float *a, int nC)
{
    float acc = 0.0f;
    for (int c = 0; c < nC; ++c) {
        float d = b[c] - a[c];
        acc = fmaf(d, d, acc);
    }
    return acc;
}

/* search_min_drift.cu:24-94.  vnConst = {nC, nF, nBB, iA0, nA}; the launch
 * (matlab/irc2.m:3775) covers every query of the chunk, wrapped blocks write
 * identical values, so each query is evaluated once here.  D, I: [nT x nA]. */
void orc_search_min_drift(float *D, int32_t *I, const float *F,
                          const int32_t *IBB, const int32_t *NBB,
                          const int32_t *vnConst, int nT)
{
    const int nC = vnConst[0], nBB = vnConst[2], iA0 = vnConst[3], nA = vnConst[4];
    const int nT0 = nT / nBB;
#pragma omp parallel for schedule(dynamic, 4)
    for (int iA1 = 0; iA1 < nA; ++iA1) {
        const int iA = iA0 + iA1;
        const float *a = F + (size_t)iA * nC;
        for (int tx = 0; tx < nT; ++tx) {
            float tD = ORC_SINGLE_INF;
            int tI = iA;
            const int b = tx % nBB, iB0 = IBB[b], nB0 = NBB[b], iT0 = tx / nBB;
            for (int iB = iT0 + iB0; iB < nB0 + iB0; iB += nT0) {
                float d2 = dist2_fma(F + (size_t)iB * nC, a, nC);
                if (d2 < tD && d2 > 0.0f) { tD = d2; tI = iB; }
            }
            D[tx + (size_t)nT * iA1] = sqrtf(tD < 0 ? -tD : tD);
            I[tx + (size_t)nT * iA1] = tI + 1;
        }
    }
}

/* search_delta_drift.cu:24-106.  A candidate is masked when R[iB] <= R[iA]
 * (so a NaN rho is NOT masked, as in the source). */
void orc_search_delta_drift(float *D, int32_t *I, const float *F, const float *R,
                            const int32_t *IBB, const int32_t *NBB,
                            const int32_t *vnConst, int nT)
{
    const int nC = vnConst[0], nBB = vnConst[2], iA0 = vnConst[3], nA = vnConst[4];
    const int nT0 = nT / nBB;
#pragma omp parallel for schedule(dynamic, 4)
    for (int iA1 = 0; iA1 < nA; ++iA1) {
        const int iA = iA0 + iA1;
        const float *a = F + (size_t)iA * nC;
        const float ra = R[iA];
        for (int tx = 0; tx < nT; ++tx) {
            float tD = ORC_SINGLE_INF;
            int tI = iA;
            const int b = tx % nBB, iB0 = IBB[b], nB0 = NBB[b], iT0 = tx / nBB;
            for (int iB = iT0 + iB0; iB < nB0 + iB0; iB += nT0) {
                if (R[iB] <= ra) continue;          /* dist = SINGLE_INF + ... never wins */
                float d2 = dist2_fma(F + (size_t)iB * nC, a, nC);
                if (d2 < tD && d2 > 0.0f) { tD = d2; tI = iB; }
            }
            D[tx + (size_t)nT * iA1] = sqrtf(tD < 0 ? -tD : tD);
            I[tx + (size_t)nT * iA1] = tI + 1;
        }
    }
}

/* The binned minimum + selection sort shared by cuda_knn_index.cu:27-111,
 * cuda_knn.cu, cuda_knn_full.cu and cuda_knn_ib.cu.  vnConst = {nB, nA, nC,
 * knn}.  Thread slot t keeps the first strict minimum over iiB = t, t+nT, ...
 * (self kept, no d2 > 0 filter; IB, when given, maps iiB to the B column
 * IB[iiB]-1, and the slot records that column), then knn steps of a
 * selection sort with swaps over the nT slots (a slot holding NaN at step iK
 * stays: nothing compares below NaN).  K: sqrt(|d|) of the knn-th slot, or of
 * every slot 0..knn-1 when kall; I (optional): recorded column + 1, 1 for a
 * slot that saw no candidate. */
static void knn_bins(float *K, int32_t *I, const float *B, const float *A, const int32_t *IB,
                     const int32_t *vnConst, int nT, int kall)
{
    const int nB = vnConst[0], nA = vnConst[1], nC = vnConst[2], knn = vnConst[3];
#pragma omp parallel
    {
        float *sD = (float *)malloc(sizeof(float) * nT);
        int *sI = (int *)malloc(sizeof(int) * nT);
#pragma omp for schedule(dynamic, 4)
        for (int iA = 0; iA < nA; ++iA) {
            const float *a = A + (size_t)iA * nC;
            for (int t = 0; t < nT; ++t) { sD[t] = ORC_SINGLE_INF; sI[t] = 0; }
            for (int tx = 0; tx < nT; ++tx)
                for (int iiB = tx; iiB < nB; iiB += nT) {
                    const int iB = IB ? IB[iiB] - 1 : iiB;
                    float d2 = dist2_fma(B + (size_t)iB * nC, a, nC);
                    if (d2 < sD[tx]) { sD[tx] = d2; sI[tx] = iB; }
                }
            for (int iK = 0; iK < knn; ++iK) {
                float dmin = sD[iK];
                int imin = iK;
                for (int j = iK; j < nT; ++j)
                    if (sD[j] < dmin) { dmin = sD[j]; imin = j; }
                float tf = sD[imin]; sD[imin] = sD[iK]; sD[iK] = tf;
                int ti = sI[imin]; sI[imin] = sI[iK]; sI[iK] = ti;
            }
            if (kall) {
                for (int iK = 0; iK < knn; ++iK) {
                    float v = sD[iK];
                    K[iK + (size_t)knn * iA] = sqrtf(v < 0 ? -v : v);
                }
            } else {
                float v = sD[knn - 1];
                K[iA] = sqrtf(v < 0 ? -v : v);
            }
            if (I)
                for (int iK = 0; iK < knn; ++iK) I[iK + (size_t)knn * iA] = sI[iK] + 1;
        }
        free(sD); free(sI);
    }
}

/* cuda_knn_index.cu:27-111: K [nA] = k-th distance, I [knn x nA]. */
void orc_cuda_knn_index(float *K, int32_t *I, const float *B, const float *A,
                        const int32_t *vnConst, int nT)
{
    knn_bins(K, I, B, A, NULL, vnConst, nT, 0);
}

/* cuda_knn.cu:24-103: K [nA] only (its index output is commented out). */
void orc_cuda_knn(float *K, const float *B, const float *A, const int32_t *vnConst, int nT)
{
    knn_bins(K, NULL, B, A, NULL, vnConst, nT, 0);
}

/* cuda_knn_full.cu:27-103: K [knn x nA] (every sorted distance), I [knn x nA]. */
void orc_cuda_knn_full(float *K, int32_t *I, const float *B, const float *A, const int32_t *vnConst,
                       int nT)
{
    knn_bins(K, I, B, A, NULL, vnConst, nT, 1);
}

/* cuda_knn_ib.cu:27-103: B columns through IB (1-based, nB entries); K [nA],
 * I [knn x nA] = IB-mapped column + 1. */
void orc_cuda_knn_ib(float *K, int32_t *I, const float *B, const float *A, const int32_t *IB,
                     const int32_t *vnConst, int nT)
{
    knn_bins(K, I, B, A, IB, vnConst, nT, 0);
}

/* Spike-specific cut-off of the fDc_spk option (irc_cuda_rho.cu:58-66,
 * irc_cuda_delta.cu:66-73): dc2 times the query's squared norm, accumulated
 * with fused multiply-adds in feature order, then one rounded multiply. */
static inline float dc_spk(const float *a, int nC, float dc2)
{
    float v = 0.0f;
    for (int c = 0; c < nC; ++c) v = fmaf(a[c], a[c], v);
    return v * dc2;
}

/* irc_cuda_rho.cu:24-129 (jrc3_cuda_rho).  vnConst = {n1, n12, nC, dn_max,
 * fDc_spk}.  Query i1 < n1 counts the candidates j < n12 within the time
 * window |ord[i1] - ord[j]| <= dn_max (self included) and, of those, the
 * ones at d2 <= dc2 (fDc_spk = 1: d2 < dc2 * |query|^2); rho = count /
 * compared, divided in double.  Integer counts: no scan-order dependence. */
void orc_cuda_rho(float *vrRho1, const float *mrFet12, const int32_t *viiSpk12_ord,
                  const int32_t *vnConst, float dc2)
{
    const int n1 = vnConst[0], n12 = vnConst[1], nC = vnConst[2], dn_max = vnConst[3], fdc = vnConst[4];
#pragma omp parallel for schedule(dynamic, 4)
    for (int i1 = 0; i1 < n1; ++i1) {
        const float *a = mrFet12 + (size_t)i1 * nC;
        const float cut = fdc == 1 ? dc_spk(a, nC, dc2) : dc2;
        long nRho = 0, nComp = 0;
        for (int j = 0; j < n12; ++j) {
            int dt = viiSpk12_ord[i1] - viiSpk12_ord[j];
            if ((dt < 0 ? -dt : dt) > dn_max) continue;
            float d2 = dist2_fma(mrFet12 + (size_t)j * nC, a, nC);
            ++nComp;
            if (fdc == 0 ? (d2 <= cut) : (d2 < cut)) ++nRho;
        }
        vrRho1[i1] = (float)((double)nRho / (double)nComp);
    }
}

/* irc_cuda_delta.cu:26-153 (jrc3_cuda_delta).  vnConst as orc_cuda_rho;
 * viiRho12_ord = rank in descending rho.  Candidate j of query i1 is kept
 * when within the time window and ranked before it (viiRho12_ord[j] <
 * viiRho12_ord[i1]).  Thread slot t of nT keeps its first strict minimum
 * over j = t, t+nT, ...; the lowest slot holding the overall minimum wins;
 * none below SINGLE_INF -> the query itself.  delta = sqrt(d2 / dc2)
 * (fDc_spk = 1: / (dc2 * |query|^2)); the source's ABS applies to a
 * non-negative value.  nneigh = index + 1. */
void orc_cuda_delta(float *vrDelta1, uint32_t *viNneigh1, const float *mrFet12, const int32_t *viiSpk12_ord,
                    const int32_t *viiRho12_ord, const int32_t *vnConst, float dc2, int nT)
{
    const int n1 = vnConst[0], n12 = vnConst[1], nC = vnConst[2], dn_max = vnConst[3], fdc = vnConst[4];
#pragma omp parallel for schedule(dynamic, 4)
    for (int i1 = 0; i1 < n1; ++i1) {
        const float *a = mrFet12 + (size_t)i1 * nC;
        float best = ORC_SINGLE_INF;
        uint32_t bi = (uint32_t)i1;
        for (int t = 0; t < nT; ++t) {
            float tmin = ORC_SINGLE_INF;
            uint32_t timin = (uint32_t)i1;
            for (int j = t; j < n12; j += nT) {
                int dt = viiSpk12_ord[i1] - viiSpk12_ord[j];
                if ((dt < 0 ? -dt : dt) > dn_max || !(viiRho12_ord[j] < viiRho12_ord[i1])) continue;
                float d2 = dist2_fma(mrFet12 + (size_t)j * nC, a, nC);
                if (d2 < tmin) { tmin = d2; timin = (uint32_t)j; }
            }
            if (tmin < best) { best = tmin; bi = timin; }
        }
        vrDelta1[i1] = sqrtf(best / (fdc == 0 ? dc2 : dc_spk(a, nC, dc2)));
        viNneigh1[i1] = bi + 1;
    }
}

/* cuda_delta_knn.cu:19-87.  vnConst = {nB, nA, nC}.  Candidate kept when
 * R_B > R_A (strict; NaN excluded), zero distance kept, lowest thread slot
 * wins ties, fallback index = iA (an A-space index, as in the source). */
void orc_cuda_delta_knn(float *D, uint32_t *N, const float *B, const float *A,
                        const float *R_B, const float *R_A, const int32_t *vnConst, int nT)
{
    const int nB = vnConst[0], nA = vnConst[1], nC = vnConst[2];
#pragma omp parallel
    {
        float *sD = (float *)malloc(sizeof(float) * nT);
        uint32_t *sN = (uint32_t *)malloc(sizeof(uint32_t) * nT);
#pragma omp for schedule(dynamic, 4)
        for (int iA = 0; iA < nA; ++iA) {
            const float *a = A + (size_t)iA * nC;
            const float ra = R_A[iA];
            for (int t = 0; t < nT; ++t) { sD[t] = ORC_SINGLE_INF; sN[t] = 0; }
            for (int tx = 0; tx < nT; ++tx)
                for (int iB = tx; iB < nB; iB += nT) {
                    float d2 = dist2_fma(B + (size_t)iB * nC, a, nC);
                    if (R_B[iB] > ra && d2 < sD[tx]) { sD[tx] = d2; sN[tx] = (uint32_t)iB; }
                }
            float dmin = ORC_SINGLE_INF;
            uint32_t imin = (uint32_t)iA;
            for (int t = 0; t < nT; ++t)
                if (sD[t] < dmin) { dmin = sD[t]; imin = sN[t]; }
            D[iA] = sqrtf(dmin < 0 ? -dmin : dmin);
            N[iA] = imin + 1;
        }
        free(sD); free(sN);
    }
}

/* irc_cuda_rho_drift.cu:28-108.  vnConst = {n1, n12, nC}; miSite12 is
 * [n12 x 2] column-major (primary, secondary site).  Distance = query minus
 * candidate, fused per feature (calc_dist_, :18-25); counts are integers so
 * the result does not depend on the scan order. */
void orc_rho_drift(float *vrRho1, const int32_t *miSite12, const float *mrFet1,
                   const float *mrFet2, const int32_t *vnConst, float dc2)
{
    const int n1 = vnConst[0], n12 = vnConst[1], nC = vnConst[2];
#pragma omp parallel for schedule(dynamic, 4)
    for (int i1 = 0; i1 < n1; ++i1) {
        const int s = miSite12[i1];
        const float *q = mrFet1 + (size_t)i1 * nC;
        int nRho = 0, nComp = 0;
        for (int j = 0; j < n12; ++j) {
            const float *c;
            if (miSite12[j] == s) c = mrFet1 + (size_t)j * nC;
            else if (miSite12[j + n12] == s) c = mrFet2 + (size_t)j * nC;
            else continue;
            float acc = 0.0f;
            for (int k = 0; k < nC; ++k) { float t = q[k] - c[k]; acc = fmaf(t, t, acc); }
            if (acc <= dc2) ++nRho;
            ++nComp;
        }
        vrRho1[i1] = (float)((double)nRho / (double)nComp);
    }
}

/* ------------------------------------------------------------------------ */
/* 2. MATLAB post-processing                                                 */
/* ------------------------------------------------------------------------ */

/* MATLAB `sort` ascending on single data: stable, NaN placed last. */
static inline int mat_less(float x, int ix, float y, int iy)
{
    int nx = isnan(x), ny = isnan(y);
    if (nx || ny) {
        if (nx && ny) return ix < iy;
        return ny;               /* non-NaN before NaN */
    }
    if (x < y) return 1;
    if (y < x) return 0;
    return ix < iy;
}

/* [vs, order] = sort(D); vrKnn = vs(knn,:); miKnn = I(order(1:knn,:))
 * matlab/irc2.m:3784-3787.  D, I: [nT x nA]; outputs vrKnn [nA], miKnn [knn x nA]. */
void orc_post_sort_knn(const float *D, const int32_t *I, int nT, int nA, int knn,
                       float *vrKnn, int32_t *miKnn)
{
#pragma omp parallel
    {
        int *sel = (int *)malloc(sizeof(int) * (size_t)knn);
#pragma omp for schedule(dynamic, 16)
        for (int a = 0; a < nA; ++a) {
            const float *col = D + (size_t)nT * a;
            int n = 0;
            /* partial insertion sort of the first knn in (value, position) order */
            for (int t = 0; t < nT; ++t) {
                if (n == knn && !mat_less(col[t], t, col[sel[n - 1]], sel[n - 1])) continue;
                int p = (n < knn) ? n++ : n - 1;
                while (p > 0 && mat_less(col[t], t, col[sel[p - 1]], sel[p - 1])) {
                    sel[p] = sel[p - 1];
                    --p;
                }
                sel[p] = t;
            }
            vrKnn[a] = col[sel[knn - 1]];
            for (int k = 0; k < knn; ++k) miKnn[k + (size_t)knn * a] = I[sel[k] + (size_t)nT * a];
        }
        free(sel);
    }
}

/* [vrMin, viMin] = min(D); viNneigh = I(viMin)   matlab/irc2.m:3855-3857 */
void orc_post_min(const float *D, const int32_t *I, int nT, int nA,
                  float *vrMin, int32_t *viNneigh)
{
    for (int a = 0; a < nA; ++a) {
        const float *col = D + (size_t)nT * a;
        int best = -1;
        for (int t = 0; t < nT; ++t) {
            if (isnan(col[t])) continue;
            if (best < 0 || col[t] < col[best]) best = t;
        }
        if (best < 0) { vrMin[a] = NAN; best = 0; }
        else vrMin[a] = col[best];
        viNneigh[a] = I[best + (size_t)nT * a];
    }
}

/* ------------------------------------------------------------------------ */
/* 3a. exact FP64 references over a drift plan                              */
/* ------------------------------------------------------------------------ */

static inline double dist2_f64(const float *b, const float *a, int nC)
{
    double acc = 0.0;
    for (int c = 0; c < nC; ++c) {
        double d = (double)b[c] - (double)a[c];
        acc += d * d;
    }
    return acc;
}

/* The exact references below visit the queries of a chunk in blocks of
 * ORC_QB: every candidate row is read once per block and its distances to the
 * block's queries are formed side by side (each query's own sum still runs in
 * feature order, exactly as the one-query loops would form it), which lets
 * the compiler vectorise across the queries.  Work items are (chunk, block)
 * pairs over the whole plan, scheduled dynamically. */
#define ORC_QB 8

typedef struct {
    int *off;                /* [nChunks + 1] prefix of ceil(nq / ORC_QB) */
    long total;
} orc_blocks;

static orc_blocks plan_blocks(const int32_t *nq, int nChunks)
{
    orc_blocks b;
    b.off = (int *)malloc(sizeof(int) * ((size_t)nChunks + 1));
    b.off[0] = 0;
    for (int i = 0; i < nChunks; ++i) b.off[i + 1] = b.off[i] + (nq[i] + ORC_QB - 1) / ORC_QB;
    b.total = b.off[nChunks];
    return b;
}

/* chunk of flat block w and the first query / query count of that block */
static inline int block_chunk(const orc_blocks *b, int nChunks, long w)
{
    int lo = 0, hi = nChunks;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (b->off[mid] <= w) lo = mid; else hi = mid;
    }
    return lo;
}

/* queries q0 .. q0+n-1 transposed into aT[c * ORC_QB + j] (unused lanes
 * repeat the last query) */
static inline void stage_f32(float *aT, const float *F, int q0, int n, int nC)
{
    for (int j = 0; j < ORC_QB; ++j) {
        const float *a = F + (size_t)(q0 + (j < n ? j : n - 1)) * nC;
        for (int c = 0; c < nC; ++c) aT[c * ORC_QB + j] = a[c];
    }
}

static inline void stage_f64(double *aT, const float *F, int q0, int n, int nC)
{
    for (int j = 0; j < ORC_QB; ++j) {
        const float *a = F + (size_t)(q0 + (j < n ? j : n - 1)) * nC;
        for (int c = 0; c < nC; ++c) aT[c * ORC_QB + j] = (double)a[c];
    }
}

/* dist2_f64 of candidate row b to the ORC_QB staged queries */
static inline void dist2_f64_qb(double *out, const float *b, const double *aT, int nC)
{
    double acc[ORC_QB];
    for (int j = 0; j < ORC_QB; ++j) acc[j] = 0.0;
    for (int c = 0; c < nC; ++c) {
        const double bc = (double)b[c];
        for (int j = 0; j < ORC_QB; ++j) {
            const double d = bc - aT[c * ORC_QB + j];
            acc[j] += d * d;
        }
    }
    for (int j = 0; j < ORC_QB; ++j) out[j] = acc[j];
}

/* dist2_fma of candidate row b to the ORC_QB staged queries */
static inline void dist2_fma_qb(float *out, const float *b, const float *aT, int nC)
{
    float acc[ORC_QB];
    for (int j = 0; j < ORC_QB; ++j) acc[j] = 0.0f;
    for (int c = 0; c < nC; ++c) {
        const float bc = b[c];
        for (int j = 0; j < ORC_QB; ++j) {
            const float d = bc - aT[c * ORC_QB + j];
            acc[j] = fmaf(d, d, acc[j]);
        }
    }
    for (int j = 0; j < ORC_QB; ++j) out[j] = acc[j];
}

/* insert (d, c) into the ascending (d, index) list bd/bi of n <= knn entries */
#define ORC_TOPK_INSERT(bd, bi, n, knn, d, c)                                                     \
    do {                                                                                          \
        if ((n) == (knn) && !((d) < (bd)[(n) - 1] || ((d) == (bd)[(n) - 1] && (c) < (bi)[(n) - 1]))) \
            break;                                                                                \
        int p_ = ((n) < (knn)) ? (n)++ : (n) - 1;                                                 \
        while (p_ > 0 && ((d) < (bd)[p_ - 1] || ((d) == (bd)[p_ - 1] && (c) < (bi)[p_ - 1]))) {   \
            (bd)[p_] = (bd)[p_ - 1];                                                              \
            (bi)[p_] = (bi)[p_ - 1];                                                              \
            --p_;                                                                                 \
        }                                                                                         \
        (bd)[p_] = (d);                                                                           \
        (bi)[p_] = (c);                                                                           \
    } while (0)

/* Top-knn by (d2, index) for every query of every chunk.  exclude_zero=1
 * drops candidates at distance exactly 0 (self and exact duplicates), as the
 * irc2 GPU kernels do; 0 keeps them, as knn_cpu_ does.  Outputs, indexed by
 * q - q_base: idx [knn x nOut] (1-based into F, 0 when fewer than knn
 * candidates exist), d2 [knn x nOut] (NAN when missing). */
void orc_exact_knn_f64(int32_t *idx, double *d2out, const float *F, int nC,
                       const int32_t *q0, const int32_t *nq, const int32_t *roff,
                       const int32_t *rs, const int32_t *rn, int nChunks,
                       int q_base, int knn, int exclude_zero)
{
    orc_blocks B = plan_blocks(nq, nChunks);
#pragma omp parallel
    {
        double *bd = (double *)malloc(sizeof(double) * (size_t)knn * ORC_QB);
        int *bi = (int *)malloc(sizeof(int) * (size_t)knn * ORC_QB);
        double *aT = (double *)malloc(sizeof(double) * (size_t)nC * ORC_QB);
#pragma omp for schedule(dynamic, 4)
        for (long w = 0; w < B.total; ++w) {
            const int ch = block_chunk(&B, nChunks, w);
            const int qa = q0[ch] + (int)(w - B.off[ch]) * ORC_QB;
            const int nb = (q0[ch] + nq[ch] - qa) < ORC_QB ? (q0[ch] + nq[ch] - qa) : ORC_QB;
            int n[ORC_QB] = {0};
            stage_f64(aT, F, qa, nb, nC);
            for (int r = roff[ch]; r < roff[ch + 1]; ++r)
                for (int c = rs[r]; c < rs[r] + rn[r]; ++c) {
                    double dd[ORC_QB];
                    dist2_f64_qb(dd, F + (size_t)c * nC, aT, nC);
                    for (int j = 0; j < nb; ++j) {
                        const double d = dd[j];
                        if (exclude_zero && d == 0.0) continue;
                        ORC_TOPK_INSERT(bd + (size_t)j * knn, bi + (size_t)j * knn, n[j], knn, d, c);
                    }
                }
            for (int j = 0; j < nb; ++j) {
                const size_t o = (size_t)(qa + j - q_base) * knn;
                for (int k = 0; k < knn; ++k) {
                    idx[o + k] = (k < n[j]) ? bi[(size_t)j * knn + k] + 1 : 0;
                    d2out[o + k] = (k < n[j]) ? bd[(size_t)j * knn + k] : NAN;
                }
            }
        }
        free(bd); free(bi); free(aT);
    }
    free(B.off);
}

/* Nearest candidate with strictly higher rho (R indexed like F, in double so
 * that an FP64 rho keeps its own order), distance > 0 when exclude_zero, ties
 * by (d2, index).  Outputs indexed by q - q_base: nn (1-based, 0 when none)
 * and d2 (INFINITY when none). */
void orc_exact_delta_f64(int32_t *nn, double *d2out, const float *F, const double *R, int nC,
                         const int32_t *q0, const int32_t *nq, const int32_t *roff,
                         const int32_t *rs, const int32_t *rn, int nChunks,
                         int q_base, int exclude_zero)
{
    orc_blocks B = plan_blocks(nq, nChunks);
#pragma omp parallel
    {
        double *aT = (double *)malloc(sizeof(double) * (size_t)nC * ORC_QB);
#pragma omp for schedule(dynamic, 4)
        for (long w = 0; w < B.total; ++w) {
            const int ch = block_chunk(&B, nChunks, w);
            const int qa = q0[ch] + (int)(w - B.off[ch]) * ORC_QB;
            const int nb = (q0[ch] + nq[ch] - qa) < ORC_QB ? (q0[ch] + nq[ch] - qa) : ORC_QB;
            double best[ORC_QB], ra[ORC_QB], rmin = INFINITY;
            int bi[ORC_QB];
            for (int j = 0; j < nb; ++j) {
                best[j] = INFINITY;
                bi[j] = -1;
                ra[j] = R[qa + j];
                if (ra[j] < rmin) rmin = ra[j];
            }
            stage_f64(aT, F, qa, nb, nC);
            for (int r = roff[ch]; r < roff[ch + 1]; ++r)
                for (int c = rs[r]; c < rs[r] + rn[r]; ++c) {
                    if (!(R[c] > rmin)) continue;          /* masked for every query of the block */
                    double dd[ORC_QB];
                    dist2_f64_qb(dd, F + (size_t)c * nC, aT, nC);
                    for (int j = 0; j < nb; ++j) {
                        if (!(R[c] > ra[j])) continue;
                        const double d = dd[j];
                        if (exclude_zero && d == 0.0) continue;
                        if (d < best[j] || (d == best[j] && c < bi[j])) { best[j] = d; bi[j] = c; }
                    }
                }
            for (int j = 0; j < nb; ++j) {
                nn[qa + j - q_base] = bi[j] + 1;
                d2out[qa + j - q_base] = best[j];
            }
        }
        free(aT);
    }
    free(B.off);
}

/* ------------------------------------------------------------------------ */
/* 3b. the reference CPU path (irc2 fGpu=0), one call per drift chunk        */
/* ------------------------------------------------------------------------ */

/* knn_cpu_ (matlab/irc2.m:4244-4263): pdist2(B', A', 'euclidean',
 * 'Smallest', knn), self included.  B = gathered candidates [nC x nB],
 * A = queries [nC x nA].  Distances in single precision, sqrt of a plain
 * (unfused) sum of squares; ties by candidate order.  Outputs vrKnn [nA]
 * (k-th distance), miKnn [knn x nA] (1-based into B, padded by repeating
 * the last row when nB < knn). */
void orc_knn_cpu(float *vrKnn, int32_t *miKnn, const float *B, int nB,
                 const float *A, int nA, int nC, int knn)
{
    const int kk = knn < nB ? knn : nB;
#pragma omp parallel
    {
        float *bd = (float *)malloc(sizeof(float) * (size_t)(kk > 0 ? kk : 1));
        int *bi = (int *)malloc(sizeof(int) * (size_t)(kk > 0 ? kk : 1));
        float *dd = (float *)malloc(sizeof(float) * (size_t)(nB > 0 ? nB : 1));
#pragma omp for schedule(dynamic, 4)
        for (int ia = 0; ia < nA; ++ia) {
            const float *a = A + (size_t)ia * nC;
            for (int ib = 0; ib < nB; ++ib) {
                const float *b = B + (size_t)ib * nC;
                float s = 0.0f;
                for (int c = 0; c < nC; ++c) { float d = a[c] - b[c]; s += d * d; }
                dd[ib] = s;
            }
            int n = 0;
            for (int ib = 0; ib < nB; ++ib) {
                float d = dd[ib];
                if (n == kk && !(d < bd[n - 1])) continue;
                int p = (n < kk) ? n++ : n - 1;
                while (p > 0 && d < bd[p - 1]) { bd[p] = bd[p - 1]; bi[p] = bi[p - 1]; --p; }
                bd[p] = d; bi[p] = ib;
            }
            vrKnn[ia] = kk > 0 ? sqrtf(bd[kk - 1]) : NAN;
            for (int k = 0; k < knn; ++k)
                miKnn[k + (size_t)knn * ia] = kk > 0 ? bi[k < kk ? k : kk - 1] + 1 : 0;
        }
        free(bd); free(bi); free(dd);
    }
}

/* delta_cpu_ (matlab/irc2.m:3981-3994): D = sum(y.^2) + (sum(x.^2)' - 2*x'*y),
 * masked to inf where rho_x <= rho_y, [v, i] = min(D) (first index), then
 * sqrt(abs(v)).  Zero distance is not excluded.  B = candidates [nC x nB]
 * with rho RB, A = queries [nC x nA] with rho RA.  Outputs delta [nA],
 * nneigh [nA] (1-based into B). */
void orc_delta_cpu(float *delta, int32_t *nneigh, const float *B, const float *RB, int nB,
                   const float *A, const float *RA, int nA, int nC)
{
    float *sx = (float *)malloc(sizeof(float) * (size_t)(nB > 0 ? nB : 1));
    for (int ib = 0; ib < nB; ++ib) {
        const float *b = B + (size_t)ib * nC;
        float s = 0.0f;
        for (int c = 0; c < nC; ++c) s += b[c] * b[c];
        sx[ib] = s;
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (int ia = 0; ia < nA; ++ia) {
        const float *a = A + (size_t)ia * nC;
        float sy = 0.0f;
        for (int c = 0; c < nC; ++c) sy += a[c] * a[c];
        const float ra = RA[ia];
        float best = NAN;
        int bi = 0;
        for (int ib = 0; ib < nB; ++ib) {
            const float *b = B + (size_t)ib * nC;
            float g = 0.0f;
            for (int c = 0; c < nC; ++c) g += b[c] * a[c];
            float d = sy + (sx[ib] - 2.0f * g);
            if (RB[ib] <= ra) d = INFINITY;
            if (isnan(d)) continue;                 /* MATLAB min skips NaN */
            if (isnan(best) || d < best) { best = d; bi = ib; }
        }
        delta[ia] = sqrtf(fabsf(best));
        nneigh[ia] = bi + 1;
    }
    free(sx);
}

/* Drive knn_cpu_ / delta_cpu_ over a drift plan exactly as rho_paged_site_ /
 * delta_paged_site_ do on their CPU branch (matlab/irc2.m:3653-3668,
 * :3703-3719): per chunk, gather the linked runs, run the call, map indices
 * back.  Outputs indexed by q - q_base; indices 1-based into F. */
void orc_site_knn_cpu(float *vrKnn, int32_t *miKnn, const float *F, int nC,
                      const int32_t *q0, const int32_t *nq, const int32_t *roff,
                      const int32_t *rs, const int32_t *rn, int nChunks, int q_base, int knn)
{
    for (int ch = 0; ch < nChunks; ++ch) {
        int nB = 0;
        for (int r = roff[ch]; r < roff[ch + 1]; ++r) nB += rn[r];
        float *B = (float *)malloc(sizeof(float) * (size_t)nC * (nB > 0 ? nB : 1));
        int32_t *map = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nB > 0 ? nB : 1));
        int p = 0;
        for (int r = roff[ch]; r < roff[ch + 1]; ++r)
            for (int c = rs[r]; c < rs[r] + rn[r]; ++c, ++p) {
                memcpy(B + (size_t)p * nC, F + (size_t)c * nC, sizeof(float) * nC);
                map[p] = c;
            }
        const int o = q0[ch] - q_base;
        int32_t *mk = miKnn + (size_t)o * knn;
        orc_knn_cpu(vrKnn + o, mk, B, nB, F + (size_t)q0[ch] * nC, nq[ch], nC, knn);
        for (size_t i = 0; i < (size_t)knn * nq[ch]; ++i)
            if (mk[i] > 0) mk[i] = map[mk[i] - 1] + 1;
        free(B); free(map);
    }
}

void orc_site_delta_cpu(float *delta, int32_t *nneigh, const float *F, const float *R, int nC,
                        const int32_t *q0, const int32_t *nq, const int32_t *roff,
                        const int32_t *rs, const int32_t *rn, int nChunks, int q_base)
{
    for (int ch = 0; ch < nChunks; ++ch) {
        int nB = 0;
        for (int r = roff[ch]; r < roff[ch + 1]; ++r) nB += rn[r];
        float *B = (float *)malloc(sizeof(float) * (size_t)nC * (nB > 0 ? nB : 1));
        float *RB = (float *)malloc(sizeof(float) * (size_t)(nB > 0 ? nB : 1));
        int32_t *map = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nB > 0 ? nB : 1));
        int p = 0;
        for (int r = roff[ch]; r < roff[ch + 1]; ++r)
            for (int c = rs[r]; c < rs[r] + rn[r]; ++c, ++p) {
                memcpy(B + (size_t)p * nC, F + (size_t)c * nC, sizeof(float) * nC);
                RB[p] = R[c];
                map[p] = c;
            }
        const int o = q0[ch] - q_base;
        orc_delta_cpu(delta + o, nneigh + o, B, RB, nB, F + (size_t)q0[ch] * nC,
                      R + q0[ch], nq[ch], nC);
        for (int i = 0; i < nq[ch]; ++i) nneigh[o + i] = map[nneigh[o + i] - 1] + 1;
        free(B); free(RB); free(map);
    }
}

/* ------------------------------------------------------------------------ */
/* 3c. exact references in the reference FP32 arithmetic                     */
/* ------------------------------------------------------------------------ */

/* True top-knn under the reference FP32 distance (dist2_fma: d = b - a,
 * fused accumulate in feature order), d2 > 0 and d2 < SINGLE_INF, ordered by
 * (d2, index).  Missing entries: index = query + 1, d2 = SINGLE_INF.
 * Outputs indexed by q - q_base: idx [knn x nOut] (1-based), d2 [knn x nOut]. */
void orc_exact_knn_f32(int32_t *idx, float *d2out, const float *F, int nC,
                       const int32_t *q0, const int32_t *nq, const int32_t *roff,
                       const int32_t *rs, const int32_t *rn, int nChunks, int q_base, int knn)
{
    orc_blocks B = plan_blocks(nq, nChunks);
#pragma omp parallel
    {
        float *bd = (float *)malloc(sizeof(float) * (size_t)knn * ORC_QB);
        int *bi = (int *)malloc(sizeof(int) * (size_t)knn * ORC_QB);
        float *aT = (float *)malloc(sizeof(float) * (size_t)nC * ORC_QB);
#pragma omp for schedule(dynamic, 4)
        for (long w = 0; w < B.total; ++w) {
            const int ch = block_chunk(&B, nChunks, w);
            const int qa = q0[ch] + (int)(w - B.off[ch]) * ORC_QB;
            const int nb = (q0[ch] + nq[ch] - qa) < ORC_QB ? (q0[ch] + nq[ch] - qa) : ORC_QB;
            int n[ORC_QB] = {0};
            stage_f32(aT, F, qa, nb, nC);
            for (int r = roff[ch]; r < roff[ch + 1]; ++r)
                for (int c = rs[r]; c < rs[r] + rn[r]; ++c) {
                    float dd[ORC_QB];
                    dist2_fma_qb(dd, F + (size_t)c * nC, aT, nC);
                    for (int j = 0; j < nb; ++j) {
                        const float d = dd[j];
                        if (!(d > 0.0f) || !(d < ORC_SINGLE_INF)) continue;
                        ORC_TOPK_INSERT(bd + (size_t)j * knn, bi + (size_t)j * knn, n[j], knn, d, c);
                    }
                }
            for (int j = 0; j < nb; ++j) {
                const int q = qa + j;
                const size_t o = (size_t)(q - q_base) * knn;
                for (int k = 0; k < knn; ++k) {
                    idx[o + k] = (k < n[j]) ? bi[(size_t)j * knn + k] + 1 : q + 1;
                    d2out[o + k] = (k < n[j]) ? bd[(size_t)j * knn + k] : ORC_SINGLE_INF;
                }
            }
        }
        free(bd); free(bi); free(aT);
    }
    free(B.off);
}

/* Nearest candidate not masked by R[c] <= R[q] (the search_delta_drift
 * mask), FP32 reference distance, d2 > 0 and < SINGLE_INF, ties by
 * (d2, index).  Missing: nn = q + 1, d2 = SINGLE_INF.  Indexed by q - q_base. */
void orc_exact_delta_f32(int32_t *nn, float *d2out, const float *F, const float *R, int nC,
                         const int32_t *q0, const int32_t *nq, const int32_t *roff,
                         const int32_t *rs, const int32_t *rn, int nChunks, int q_base)
{
    orc_blocks B = plan_blocks(nq, nChunks);
#pragma omp parallel
    {
        float *aT = (float *)malloc(sizeof(float) * (size_t)nC * ORC_QB);
#pragma omp for schedule(dynamic, 4)
        for (long w = 0; w < B.total; ++w) {
            const int ch = block_chunk(&B, nChunks, w);
            const int qa = q0[ch] + (int)(w - B.off[ch]) * ORC_QB;
            const int nb = (q0[ch] + nq[ch] - qa) < ORC_QB ? (q0[ch] + nq[ch] - qa) : ORC_QB;
            float best[ORC_QB], ra[ORC_QB], rmin = INFINITY;
            int bi[ORC_QB], skip = 1;
            for (int j = 0; j < nb; ++j) {
                best[j] = ORC_SINGLE_INF;
                bi[j] = -1;
                ra[j] = R[qa + j];
                if (ra[j] < rmin) rmin = ra[j];
                if (ra[j] != ra[j]) skip = 0;     /* a NaN query masks nothing: no block-wide skip */
            }
            stage_f32(aT, F, qa, nb, nC);
            for (int r = roff[ch]; r < roff[ch + 1]; ++r)
                for (int c = rs[r]; c < rs[r] + rn[r]; ++c) {
                    if (skip && R[c] <= rmin) continue;       /* masked for every query of the block */
                    float dd[ORC_QB];
                    dist2_fma_qb(dd, F + (size_t)c * nC, aT, nC);
                    for (int j = 0; j < nb; ++j) {
                        if (R[c] <= ra[j]) continue;
                        const float d = dd[j];
                        if (!(d > 0.0f) || !(d < ORC_SINGLE_INF)) continue;
                        if (bi[j] < 0 || d < best[j] || (d == best[j] && c < bi[j])) { best[j] = d; bi[j] = c; }
                    }
                }
            for (int j = 0; j < nb; ++j) {
                nn[qa + j - q_base] = (bi[j] < 0 ? qa + j : bi[j]) + 1;
                d2out[qa + j - q_base] = best[j];
            }
        }
        free(aT);
    }
    free(B.off);
}

/* irc_cuda_delta_drift.cu:28-131 (jrc3_cuda_delta_drift).  vnConst = {n1,
 * n12, nC}.  For query i1 (site s = site1[i1], rho R[i1]) the candidates j
 * of the n12 window with R[j] > R[i1] (masked when R[j] <= R[i1]) and a site
 * match (primary features when site1[j] == s, else secondary when
 * site2[j] == s); distance query minus candidate, fused per feature; each
 * of the nT = 128 threads keeps its first strict minimum over j = t, t+nT,
 * ...; the lowest thread holding the overall minimum wins; no candidate ->
 * SINGLE_INF and the query itself.  delta = sqrt(min / dc2) (the source's
 * ABS applies to a non-negative value), nneigh = index + 1. */
void orc_delta_drift(float *vrDelta1, uint32_t *viNneigh1, const int32_t *miSite12, const float *mrFet1,
                     const float *mrFet2, const float *vrRho1, const int32_t *vnConst, float dc2)
{
    const int n1 = vnConst[0], n12 = vnConst[1], nC = vnConst[2], nT = 128;
#pragma omp parallel for schedule(dynamic, 4)
    for (int i1 = 0; i1 < n1; ++i1) {
        const int s = miSite12[i1];
        const float *q = mrFet1 + (size_t)i1 * nC;
        const float rq = vrRho1[i1];
        float best = ORC_SINGLE_INF;
        uint32_t bi = (uint32_t)i1;
        for (int t = 0; t < nT; ++t) {
            float tmin = ORC_SINGLE_INF;
            uint32_t timin = (uint32_t)i1;
            for (int j = t; j < n12; j += nT) {
                if (vrRho1[j] <= rq) continue;
                const float *c;
                if (miSite12[j] == s) c = mrFet1 + (size_t)j * nC;
                else if (miSite12[j + n12] == s) c = mrFet2 + (size_t)j * nC;
                else continue;
                float acc = 0.0f;
                for (int k = 0; k < nC; ++k) { float d = q[k] - c[k]; acc = fmaf(d, d, acc); }
                if (acc < tmin) { tmin = acc; timin = (uint32_t)j; }
            }
            if (tmin < best) { best = tmin; bi = timin; }
        }
        vrDelta1[i1] = sqrtf((best < 0 ? -best : best) / dc2);
        viNneigh1[i1] = bi + 1;
    }
}

/* ------------------------------------------------------------------------ */
/* 3d. calc_dc2_drift_ (matlab/irc.m:24582-24608)                            */
/* ------------------------------------------------------------------------ */

/* subsample_vr_ (matlab/irc.m:11322-11337) on a list of n 0-based positions,
 * in place; returns the new length.  Every nSkip-th entry (nSkip =
 * floor(n / nMax) when above 1), then the entries at round(linspace(1, n',
 * nRemove)) removed, MATLAB's linspace being d1 + ((0:m-1) (d2 - d1)) / (m-1)
 * with its first and last points set to d1 and d2 (a one-point linspace is
 * d2), MATLAB's round half away from zero. */
static int dc2_subsample(int32_t *vi, int n, int nMax)
{
    if (n <= nMax) return n;
    const int nSkip = n / nMax;
    if (nSkip > 1) {
        int m = 0;
        for (int i = 0; i < n; i += nSkip) vi[m++] = vi[i];
        n = m;
    }
    if (n > nMax) {
        const int nRemove = n - nMax;
        char *rm = (char *)calloc((size_t)n, 1);
        for (int i = 0; i < nRemove; ++i) {
            double y;
            if (nRemove == 1) y = n;
            else if (i == 0) y = 1.0;
            else if (i == nRemove - 1) y = n;
            else y = 1.0 + ((double)i * ((double)n - 1.0)) / (double)(nRemove - 1);
            long r = lround(y);
            if (r < 1) r = 1;
            if (r > n) r = n;
            rm[r - 1] = 1;
        }
        int m = 0;
        for (int i = 0; i < n; ++i)
            if (!rm[i]) vi[m++] = vi[i];
        free(rm);
        n = m;
    }
    return n;
}

static int cmp_float_nan_last(const void *pa, const void *pb)
{
    const float a = *(const float *)pa, b = *(const float *)pb;
    const int na = a != a, nb = b != b;
    if (na || nb) return na - nb;
    return (a > b) - (a < b);
}

/* MATLAB median of single values: NaN if any (or none); the middle value, or
 * a + (b - a) / 2 of the two middle values ((a + b) / 2 when their signs
 * differ or one is infinite). */
static float dc2_median(float *v, int n)
{
    if (n == 0) return NAN;
    for (int i = 0; i < n; ++i)
        if (v[i] != v[i]) return NAN;
    qsort(v, (size_t)n, sizeof(float), cmp_float_nan_last);
    if (n & 1) return v[n / 2];
    const float a = v[n / 2 - 1], b = v[n / 2];
    if (signbit(a) != signbit(b) || isinf(a) || isinf(b)) return (a + b) / 2.0f;
    return a + (b - a) / 2.0f;
}

/* calc_dc2_drift_: window of n12 spikes (its own chunk's n1 first), sites
 * 1-based (viSite1 primary, viSite2 secondary), features F1 / F2 [n12 x nC]
 * (primary / secondary, MATLAB [nC x n12]).  Per site: queries = subsample of
 * the own spikes on the site (dc_subsample), candidates = subsample of the
 * window spikes with that primary site (4 dc_subsample, F1) then of those with
 * that secondary site (4 dc_subsample, F2); squared distances in eucl2_dist_'s
 * expansion form yy + (xx - 2 xy) (yy, xx: rounded squares summed in feature
 * order; xy: fused multiply-adds in feature order), each query's sorted
 * distances cut at entry ceil(n2 * dc_percent / 100); site dc2 = median over
 * its queries.  Returns the nanmedian over sites; dc2_site [nSites] (NULL
 * allowed) receives the per-site values (NaN for a site without queries). */
float orc_calc_dc2_drift(float *dc2_site, int n1, int n12, int nC, const int32_t *viSite1, const int32_t *viSite2,
                         const float *F1, const float *F2, int nSites, int dc_subsample, double dc_percent)
{
    int32_t *v11 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n12 + 1));
    int32_t *v21 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n12 + 1));
    int32_t *v22 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n12 + 1));
    float *sites = (float *)malloc(sizeof(float) * (size_t)nSites);
    int ns = 0;
    for (int s = 0; s < nSites; ++s) {
        const int site = s + 1;
        int a = 0, b = 0, c = 0;
        for (int i = 0; i < n12; ++i) {
            if (i < n1 && viSite1[i] == site) v11[a++] = i;
            if (viSite1[i] == site) v21[b++] = i;
            if (viSite2[i] == site) v22[c++] = i;
        }
        a = dc2_subsample(v11, a, dc_subsample);
        b = dc2_subsample(v21, b, 4 * dc_subsample);
        c = dc2_subsample(v22, c, 4 * dc_subsample);
        const int n2 = b + c;
        float m = NAN;
        if (a > 0 && n2 > 0) {
            const int icut = (int)ceil((double)n2 * dc_percent / 100.0);
            float *d = (float *)malloc(sizeof(float) * (size_t)n2);
            float *cut = (float *)malloc(sizeof(float) * (size_t)a);
            for (int q = 0; q < a; ++q) {
                const float *y = F1 + (size_t)v11[q] * nC;
                float yy = 0.0f;
                for (int k = 0; k < nC; ++k) yy = yy + y[k] * y[k];
                for (int j = 0; j < n2; ++j) {
                    const float *x = j < b ? F1 + (size_t)v21[j] * nC : F2 + (size_t)v22[j - b] * nC;
                    float xx = 0.0f, xy = 0.0f;
                    for (int k = 0; k < nC; ++k) {
                        xx = xx + x[k] * x[k];
                        xy = fmaf(x[k], y[k], xy);
                    }
                    d[j] = yy + (xx - 2.0f * xy);
                }
                qsort(d, (size_t)n2, sizeof(float), cmp_float_nan_last);
                cut[q] = d[icut - 1];
            }
            m = dc2_median(cut, a);
            free(d);
            free(cut);
        }
        if (dc2_site) dc2_site[s] = m;
        if (m == m) sites[ns++] = m;
    }
    const float r = dc2_median(sites, ns);
    free(v11); free(v21); free(v22); free(sites);
    return r;
}
