/*
 * irc_oracle_cluster.c -- CPU oracle for the clustering step that consumes
 * rho, delta, nneigh and the kNN lists.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this file; only the tests, the smoke check and the CPU-baseline leg of
 * the benchmark use it, as the checker.
 *
 *   orc_sort_rho            the output normalisation of sort_:
 *                           rho = rho / max(rho); [~, ordrho] = sort(rho, 'descend')
 *                           matlab/irc2.m:3263-3264
 *   orc_assign_cluster_knn  postCluster_ (matlab/irc2.m:6520-6535) with
 *                           assignCluster_knn_ (:6640-6694), cell2map_
 *                           (:6754-6805) and dpclus_remove_count_ (:6735-6750)
 *
 * The MATLAB code is restated step by step with the same visiting orders, so
 * that its order-dependent results (the overwrite order of cell2map_'s set
 * unions, the ten-pass caps, the in-place label propagation along nneigh in
 * ordrho order) come out the same.  Indices are 1-based at the interface,
 * as in MATLAB.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* MATLAB sort(..., 'descend') on single data: NaN first, then larger first,
 * equal elements in their original order. */
static int desc_before(float x, float y)
{
    const int nx = isnan(x), ny = isnan(y);
    if (nx || ny) return nx && !ny;
    return x > y;
}

/* stable bottom-up merge sort of pos[0..n) by key[pos[.]] under desc_before */
static void msort_desc(int64_t *pos, const float *key, int64_t n)
{
    int64_t *tmp = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    for (int64_t w = 1; w < n; w *= 2) {
        for (int64_t lo = 0; lo < n; lo += 2 * w) {
            int64_t mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
            int64_t a = lo, b = mid, o = lo;
            while (a < mid && b < hi)
                tmp[o++] = desc_before(key[pos[b]], key[pos[a]]) ? pos[b++] : pos[a++];
            while (a < mid) tmp[o++] = pos[a++];
            while (b < hi) tmp[o++] = pos[b++];
        }
        memcpy(pos, tmp, (size_t)n * sizeof(int64_t));
    }
    free(tmp);
}

/* vrRho = vrRho / max(vrRho); [~, ordrho] = sort(vrRho, 'descend').
 * MATLAB's max skips NaN (all NaN -> NaN); the division is single
 * precision.  ordrho is 1-based. */
void orc_sort_rho(float *rho, int64_t *ordrho, int64_t n)
{
    float m = NAN;
    for (int64_t i = 0; i < n; ++i)
        if (!isnan(rho[i]) && (isnan(m) || rho[i] > m)) m = rho[i];
    for (int64_t i = 0; i < n; ++i) rho[i] = rho[i] / m;
    for (int64_t i = 0; i < n; ++i) ordrho[i] = i;
    msort_desc(ordrho, rho, n);
    for (int64_t i = 0; i < n; ++i) ordrho[i] += 1;
}

typedef struct { int32_t *v; int64_t n; } ilist;

static int cmp_i32(const void *a, const void *b)
{
    const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

typedef struct { int64_t val; int32_t col; } vc_pair;

static int cmp_vc(const void *a, const void *b)
{
    const vc_pair *x = (const vc_pair *)a, *y = (const vc_pair *)b;
    if (x->val != y->val) return (x->val > y->val) - (x->val < y->val);
    return (x->col > y->col) - (x->col < y->col);
}

/*
 * assignCluster_knn_ + dpclus_remove_count_.
 *
 *   viClu     [nSpk]  out: cluster label per spike (0 = unassigned)
 *   icl       [nSpk]  out: the cluster centres, 1-based spike ids (first counts[0])
 *   vnSpk_clu [nSpk]  out: spikes per cluster (first counts[0])
 *   counts    [3]     out: nClu (after dpclus_remove_count_), nClu_pre
 *                          (peaks with delta >= delta_cut), nClu_post (after
 *                          the kNN-overlap merge)
 *   rho, delta [nSpk] normalised rho and delta (single)
 *   ordrho    [nSpk]  1-based spike ids in descending rho order
 *   nneigh    [nSpk]  1-based spike id of the nearest higher-rho spike
 *   miKnn     [knn x nSpk] column-major kNN lists (any int64 values;
 *                          only equality between them matters)
 *
 * Returns 0, or -1 when an index that MATLAB would evaluate is out of range
 * (MATLAB raises an error there).
 */
int orc_assign_cluster_knn(int32_t *viClu, int64_t *icl, int32_t *vnSpk_clu, int64_t *counts,
                           const float *rho, const float *delta, const int64_t *ordrho,
                           const int64_t *nneigh, const int64_t *miKnn, int knn, int64_t nSpk,
                           float delta_cut, int min_count)
{
    int rc = 0;
    if (nSpk < 1 || knn < 1) return -1;

    /* viSpk_peak = find(vrDelta_spk(:) >= delta_cut)   :6645 */
    int64_t nPk = 0;
    for (int64_t s = 0; s < nSpk; ++s) nPk += (delta[s] >= delta_cut);
    int64_t *pk = (int64_t *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(int64_t));
    nPk = 0;
    for (int64_t s = 0; s < nSpk; ++s)
        if (delta[s] >= delta_cut) pk[nPk++] = s;          /* 0-based here */
    counts[1] = nPk;

    /* [vrRho_peak, ix_] = sort(vrRho_spk(viSpk_peak), 'descend')   :6654 */
    float *rpk = (float *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(float));
    int64_t *ix = (int64_t *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(int64_t));
    for (int64_t i = 0; i < nPk; ++i) { rpk[i] = rho[pk[i]]; ix[i] = i; }
    msort_desc(ix, rpk, nPk);
    int64_t *pks = (int64_t *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(int64_t));
    for (int64_t i = 0; i < nPk; ++i) pks[i] = pk[ix[i]];

    /* cvi_peak{i} = find(any(ismember(miKnn_peak, miKnn_peak(:,i))))'   :6662
     * = the columns j holding any element of column i, ascending.  Found
     * through the (value, column) pairs sorted by value. */
    ilist *cvi = (ilist *)calloc((size_t)(nPk > 0 ? nPk : 1), sizeof(ilist));
    {
        const int64_t nE = nPk * (int64_t)knn;
        vc_pair *E = (vc_pair *)malloc((size_t)(nE > 0 ? nE : 1) * sizeof(vc_pair));
        for (int64_t j = 0; j < nPk; ++j)
            for (int k = 0; k < knn; ++k) {
                E[j * knn + k].val = miKnn[pks[j] * knn + k];
                E[j * knn + k].col = (int32_t)j;
            }
        qsort(E, (size_t)nE, sizeof(vc_pair), cmp_vc);
        int64_t *mark = (int64_t *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(int64_t));
        for (int64_t j = 0; j < nPk; ++j) mark[j] = -1;
        int32_t *buf = (int32_t *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(int32_t));
        for (int64_t i = 0; i < nPk; ++i) {
            int64_t nb = 0;
            for (int k = 0; k < knn; ++k) {
                const int64_t v = miKnn[pks[i] * knn + k];
                int64_t lo = 0, hi = nE;                 /* first pair with val >= v */
                while (lo < hi) { int64_t md = (lo + hi) / 2; if (E[md].val < v) lo = md + 1; else hi = md; }
                for (int64_t p = lo; p < nE && E[p].val == v; ++p)
                    if (mark[E[p].col] != i) { mark[E[p].col] = i; buf[nb++] = E[p].col; }
            }
            qsort(buf, (size_t)nb, sizeof(int32_t), cmp_i32);
            cvi[i].n = nb;
            cvi[i].v = (int32_t *)malloc((size_t)nb * sizeof(int32_t));
            memcpy(cvi[i].v, buf, (size_t)nb * sizeof(int32_t));
        }
        free(E); free(mark); free(buf);
    }

    /* cell2map_(cvi_peak, [], fParfor)   :6754-6805 (0-based sets here) */
    int64_t *viMapClu = (int64_t *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(int64_t));
    int64_t *uniq = (int64_t *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(int64_t));
    int64_t nUniq = 0;
    {
        ilist *U = (ilist *)calloc((size_t)(nPk > 0 ? nPk : 1), sizeof(ilist));
        int64_t *owner = (int64_t *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(int64_t));
        int64_t *mark = (int64_t *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(int64_t));
        int32_t *buf = (int32_t *)malloc((size_t)(nPk > 0 ? nPk : 1) * sizeof(int32_t));
        for (int rep = 0; rep < 10; ++rep) {
            for (int64_t m = 0; m < nPk; ++m) { owner[m] = -1; mark[m] = -1; }
            /* for iClu = find(numel > 1): viClu1 = unique([cvi{iClu}; cvi{cvi{iClu}}]);
             *                            cvi_clu1(viClu1) = {viClu1}  (later iClu overwrite) */
            for (int64_t i = 0; i < nPk; ++i) {
                U[i].n = 0;
                if (cvi[i].n <= 1) continue;
                int64_t nb = 0;
                for (int64_t a = 0; a < cvi[i].n; ++a) {
                    const int32_t x = cvi[i].v[a];
                    if (mark[x] != i) { mark[x] = i; buf[nb++] = x; }
                }
                for (int64_t a = 0; a < cvi[i].n; ++a) {
                    const ilist *cm = &cvi[cvi[i].v[a]];
                    for (int64_t b = 0; b < cm->n; ++b) {
                        const int32_t x = cm->v[b];
                        if (mark[x] != i) { mark[x] = i; buf[nb++] = x; }
                    }
                }
                qsort(buf, (size_t)nb, sizeof(int32_t), cmp_i32);
                U[i].v = (int32_t *)malloc((size_t)nb * sizeof(int32_t));
                memcpy(U[i].v, buf, (size_t)nb * sizeof(int32_t));
                U[i].n = nb;
                for (int64_t a = 0; a < nb; ++a) owner[buf[a]] = i;
            }
            /* if all(cellfun(@numel, cvi_clu1) == cellfun(@numel, cvi_clu)) break */
            int same = 1;
            for (int64_t m = 0; m < nPk && same; ++m)
                same = ((owner[m] >= 0 ? U[owner[m]].n : 0) == cvi[m].n);
            if (!same) {
                ilist *nc = (ilist *)calloc((size_t)(nPk > 0 ? nPk : 1), sizeof(ilist));
                for (int64_t m = 0; m < nPk; ++m)
                    if (owner[m] >= 0) {
                        nc[m].n = U[owner[m]].n;
                        nc[m].v = (int32_t *)malloc((size_t)nc[m].n * sizeof(int32_t));
                        memcpy(nc[m].v, U[owner[m]].v, (size_t)nc[m].n * sizeof(int32_t));
                    }
                for (int64_t m = 0; m < nPk; ++m) free(cvi[m].v);
                free(cvi);
                cvi = nc;
            }
            for (int64_t i = 0; i < nPk; ++i) { free(U[i].v); U[i].v = NULL; U[i].n = 0; }
            if (same) break;
        }
        free(U); free(owner); free(mark); free(buf);

        /* viMapClu(iClu) = min(cvi_clu{iClu}) where non-empty, else iClu;
         * viUniq_ = setdiff(unique(viMapClu), 0); compact to 1..numel(viUniq_) */
        for (int64_t i = 0; i < nPk; ++i) viMapClu[i] = cvi[i].n ? (int64_t)cvi[i].v[0] + 1 : i + 1;
        char *isrep = (char *)calloc((size_t)(nPk > 0 ? nPk : 1) + 1, 1);
        for (int64_t i = 0; i < nPk; ++i) isrep[viMapClu[i]] = 1;
        int64_t *rank = (int64_t *)calloc((size_t)(nPk > 0 ? nPk : 1) + 1, sizeof(int64_t));
        for (int64_t r = 1; r <= nPk; ++r)
            if (isrep[r]) { uniq[nUniq] = r; rank[r] = ++nUniq; }
        for (int64_t i = 0; i < nPk; ++i) viMapClu[i] = rank[viMapClu[i]];
        free(isrep); free(rank);
        for (int64_t m = 0; m < nPk; ++m) free(cvi[m].v);
        free(cvi);
    }

    /* viClu_spk(viSpk_peak) = viMapClu_new; viSpk_peak = viSpk_peak(viiPeak)   :6673-6674 */
    for (int64_t s = 0; s < nSpk; ++s) viClu[s] = 0;
    for (int64_t i = 0; i < nPk; ++i) viClu[pks[i]] = (int32_t)viMapClu[i];
    int64_t nIcl = nUniq;
    for (int64_t k = 0; k < nUniq; ++k) icl[k] = pks[uniq[k] - 1] + 1;

    if (nUniq == 0 || nUniq == 1) {
        /* :6676-6678; only ordrho_spk(1) is read on this branch */
        if (ordrho[0] < 1 || ordrho[0] > nSpk) rc = -1;
        for (int64_t s = 0; s < nSpk; ++s) viClu[s] = 1;
        icl[0] = ordrho[0];
        nIcl = 1;
    } else {
        for (int64_t i = 0; i < nSpk; ++i)        /* viSpk_nneigh(ordrho_spk) */
            if (ordrho[i] < 1 || ordrho[i] > nSpk) rc = -1;
        /* nneigh1 = viSpk_nneigh(ordrho_spk); up to ten in-place passes over the
         * unassigned spikes in ordrho order   :6681-6692 */
        for (int rep = 0; rep < 10 && rc == 0; ++rep) {
            int64_t nvi = 0;
            for (int64_t ii = 0; ii < nSpk; ++ii) nvi += (viClu[ordrho[ii] - 1] <= 0);
            if (nvi == 0) break;
            char *in_vi = (char *)malloc((size_t)nSpk);
            for (int64_t ii = 0; ii < nSpk; ++ii) in_vi[ii] = (viClu[ordrho[ii] - 1] <= 0);
            for (int64_t ii = 0; ii < nSpk; ++ii) {
                if (!in_vi[ii]) continue;
                const int64_t nn = nneigh[ordrho[ii] - 1];
                if (nn < 1 || nn > nSpk) { rc = -1; break; }
                viClu[ordrho[ii] - 1] = viClu[nn - 1];
            }
            free(in_vi);
            int64_t n1 = 0;
            for (int64_t s = 0; s < nSpk; ++s) n1 += (viClu[s] <= 0);
            if (n1 == 0) break;
        }
    }
    counts[2] = nIcl;

    /* dpclus_remove_count_(viClu, icl, min_count)   :6735-6750 */
    {
        int64_t *cnt = (int64_t *)calloc((size_t)nIcl + 1, sizeof(int64_t));
        for (int64_t s = 0; s < nSpk; ++s)
            if (viClu[s] >= 1 && viClu[s] <= nIcl) cnt[viClu[s]]++;
        int64_t *viMap = (int64_t *)calloc((size_t)nIcl + 1, sizeof(int64_t));
        int64_t nKeep = 0;
        for (int64_t c = 1; c <= nIcl; ++c)
            if (cnt[c] >= min_count) viMap[c] = ++nKeep;
        if (nKeep < nIcl) {
            for (int64_t s = 0; s < nSpk; ++s)
                viClu[s] = (viClu[s] >= 1 && viClu[s] <= nIcl) ? (int32_t)viMap[viClu[s]] : 0;
            int64_t o = 0;
            for (int64_t c = 1; c <= nIcl; ++c)
                if (viMap[c]) { icl[o] = icl[c - 1]; vnSpk_clu[o] = (int32_t)cnt[c]; ++o; }
        } else {
            for (int64_t c = 1; c <= nIcl; ++c) vnSpk_clu[c - 1] = (int32_t)cnt[c];
        }
        counts[0] = nKeep;
        free(cnt); free(viMap);
    }

    free(pk); free(rpk); free(ix); free(pks); free(viMapClu); free(uniq);
    return rc;
}
