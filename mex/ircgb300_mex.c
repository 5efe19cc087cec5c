/*
 * ircgb300_mex.c -- MATLAB / Octave gateway to libircgb300.so.
 *
 * Replaces `feval(CK, out1, out2, in..., vnConst)` of the reference's
 * parallel.gpu.CUDAKernel objects with one MEX call per kernel, keeping the
 * argument order, shapes and outputs:
 *
 *   [D, I] = ircgb300_mex('search_min_drift',   F, IBB, NBB, vnConst, nThreads [, mode, knn])
 *   [D, I] = ircgb300_mex('search_delta_drift', F, R, IBB, NBB, vnConst, nThreads)
 *   [K, I] = ircgb300_mex('cuda_knn_index',     B, A, vnConst, nThreads)
 *   [D, N] = ircgb300_mex('cuda_delta_knn',     B, A, R_B, R_A, vnConst, nThreads)
 *   rho    = ircgb300_mex('rho_drift',          miSite12, mrFet1, mrFet2, vnConst, dc2)
 *   [D, N] = ircgb300_mex('delta_drift',        miSite12, mrFet1, mrFet2, vrRho1, vnConst, dc2)
 *   [dc2, vrDc2_site] = ircgb300_mex('calc_dc2_drift', n1, viSite1, viSite2, mrFet1, mrFet2, nSites,
 *                                    dc_subsample, dc_percent)
 *   K      = ircgb300_mex('cuda_knn',           B, A, vnConst, nThreads)
 *   [K, I] = ircgb300_mex('cuda_knn_full',      B, A, vnConst, nThreads)
 *   [K, I] = ircgb300_mex('cuda_knn_ib',        B, A, IB, vnConst, nThreads)
 *   rho    = ircgb300_mex('cuda_rho',           mrFet12, viiSpk12_ord, vnConst, dc2)
 *   [D, N] = ircgb300_mex('cuda_delta',         mrFet12, viiSpk12_ord, viiRho12_ord, vnConst, dc2, nThreads)
 *   [miDrift, viLim] = ircgb300_mex('calc_drift', vrAmp, vrPos, nSites, nTime_drift, nTime_batch,
 *                                   nTime_max_drift, nQuantile_drift)
 *   [rho, ordrho] = ircgb300_mex('sort_rho',    vrRho)
 *   [viClu, icl, vnSpk_clu, nClu_pre, nClu_post] =
 *            ircgb300_mex('assign_cluster_knn', rho, delta, ordrho, nneigh, miKnn, delta_cut, min_count)
 *   F      = ircgb300_mex('fet_load_site',      csFiles_fet, vnSpkBefore, vnSpkSite, dimm_fet, mlPc [, viSel])
 *            ircgb300_mex('knn_save_site',      vcFile_knn, fAppend, miKnn, viSpk_out, knn)
 *            ircgb300_mex('sort_save',          vcFile, rho, delta, nneigh, ordrho)
 *   [vrKnn, rho, miKnn, delta, nneigh] =
 *            ircgb300_mex('knn_rho_delta_site', F, q0, nq, roff, rs, rn, q_base, n_out, knn, mode
 *                         [, R [, site_rows, site_dims]])
 *   v      = ircgb300_mex('version')
 *
 * sort_rho replaces `vrRho = vrRho / max(vrRho); [~, ordrho] = sort(vrRho,
 * 'descend')` of sort_ (ordrho comes back as an int64 gpuArray; MATLAB
 * indexes with it as with the double one).  assign_cluster_knn replaces
 * assignCluster_knn_ + dpclus_remove_count_ inside postCluster_; ordrho,
 * nneigh and miKnn [knn x nSpk] are int64 gpuArrays (S_clu.nneigh already
 * is; pass int64(ordrho) and the kNN lists the path kept on the device
 * instead of the _knn_<site>.irc files), icl and vnSpk_clu come back on the
 * host.
 *
 * knn_rho_delta_site runs one page of a site (or a batch of sites) through
 * irc_plan_create + irc_knn_rho_delta_site + irc_plan_destroy: F is the
 * single [nC x nF] gpuArray, the plan arrays are host int32 vectors with
 * 0-based rows (the run selection of search_knn_drift_, as
 * ironclust_gb300/drift.py:build_plan builds it), mode 0 REF, 1 EXACT,
 * 2 BF16, 3 FP8; R (optional, single [nF]) is the rho of every column when
 * the queries are not all of F.  miKnn / nneigh are 1-based into F.
 *
 * Array arguments are gpuArrays (single / int32 as the reference kernels
 * take them); vnConst may be a host or a gpuArray int32 vector (it is read on
 * the host).  A failed call raises 'ircgb300:<status>' so the reference's
 * try/catch falls back to its CPU path exactly as before.
 *
 * Build (MATLAB): mex -R2018a -I../include ircgb300_mex.c -L.. -lircgb300 -lmwgpu
 * MATLAB's mex.h and gpu/mxGPUArray.h are required; without them (as in a
 * plain C build) the file compiles to nothing.
 */
#if defined(MATLAB_MEX_FILE)
#include <stdint.h>
#include <string.h>

#include "gpu/mxGPUArray.h"
#include "ircgb300.h"
#include "mex.h"

static void fail(int rc, const char *what)
{
    char id[64];
    snprintf(id, sizeof(id), "ircgb300:status%d", -rc);
    mexErrMsgIdAndTxt(id, "%s: %s (%s)", what, irc_status_string(rc), irc_last_error());
}

static const mxGPUArray *gin(const mxArray *a) { return mxGPUCreateFromMxArray(a); }

static void host_i32(const mxArray *a, int32_t *out, int n)
{
    if (mxIsGPUArray(a)) {
        const mxGPUArray *g = mxGPUCreateFromMxArray(a);
        mxArray *h = mxGPUCreateMxArrayOnCPU(g);
        memcpy(out, mxGetData(h), sizeof(int32_t) * (size_t)n);
        mxDestroyArray(h);
        mxGPUDestroyGPUArray(g);
    } else {
        memcpy(out, mxGetData(a), sizeof(int32_t) * (size_t)n);
    }
}

static mxGPUArray *gout(mwSize rows, mwSize cols, mxClassID cls)
{
    mwSize dims[2] = {rows, cols};
    return mxGPUCreateGPUArray(2, dims, cls, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    char cmd[64];
    int32_t vn[5];
    int rc = IRC_OK;
    if (nrhs < 1 || mxGetString(prhs[0], cmd, sizeof(cmd)) != 0) mexErrMsgTxt("ircgb300_mex: command string expected");
    mxInitGPU();
    if (!strcmp(cmd, "version")) {
        plhs[0] = mxCreateDoubleScalar((double)irc_version());
        return;
    }
    if (!strcmp(cmd, "search_min_drift") || !strcmp(cmd, "search_delta_drift")) {
        const int delta = !strcmp(cmd, "search_delta_drift");
        const int a = delta ? 1 : 0;                      /* extra R argument */
        const mxGPUArray *F = gin(prhs[1]);
        const mxGPUArray *R = delta ? gin(prhs[2]) : NULL;
        const mxGPUArray *IBB = gin(prhs[2 + a]), *NBB = gin(prhs[3 + a]);
        host_i32(prhs[4 + a], vn, 5);
        const int nT = (int)mxGetScalar(prhs[5 + a]);
        const int mode = (!delta && nrhs > 6) ? (int)mxGetScalar(prhs[6]) : IRC_MODE_REF;
        const int knn = (!delta && nrhs > 7) ? (int)mxGetScalar(prhs[7]) : 30;
        mxGPUArray *D = gout((mwSize)nT, (mwSize)vn[4], mxSINGLE_CLASS);
        mxGPUArray *I = gout((mwSize)nT, (mwSize)vn[4], mxINT32_CLASS);
        if (delta)
            rc = irc_search_delta_drift((float *)mxGPUGetData(D), (int32_t *)mxGPUGetData(I),
                                        (const float *)mxGPUGetDataReadOnly(F), (const float *)mxGPUGetDataReadOnly(R),
                                        (const int32_t *)mxGPUGetDataReadOnly(IBB),
                                        (const int32_t *)mxGPUGetDataReadOnly(NBB), vn, nT, NULL);
        else
            rc = irc_search_min_drift((float *)mxGPUGetData(D), (int32_t *)mxGPUGetData(I),
                                      (const float *)mxGPUGetDataReadOnly(F), (const int32_t *)mxGPUGetDataReadOnly(IBB),
                                      (const int32_t *)mxGPUGetDataReadOnly(NBB), vn, nT, mode, knn, NULL);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(D);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(I);
        mxGPUDestroyGPUArray(D); mxGPUDestroyGPUArray(I);
        mxGPUDestroyGPUArray(F); mxGPUDestroyGPUArray(IBB); mxGPUDestroyGPUArray(NBB);
        if (R) mxGPUDestroyGPUArray(R);
        return;
    }
    if (!strcmp(cmd, "cuda_knn_index")) {
        const mxGPUArray *B = gin(prhs[1]), *A = gin(prhs[2]);
        host_i32(prhs[3], vn, 4);
        const int nT = (int)mxGetScalar(prhs[4]);
        mxGPUArray *K = gout((mwSize)vn[1], 1, mxSINGLE_CLASS);
        mxGPUArray *I = gout((mwSize)vn[3], (mwSize)vn[1], mxINT32_CLASS);
        rc = irc_cuda_knn_index((float *)mxGPUGetData(K), (int32_t *)mxGPUGetData(I),
                                (const float *)mxGPUGetDataReadOnly(B), (const float *)mxGPUGetDataReadOnly(A), vn, nT,
                                NULL);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(K);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(I);
        mxGPUDestroyGPUArray(K); mxGPUDestroyGPUArray(I); mxGPUDestroyGPUArray(B); mxGPUDestroyGPUArray(A);
        return;
    }
    if (!strcmp(cmd, "cuda_delta_knn")) {
        const mxGPUArray *B = gin(prhs[1]), *A = gin(prhs[2]), *RB = gin(prhs[3]), *RA = gin(prhs[4]);
        host_i32(prhs[5], vn, 3);
        const int nT = (int)mxGetScalar(prhs[6]);
        mxGPUArray *D = gout((mwSize)vn[1], 1, mxSINGLE_CLASS);
        mxGPUArray *N = gout((mwSize)vn[1], 1, mxUINT32_CLASS);
        rc = irc_cuda_delta_knn((float *)mxGPUGetData(D), (uint32_t *)mxGPUGetData(N),
                                (const float *)mxGPUGetDataReadOnly(B), (const float *)mxGPUGetDataReadOnly(A),
                                (const float *)mxGPUGetDataReadOnly(RB), (const float *)mxGPUGetDataReadOnly(RA), vn,
                                nT, NULL);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(D);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(N);
        mxGPUDestroyGPUArray(D); mxGPUDestroyGPUArray(N);
        mxGPUDestroyGPUArray(B); mxGPUDestroyGPUArray(A); mxGPUDestroyGPUArray(RB); mxGPUDestroyGPUArray(RA);
        return;
    }
    if (!strcmp(cmd, "rho_drift")) {
        const mxGPUArray *S = gin(prhs[1]), *F1 = gin(prhs[2]), *F2 = gin(prhs[3]);
        host_i32(prhs[4], vn, 3);
        const float dc2 = (float)mxGetScalar(prhs[5]);
        mxGPUArray *rho = gout(1, (mwSize)vn[0], mxSINGLE_CLASS);
        rc = irc_rho_drift((float *)mxGPUGetData(rho), (const int32_t *)mxGPUGetDataReadOnly(S),
                           (const float *)mxGPUGetDataReadOnly(F1), (const float *)mxGPUGetDataReadOnly(F2), vn, dc2,
                           NULL);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(rho);
        mxGPUDestroyGPUArray(rho); mxGPUDestroyGPUArray(S); mxGPUDestroyGPUArray(F1); mxGPUDestroyGPUArray(F2);
        return;
    }
    if (!strcmp(cmd, "delta_drift")) {
        const mxGPUArray *S = gin(prhs[1]), *F1 = gin(prhs[2]), *F2 = gin(prhs[3]), *R = gin(prhs[4]);
        host_i32(prhs[5], vn, 3);
        const float dc2 = (float)mxGetScalar(prhs[6]);
        mxGPUArray *D = gout(1, (mwSize)vn[0], mxSINGLE_CLASS);
        mxGPUArray *N = gout(1, (mwSize)vn[0], mxUINT32_CLASS);
        rc = irc_delta_drift((float *)mxGPUGetData(D), (uint32_t *)mxGPUGetData(N),
                             (const int32_t *)mxGPUGetDataReadOnly(S), (const float *)mxGPUGetDataReadOnly(F1),
                             (const float *)mxGPUGetDataReadOnly(F2), (const float *)mxGPUGetDataReadOnly(R), vn, dc2,
                             NULL);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(D);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(N);
        mxGPUDestroyGPUArray(D); mxGPUDestroyGPUArray(N);
        mxGPUDestroyGPUArray(S); mxGPUDestroyGPUArray(F1); mxGPUDestroyGPUArray(F2); mxGPUDestroyGPUArray(R);
        return;
    }
    if (!strcmp(cmd, "calc_dc2_drift")) {
        const int n1 = (int)mxGetScalar(prhs[1]), n12 = (int)mxGetNumberOfElements(prhs[2]);
        const int nSites = (int)mxGetScalar(prhs[6]);
        const mxGPUArray *F1 = gin(prhs[4]), *F2 = gin(prhs[5]);
        int32_t *s1 = (int32_t *)mxMalloc(sizeof(int32_t) * (size_t)(n12 > 0 ? n12 : 1));
        int32_t *s2 = (int32_t *)mxMalloc(sizeof(int32_t) * (size_t)(n12 > 0 ? n12 : 1));
        host_i32(prhs[2], s1, n12);
        host_i32(prhs[3], s2, n12);
        float dc2 = 0.0f;
        float *site = (float *)mxCalloc((size_t)(nSites > 0 ? nSites : 1), sizeof(float));
        const int nC = n12 > 0 ? (int)(mxGPUGetNumberOfElements(F1) / (size_t)n12) : 0;
        rc = irc_calc_dc2_drift(&dc2, site, n1, n12, nC, s1, s2, (const float *)mxGPUGetDataReadOnly(F1),
                                (const float *)mxGPUGetDataReadOnly(F2), nSites, (int)mxGetScalar(prhs[7]),
                                mxGetScalar(prhs[8]), NULL);
        mxFree(s1);
        mxFree(s2);
        mxGPUDestroyGPUArray(F1);
        mxGPUDestroyGPUArray(F2);
        if (rc != IRC_OK) { mxFree(site); fail(rc, cmd); }
        plhs[0] = mxCreateDoubleScalar((double)dc2);
        if (nlhs > 1) {
            plhs[1] = mxCreateNumericMatrix((mwSize)nSites, 1, mxSINGLE_CLASS, mxREAL);
            memcpy(mxGetData(plhs[1]), site, sizeof(float) * (size_t)nSites);
        }
        mxFree(site);
        return;
    }
    if (!strcmp(cmd, "cuda_knn") || !strcmp(cmd, "cuda_knn_full") || !strcmp(cmd, "cuda_knn_ib")) {
        const int full = !strcmp(cmd, "cuda_knn_full"), ib = !strcmp(cmd, "cuda_knn_ib");
        const mxGPUArray *B = gin(prhs[1]), *A = gin(prhs[2]), *IB = ib ? gin(prhs[3]) : NULL;
        host_i32(prhs[3 + ib], vn, 4);
        const int nT = (int)mxGetScalar(prhs[4 + ib]);
        mxGPUArray *K = full ? gout((mwSize)vn[3], (mwSize)vn[1], mxSINGLE_CLASS) : gout((mwSize)vn[1], 1, mxSINGLE_CLASS);
        mxGPUArray *I = (full || ib) ? gout((mwSize)vn[3], (mwSize)vn[1], mxINT32_CLASS) : NULL;
        const float *pB = (const float *)mxGPUGetDataReadOnly(B), *pA = (const float *)mxGPUGetDataReadOnly(A);
        if (ib)
            rc = irc_cuda_knn_ib((float *)mxGPUGetData(K), (int32_t *)mxGPUGetData(I), pB, pA,
                                 (const int32_t *)mxGPUGetDataReadOnly(IB),
                                 (int)(mxGPUGetNumberOfElements(B) / (mwSize)vn[2]), vn, nT, NULL);
        else if (full)
            rc = irc_cuda_knn_full((float *)mxGPUGetData(K), (int32_t *)mxGPUGetData(I), pB, pA, vn, nT, NULL);
        else
            rc = irc_cuda_knn((float *)mxGPUGetData(K), pB, pA, vn, nT, NULL);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(K);
        if (I && nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(I);
        mxGPUDestroyGPUArray(K);
        if (I) mxGPUDestroyGPUArray(I);
        mxGPUDestroyGPUArray(B); mxGPUDestroyGPUArray(A);
        if (IB) mxGPUDestroyGPUArray(IB);
        return;
    }
    if (!strcmp(cmd, "cuda_rho") || !strcmp(cmd, "cuda_delta")) {
        const int delta = !strcmp(cmd, "cuda_delta");
        const mxGPUArray *F = gin(prhs[1]), *O = gin(prhs[2]), *RR = delta ? gin(prhs[3]) : NULL;
        host_i32(prhs[3 + delta], vn, 5);
        const float dc2 = (float)mxGetScalar(prhs[4 + delta]);
        mxGPUArray *D = gout(1, (mwSize)vn[0], mxSINGLE_CLASS);
        mxGPUArray *N = delta ? gout(1, (mwSize)vn[0], mxUINT32_CLASS) : NULL;
        if (delta)
            rc = irc_cuda_delta((float *)mxGPUGetData(D), (uint32_t *)mxGPUGetData(N),
                                (const float *)mxGPUGetDataReadOnly(F), (const int32_t *)mxGPUGetDataReadOnly(O),
                                (const int32_t *)mxGPUGetDataReadOnly(RR), vn, dc2, (int)mxGetScalar(prhs[6]), NULL);
        else
            rc = irc_cuda_rho((float *)mxGPUGetData(D), (const float *)mxGPUGetDataReadOnly(F),
                              (const int32_t *)mxGPUGetDataReadOnly(O), vn, dc2, NULL);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(D);
        if (N && nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(N);
        mxGPUDestroyGPUArray(D);
        if (N) mxGPUDestroyGPUArray(N);
        mxGPUDestroyGPUArray(F); mxGPUDestroyGPUArray(O);
        if (RR) mxGPUDestroyGPUArray(RR);
        return;
    }
    if (!strcmp(cmd, "calc_drift")) {
        /* miDrift [nTime_batch x n] int32 and viLim [n+1] int64, both 0-based
         * (add 1 for MATLAB); mlDrift = mi2ml_drift_(miDrift + 1) */
        const mxGPUArray *A = gin(prhs[1]), *P = gin(prhs[2]);
        const int nSites = (int)mxGetScalar(prhs[3]), nDrift = (int)mxGetScalar(prhs[4]);
        const int nBatch = (int)mxGetScalar(prhs[5]), nMax = (int)mxGetScalar(prhs[6]);
        const int nQ = (int)mxGetScalar(prhs[7]);
        const int cap = nDrift > 1 ? nDrift : 1, nb = nBatch > 1 ? nBatch : 1;
        mxGPUArray *mi = gout((mwSize)nb, (mwSize)cap, mxINT32_CLASS);
        mxGPUArray *lim = gout((mwSize)cap + 1, 1, mxINT64_CLASS);
        int n = 0;
        rc = irc_calc_drift((int32_t *)mxGPUGetData(mi), (int64_t *)mxGPUGetData(lim), &n,
                            (const float *)mxGPUGetDataReadOnly(A), (const float *)mxGPUGetDataReadOnly(P),
                            (int64_t)mxGPUGetNumberOfElements(A), nSites, nDrift, nBatch, nMax, nQ, NULL);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnCPU(mi);
        mxSetN(plhs[0], (mwSize)n);
        if (nlhs > 1) { plhs[1] = mxGPUCreateMxArrayOnCPU(lim); mxSetM(plhs[1], (mwSize)n + 1); }
        mxGPUDestroyGPUArray(mi); mxGPUDestroyGPUArray(lim); mxGPUDestroyGPUArray(A); mxGPUDestroyGPUArray(P);
        return;
    }
    if (!strcmp(cmd, "fet_load_site")) {
        /* csFiles_fet: cell of load file names; vnSpkBefore, vnSpkSite: double
         * vectors per load; dimm_fet = [nPc, nSites_spk]; mlPc logical;
         * viSel: optional int64 gpuArray, 0-based into the site's records */
        const mxArray *cs = prhs[1];
        const int nLoads = (int)mxGetNumberOfElements(cs);
        char **names = (char **)mxCalloc((size_t)nLoads, sizeof(char *));
        int64_t *bef = (int64_t *)mxCalloc((size_t)nLoads, sizeof(int64_t));
        int64_t *cnt = (int64_t *)mxCalloc((size_t)nLoads, sizeof(int64_t));
        int64_t nRec = 0;
        for (int l = 0; l < nLoads; ++l) {
            names[l] = mxArrayToString(mxGetCell(cs, (mwIndex)l));
            bef[l] = (int64_t)mxGetPr(prhs[2])[l];
            cnt[l] = (int64_t)mxGetPr(prhs[3])[l];
            nRec += cnt[l];
        }
        const int nPc = (int)mxGetPr(prhs[4])[0], nSitesSpk = (int)mxGetPr(prhs[4])[1];
        const mxLogical *ml = mxGetNumberOfElements(prhs[5]) ? mxGetLogicals(prhs[5]) : NULL;
        int nC = nPc * nSitesSpk;
        if (ml) { nC = 0; for (int i = 0; i < nPc * nSitesSpk; ++i) nC += ml[i] ? 1 : 0; }
        const mxGPUArray *sel = nrhs > 6 ? gin(prhs[6]) : NULL;
        const int64_t nOut = sel ? (int64_t)mxGPUGetNumberOfElements(sel) : nRec;
        mxGPUArray *F = gout((mwSize)nC, (mwSize)nOut, mxSINGLE_CLASS);
        int ncOut = 0;
        rc = irc_fet_load_site((float *)mxGPUGetData(F), &ncOut, (const char *const *)names, nLoads, bef, cnt, nPc,
                               nSitesSpk, (const uint8_t *)ml, sel ? (const int64_t *)mxGPUGetDataReadOnly(sel) : NULL,
                               nOut, NULL);
        for (int l = 0; l < nLoads; ++l) mxFree(names[l]);
        mxFree(names); mxFree(bef); mxFree(cnt);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(F);
        mxGPUDestroyGPUArray(F);
        if (sel) mxGPUDestroyGPUArray(sel);
        return;
    }
    if (!strcmp(cmd, "knn_save_site")) {
        char *path = mxArrayToString(prhs[1]);
        const int fAppend = (int)mxGetScalar(prhs[2]);
        const mxGPUArray *K = gin(prhs[3]), *V = gin(prhs[4]);
        const int knn = (int)mxGetScalar(prhs[5]);
        const mwSize *dk = mxGPUGetDimensions(K);
        rc = irc_knn_save_site(path, fAppend, (const int32_t *)mxGPUGetDataReadOnly(K), (int)dk[0], knn,
                               (int64_t)dk[1], (const int64_t *)mxGPUGetDataReadOnly(V),
                               (int64_t)mxGPUGetNumberOfElements(V), NULL);
        mxFree((void *)dk);
        mxFree(path);
        mxGPUDestroyGPUArray(K); mxGPUDestroyGPUArray(V);
        if (rc != IRC_OK) fail(rc, cmd);
        return;
    }
    if (!strcmp(cmd, "sort_save")) {
        char *path = mxArrayToString(prhs[1]);
        const mxGPUArray *R = gin(prhs[2]), *D = gin(prhs[3]), *NN = gin(prhs[4]), *O = gin(prhs[5]);
        rc = irc_sort_save(path, (const float *)mxGPUGetDataReadOnly(R), (const float *)mxGPUGetDataReadOnly(D),
                           (const int64_t *)mxGPUGetDataReadOnly(NN), (const int64_t *)mxGPUGetDataReadOnly(O),
                           (int64_t)mxGPUGetNumberOfElements(R), NULL);
        mxFree(path);
        mxGPUDestroyGPUArray(R); mxGPUDestroyGPUArray(D); mxGPUDestroyGPUArray(NN); mxGPUDestroyGPUArray(O);
        if (rc != IRC_OK) fail(rc, cmd);
        return;
    }
    if (!strcmp(cmd, "knn_rho_delta_site")) {
        if (nrhs < 11)
            mexErrMsgTxt("knn_rho_delta_site: F, q0, nq, roff, rs, rn, q_base, n_out, knn, mode [, R [, site_rows, "
                         "site_dims]]");
        const mxGPUArray *F = gin(prhs[1]);
        const mwSize *fd = mxGPUGetDimensions(F);
        const int nC = (int)fd[0], nF = (int)(mxGPUGetNumberOfElements(F) / (fd[0] ? fd[0] : 1));
        mxFree((void *)fd);
        const int nCh = (int)mxGetNumberOfElements(prhs[2]);
        const int nRuns = (int)mxGetNumberOfElements(prhs[5]);
        if ((int)mxGetNumberOfElements(prhs[3]) != nCh || (int)mxGetNumberOfElements(prhs[4]) != nCh + 1 ||
            (int)mxGetNumberOfElements(prhs[6]) != nRuns)
            mexErrMsgIdAndTxt("ircgb300:shape", "knn_rho_delta_site: plan array sizes disagree");
        int32_t *q0 = (int32_t *)mxMalloc(sizeof(int32_t) * nCh), *nq = (int32_t *)mxMalloc(sizeof(int32_t) * nCh),
                *roff = (int32_t *)mxMalloc(sizeof(int32_t) * (nCh + 1)),
                *rs = (int32_t *)mxMalloc(sizeof(int32_t) * nRuns), *rn = (int32_t *)mxMalloc(sizeof(int32_t) * nRuns);
        host_i32(prhs[2], q0, nCh); host_i32(prhs[3], nq, nCh); host_i32(prhs[4], roff, nCh + 1);
        host_i32(prhs[5], rs, nRuns); host_i32(prhs[6], rn, nRuns);
        const int q_base = (int)mxGetScalar(prhs[7]), n_out = (int)mxGetScalar(prhs[8]);
        const int knn = (int)mxGetScalar(prhs[9]), mode = (int)mxGetScalar(prhs[10]);
        /* R may be [] to keep the rho computed here */
        const mxGPUArray *R = nrhs > 11 && mxGetNumberOfElements(prhs[11]) ? gin(prhs[11]) : NULL;
        irc_plan *plan = NULL;
        rc = irc_plan_create(&plan, q0, nq, roff, rs, rn, nCh, q_base, n_out, nF);
        mxFree(q0); mxFree(nq); mxFree(roff); mxFree(rs); mxFree(rn);
        if (rc != IRC_OK) fail(rc, cmd);
        if (nrhs > 13) {
            /* stacked sites: int32 row starts (nSites + 1, 0-based, last = nF) and
             * widths; features past a site's width are zero (irc_plan_set_site_dims) */
            const int nSites = (int)mxGetNumberOfElements(prhs[13]);
            if ((int)mxGetNumberOfElements(prhs[12]) != nSites + 1) {
                irc_plan_destroy(plan);
                mexErrMsgIdAndTxt("ircgb300:shape", "knn_rho_delta_site: site_rows needs one more entry than site_dims");
            }
            int32_t *r32 = (int32_t *)mxMalloc(sizeof(int32_t) * (nSites + 1));
            int64_t *rows = (int64_t *)mxMalloc(sizeof(int64_t) * (nSites + 1));
            int32_t *dims = (int32_t *)mxMalloc(sizeof(int32_t) * (nSites ? nSites : 1));
            host_i32(prhs[12], r32, nSites + 1);
            host_i32(prhs[13], dims, nSites);
            for (int k = 0; k <= nSites; ++k) rows[k] = r32[k];
            rc = irc_plan_set_site_dims(plan, nSites, rows, dims);
            mxFree(r32); mxFree(rows); mxFree(dims);
            if (rc != IRC_OK) { irc_plan_destroy(plan); fail(rc, cmd); }
        }
        mxGPUArray *vr = gout(n_out, 1, mxSINGLE_CLASS), *rho = gout(n_out, 1, mxSINGLE_CLASS),
                   *mi = gout(knn, n_out, mxINT32_CLASS), *de = gout(n_out, 1, mxSINGLE_CLASS),
                   *nn = gout(n_out, 1, mxINT32_CLASS);
        mxGPUArray *d2 = mode != IRC_MODE_REF ? gout(knn, n_out, mxSINGLE_CLASS) : NULL;
        rc = irc_knn_rho_delta_site(plan, (const float *)mxGPUGetDataReadOnly(F), nC,
                                    R ? (const float *)mxGPUGetDataReadOnly(R) : NULL, knn, mode,
                                    (float *)mxGPUGetData(vr), (float *)mxGPUGetData(rho), (int32_t *)mxGPUGetData(mi),
                                    d2 ? (float *)mxGPUGetData(d2) : NULL, (float *)mxGPUGetData(de),
                                    (int32_t *)mxGPUGetData(nn), NULL);
        if (rc == IRC_OK) rc = irc_plan_check(plan, NULL);
        irc_plan_destroy(plan);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(vr);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(rho);
        if (nlhs > 2) plhs[2] = mxGPUCreateMxArrayOnGPU(mi);
        if (nlhs > 3) plhs[3] = mxGPUCreateMxArrayOnGPU(de);
        if (nlhs > 4) plhs[4] = mxGPUCreateMxArrayOnGPU(nn);
        mxGPUDestroyGPUArray(vr); mxGPUDestroyGPUArray(rho); mxGPUDestroyGPUArray(mi);
        mxGPUDestroyGPUArray(de); mxGPUDestroyGPUArray(nn);
        if (d2) mxGPUDestroyGPUArray(d2);
        if (R) mxGPUDestroyGPUArray(R);
        mxGPUDestroyGPUArray(F);
        return;
    }
    if (!strcmp(cmd, "sort_rho")) {
        const mxGPUArray *R = gin(prhs[1]);
        const mwSize n = mxGPUGetNumberOfElements(R);
        mxGPUArray *rho = mxGPUCopyGPUArray(R);
        mxGPUArray *ord = gout(n, 1, mxINT64_CLASS);
        rc = irc_sort_rho((float *)mxGPUGetData(rho), (int64_t *)mxGPUGetData(ord), (int64_t)n, NULL);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(rho);
        if (nlhs > 1) plhs[1] = mxGPUCreateMxArrayOnGPU(ord);
        mxGPUDestroyGPUArray(rho); mxGPUDestroyGPUArray(ord); mxGPUDestroyGPUArray(R);
        return;
    }
    if (!strcmp(cmd, "assign_cluster_knn")) {
        const mxGPUArray *R = gin(prhs[1]), *De = gin(prhs[2]), *O = gin(prhs[3]), *NN = gin(prhs[4]),
                         *K = gin(prhs[5]);
        if (mxGPUGetClassID(O) != mxINT64_CLASS || mxGPUGetClassID(NN) != mxINT64_CLASS ||
            mxGPUGetClassID(K) != mxINT64_CLASS)
            mexErrMsgIdAndTxt("ircgb300:class", "assign_cluster_knn: ordrho, nneigh and miKnn must be int64");
        const mwSize n = mxGPUGetNumberOfElements(R);
        const int knn = (int)(mxGPUGetNumberOfElements(K) / (n ? n : 1));
        const float cut = (float)mxGetScalar(prhs[6]);
        const int min_count = (int)mxGetScalar(prhs[7]);
        mxGPUArray *viClu = gout(n, 1, mxINT32_CLASS), *icl = gout(n, 1, mxINT64_CLASS),
                   *vnc = gout(n, 1, mxINT32_CLASS);
        int64_t counts[3] = {0, 0, 0};
        rc = irc_assign_cluster_knn((int32_t *)mxGPUGetData(viClu), (int64_t *)mxGPUGetData(icl),
                                    (int32_t *)mxGPUGetData(vnc), (int64_t)n, counts,
                                    (const float *)mxGPUGetDataReadOnly(R), (const float *)mxGPUGetDataReadOnly(De),
                                    (const int64_t *)mxGPUGetDataReadOnly(O), (const int64_t *)mxGPUGetDataReadOnly(NN),
                                    (const int64_t *)mxGPUGetDataReadOnly(K), knn, (int64_t)n, cut, min_count, NULL);
        if (rc != IRC_OK) fail(rc, cmd);
        plhs[0] = mxGPUCreateMxArrayOnGPU(viClu);
        if (nlhs > 1) { plhs[1] = mxGPUCreateMxArrayOnCPU(icl); mxSetM(plhs[1], (mwSize)counts[0]); }
        if (nlhs > 2) { plhs[2] = mxGPUCreateMxArrayOnCPU(vnc); mxSetM(plhs[2], (mwSize)counts[0]); }
        if (nlhs > 3) plhs[3] = mxCreateDoubleScalar((double)counts[1]);
        if (nlhs > 4) plhs[4] = mxCreateDoubleScalar((double)counts[2]);
        mxGPUDestroyGPUArray(viClu); mxGPUDestroyGPUArray(icl); mxGPUDestroyGPUArray(vnc);
        mxGPUDestroyGPUArray(R); mxGPUDestroyGPUArray(De); mxGPUDestroyGPUArray(O); mxGPUDestroyGPUArray(NN);
        mxGPUDestroyGPUArray(K);
        return;
    }
    mexErrMsgIdAndTxt("ircgb300:command", "unknown command '%s'", cmd);
}
#endif /* MATLAB_MEX_FILE */
