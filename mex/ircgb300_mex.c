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
 *   v      = ircgb300_mex('version')
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
    mexErrMsgIdAndTxt("ircgb300:command", "unknown command '%s'", cmd);
}
#endif /* MATLAB_MEX_FILE */
