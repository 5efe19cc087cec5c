/* Declaration-only stand-in for MATLAB's mex.h / matrix.h (the public C API
 * signatures the gateway uses), so tests can type-check mex/ircgb300_mex.c
 * against include/ircgb300.h without MATLAB.  Nothing here links or runs. */
#pragma once
#include <stdbool.h>
#include <stddef.h>
#include <stdio.h>

typedef size_t mwSize;
typedef size_t mwIndex;
typedef struct mxArray_tag mxArray;
typedef bool mxLogical;
typedef enum {
    mxUNKNOWN_CLASS, mxCELL_CLASS, mxSTRUCT_CLASS, mxLOGICAL_CLASS, mxCHAR_CLASS, mxVOID_CLASS, mxDOUBLE_CLASS,
    mxSINGLE_CLASS, mxINT8_CLASS, mxUINT8_CLASS, mxINT16_CLASS, mxUINT16_CLASS, mxINT32_CLASS, mxUINT32_CLASS,
    mxINT64_CLASS, mxUINT64_CLASS
} mxClassID;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;

double mxGetScalar(const mxArray *a);
size_t mxGetNumberOfElements(const mxArray *a);
void *mxGetData(const mxArray *a);
double *mxGetPr(const mxArray *a);
mxLogical *mxGetLogicals(const mxArray *a);
mxArray *mxGetCell(const mxArray *a, mwIndex i);
char *mxArrayToString(const mxArray *a);
int mxGetString(const mxArray *a, char *buf, mwSize n);
void mxSetM(mxArray *a, mwSize m);
void mxSetN(mxArray *a, mwSize n);
mxArray *mxCreateDoubleScalar(double v);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity c);
void mxDestroyArray(mxArray *a);
void *mxMalloc(mwSize n);
void *mxCalloc(mwSize n, mwSize size);
void mxFree(void *p);
bool mxIsGPUArray(const mxArray *a);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
void mexErrMsgTxt(const char *msg);
