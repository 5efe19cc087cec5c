/* Declaration-only stand-in for MATLAB's gpu/mxGPUArray.h (public C API
 * signatures), for type-checking the gateway without MATLAB. */
#pragma once
#include "mex.h"

typedef struct mxGPUArray_tag mxGPUArray;
typedef enum { MX_GPU_DO_NOT_INITIALIZE = 0, MX_GPU_INITIALIZE_VALUES = 1 } mxGPUInitialize;

int mxInitGPU(void);
const mxGPUArray *mxGPUCreateFromMxArray(const mxArray *a);
mxArray *mxGPUCreateMxArrayOnCPU(const mxGPUArray *g);
mxArray *mxGPUCreateMxArrayOnGPU(const mxGPUArray *g);
void mxGPUDestroyGPUArray(const mxGPUArray *g);
mxGPUArray *mxGPUCreateGPUArray(mwSize ndim, const mwSize *dims, mxClassID cls, mxComplexity cx, mxGPUInitialize init);
mxGPUArray *mxGPUCopyGPUArray(const mxGPUArray *g);
void *mxGPUGetData(mxGPUArray *g);
const void *mxGPUGetDataReadOnly(const mxGPUArray *g);
mwSize mxGPUGetNumberOfElements(const mxGPUArray *g);
mxClassID mxGPUGetClassID(const mxGPUArray *g);
const mwSize *mxGPUGetDimensions(const mxGPUArray *g);
