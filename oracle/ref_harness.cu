// ref_harness.cu -- launches the reference's own CUDA kernels, unmodified.
//
// TEST INFRASTRUCTURE ONLY (the GPU-side oracle and the same-box timing of
// the reference kernels); the shipped library never links or loads it.
//
// The reference's MATLAB host loads each kernel as PTX through
// parallel.gpu.CUDAKernel('<k>.ptx','<k>.cu') (matlab/irc2.m:3751, :3815;
// matlab/irc.m:24381, :24533, :24627) and launches it with a block size,
// grid size and dynamic shared-memory size set from MATLAB.  This harness
// does the same with the CUDA runtime's library API: the PTX files are
// produced from the reference sources by oracle/build_oracle.py (nvcc -ptx,
// as `irc2 compile`, matlab/irc2.m:7605, does), loaded with
// cudaLibraryLoadData, and launched with the MATLAB launch configuration:
//
//   search_min_drift    block nT (1024),  grid [ceil(nA/64), 8],   smem 4*8*(45+1)
//                       matlab/irc2.m:3755-3757, :3775
//   search_delta_drift  block nT (512),   grid [ceil(nA/256), 16], smem 4*16*(45+2)
//                       matlab/irc2.m:3819-3821, :3840
//   cuda_knn_index      block 512,        grid [ceil(nA/16), 4],   smem 4*4*(45+2*512)
//                       matlab/irc.m:24371, :24382-24385
//   cuda_delta_knn      block 128,        grid [ceil(nA/256), 16], smem 4*16*(45+2*128+1)
//                       matlab/irc.m:24522-24537
//   jrc3_cuda_rho_drift block 128,        grid [ceil(n1/256), 16], smem 4*16*(45+1+2*128)
//                       matlab/irc.m:24619-24631
//   jrc3_cuda_delta_drift block 128,      grid [ceil(n1/256), 16], smem 4*16*(45+2+2*128)
//                       matlab/irc.m:24646-24663
//   cuda_knn            block 256,        grid [ceil(nA/256), 16], smem 4*16*(36+256)
//                       matlab/irc.m:24440-24456 (nThreads = 2 * P.nThreads)
//   cuda_knn_full, cuda_knn_ib
//                       block 512,        grid [ceil(nA/16), 4],   smem 4*4*(60+2*512)
//                       (no MATLAB call site; launched like cuda_knn_index, whose
//                       CHUNK = 4 and NTHREADS = 512 they share)
//   jrc3_cuda_rho       block nT (128),   grid [ceil(n1/256), 16], smem 4*16*(2+48+2*nT)
//                       matlab/irc.m:2542-2551
//   jrc3_cuda_delta     block nT (128),   grid [ceil(n1/256), 16], smem 4*16*(3+48+2*nT)
//                       matlab/irc.m:2664-2673
//
// Every pointer argument is a device pointer, vnConst included (MATLAB passes
// it as a gpuArray).  Each function returns a cudaError_t value (0 = ok).
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

namespace {

enum { K_MIN = 0, K_DELTA, K_KNN, K_DKNN, K_RHO, K_DDRIFT, K_CKNN, K_CKNNF, K_CKNNIB, K_SRHO, K_SDELTA, K_COUNT };
const char *kFiles[K_COUNT] = {"search_min_drift.ptx", "search_delta_drift.ptx",
                               "cuda_knn_index.ptx", "cuda_delta_knn.ptx",
                               "irc_cuda_rho_drift.ptx", "irc_cuda_delta_drift.ptx",
                               "cuda_knn.ptx", "cuda_knn_full.ptx", "cuda_knn_ib.ptx",
                               "irc_cuda_rho.ptx", "irc_cuda_delta.ptx"};
cudaLibrary_t g_lib[K_COUNT];
cudaKernel_t g_kern[K_COUNT];
bool g_loaded = false;

cudaError_t load_one(const std::string &dir, int k)
{
    std::string path = dir + "/" + kFiles[k];
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return cudaErrorFileNotFound;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    char *buf = (char *)malloc((size_t)n + 1);
    size_t got = fread(buf, 1, (size_t)n, f);
    fclose(f);
    buf[got] = 0;
    cudaError_t e = cudaLibraryLoadData(&g_lib[k], buf, nullptr, nullptr, 0, nullptr, nullptr, 0);
    free(buf);
    if (e != cudaSuccess) return e;
    unsigned cnt = 0;
    e = cudaLibraryGetKernelCount(&cnt, g_lib[k]);
    if (e != cudaSuccess) return e;
    if (cnt != 1) return cudaErrorInvalidKernelImage;   // each reference file holds one kernel
    return cudaLibraryEnumerateKernels(&g_kern[k], 1, g_lib[k]);
}

inline unsigned cdiv(long a, long b) { return (unsigned)((a + b - 1) / b); }

cudaError_t launch(int k, dim3 grid, dim3 block, size_t smem, cudaStream_t s, void **args)
{
    if (!g_loaded) return cudaErrorNotReady;
    return cudaLaunchKernel((const void *)g_kern[k], grid, block, args, smem, s);
}

}  // namespace

extern "C" {

int refh_init(const char *ptx_dir)
{
    if (g_loaded) return 0;
    for (int k = 0; k < K_COUNT; ++k) {
        cudaError_t e = load_one(ptx_dir, k);
        if (e != cudaSuccess) return (int)e;
    }
    g_loaded = true;
    return 0;
}

// search_min_drift(float*D,int*I,const float*F,const int*IBB,const int*NBB,const int*vnConst)
int refh_search_min_drift(float *D, int *I, const float *F, const int *IBB, const int *NBB,
                          const int *vnConst_dev, int nT, int nA, void *stream)
{
    const int CHUNK = 8, nC_max = 45;
    void *args[] = {&D, &I, &F, &IBB, &NBB, &vnConst_dev};
    return (int)launch(K_MIN, dim3(cdiv(nA, CHUNK * CHUNK), CHUNK), dim3(nT),
                       4 * CHUNK * (nC_max + 1), (cudaStream_t)stream, args);
}

int refh_search_delta_drift(float *D, int *I, const float *F, const float *R, const int *IBB,
                            const int *NBB, const int *vnConst_dev, int nT, int nA, void *stream)
{
    const int CHUNK = 16, nC_max = 45;
    void *args[] = {&D, &I, &F, &R, &IBB, &NBB, &vnConst_dev};
    return (int)launch(K_DELTA, dim3(cdiv(nA, CHUNK * CHUNK), CHUNK), dim3(nT),
                       4 * CHUNK * (nC_max + 2), (cudaStream_t)stream, args);
}

int refh_cuda_knn_index(float *K, int *I, const float *B, const float *A,
                        const int *vnConst_dev, int nA, void *stream)
{
    const int CHUNK = 4, nC_max = 45, nThreads = 512;
    void *args[] = {&K, &I, &B, &A, &vnConst_dev};
    return (int)launch(K_KNN, dim3(cdiv(nA, CHUNK * CHUNK), CHUNK), dim3(nThreads),
                       4 * CHUNK * (nC_max + nThreads * 2), (cudaStream_t)stream, args);
}

int refh_cuda_delta_knn(float *D, unsigned *N, const float *B, const float *A, const float *R_B,
                        const float *R_A, const int *vnConst_dev, int nA, void *stream)
{
    const int CHUNK = 16, nC_max = 45, nThreads = 128;
    void *args[] = {&D, &N, &B, &A, &R_B, &R_A, &vnConst_dev};
    return (int)launch(K_DKNN, dim3(cdiv(nA, CHUNK * CHUNK), CHUNK), dim3(nThreads),
                       4 * CHUNK * (nC_max + nThreads * 2 + 1), (cudaStream_t)stream, args);
}

int refh_rho_drift(float *vrRho1, const int *miSite12, const float *mrFet1, const float *mrFet2,
                   const int *vnConst_dev, float dc2, int n1, void *stream)
{
    const int CHUNK = 16, nC_max = 45, nThreads = 128;
    void *args[] = {&vrRho1, &miSite12, &mrFet1, &mrFet2, &vnConst_dev, &dc2};
    return (int)launch(K_RHO, dim3(cdiv(n1, CHUNK * CHUNK), CHUNK), dim3(nThreads),
                       4 * CHUNK * (nC_max + 1 + 2 * nThreads), (cudaStream_t)stream, args);
}

// jrc3_cuda_delta_drift: block 128, grid [ceil(n1/256), 16], smem 4*16*(45+2+2*128)
// (matlab/irc.m:24646-24663)
int refh_delta_drift(float *vrDelta1, unsigned *viNneigh1, const int *miSite12, const float *mrFet1,
                     const float *mrFet2, const float *vrRho1, const int *vnConst_dev, float dc2, int n1,
                     void *stream)
{
    const int CHUNK = 16, nC_max = 45, nThreads = 128;
    void *args[] = {&vrDelta1, &viNneigh1, &miSite12, &mrFet1, &mrFet2, &vrRho1, &vnConst_dev, &dc2};
    return (int)launch(K_DDRIFT, dim3(cdiv(n1, CHUNK * CHUNK), CHUNK), dim3(nThreads),
                       4 * CHUNK * (nC_max + 2 + 2 * nThreads), (cudaStream_t)stream, args);
}

// cuda_knn(float*K,const float*B,const float*A,const int*vnConst)
int refh_cuda_knn(float *K, const float *B, const float *A, const int *vnConst_dev, int nA, void *stream)
{
    const int CHUNK = 16, nC_max = 36, nThreads = 256;
    void *args[] = {&K, &B, &A, &vnConst_dev};
    return (int)launch(K_CKNN, dim3(cdiv(nA, CHUNK * CHUNK), CHUNK), dim3(nThreads),
                       4 * CHUNK * (nC_max + nThreads), (cudaStream_t)stream, args);
}

// cuda_knn_full(float*K,int*I,const float*B,const float*A,const int*vnConst)
int refh_cuda_knn_full(float *K, int *I, const float *B, const float *A, const int *vnConst_dev, int nA,
                       void *stream)
{
    const int CHUNK = 4, nC_max = 60, nThreads = 512;
    void *args[] = {&K, &I, &B, &A, &vnConst_dev};
    return (int)launch(K_CKNNF, dim3(cdiv(nA, CHUNK * CHUNK), CHUNK), dim3(nThreads),
                       4 * CHUNK * (nC_max + nThreads * 2), (cudaStream_t)stream, args);
}

// cuda_knn_ib(float*K,int*I,const float*B,const float*A,const int*IB,const int*vnConst)
int refh_cuda_knn_ib(float *K, int *I, const float *B, const float *A, const int *IB, const int *vnConst_dev,
                     int nA, void *stream)
{
    const int CHUNK = 4, nC_max = 60, nThreads = 512;
    void *args[] = {&K, &I, &B, &A, &IB, &vnConst_dev};
    return (int)launch(K_CKNNIB, dim3(cdiv(nA, CHUNK * CHUNK), CHUNK), dim3(nThreads),
                       4 * CHUNK * (nC_max + nThreads * 2), (cudaStream_t)stream, args);
}

// jrc3_cuda_rho(float*vrRho1,const float*mrFet12,const int*viiSpk12_ord,const int*vnConst,const float dc2)
int refh_cuda_rho(float *vrRho1, const float *mrFet12, const int *viiSpk12_ord, const int *vnConst_dev,
                  float dc2, int n1, int nT, void *stream)
{
    const int CHUNK = 16, nC_max = 48;
    void *args[] = {&vrRho1, &mrFet12, &viiSpk12_ord, &vnConst_dev, &dc2};
    return (int)launch(K_SRHO, dim3(cdiv(n1, CHUNK * CHUNK), CHUNK), dim3(nT),
                       4 * CHUNK * (2 + nC_max + 2 * nT), (cudaStream_t)stream, args);
}

// jrc3_cuda_delta(float*vrDelta1,unsigned*viNneigh1,const float*mrFet12,const int*viiSpk12_ord,
//                 const int*viiRho12_ord,const int*vnConst,const float dc2)
int refh_cuda_delta(float *vrDelta1, unsigned *viNneigh1, const float *mrFet12, const int *viiSpk12_ord,
                    const int *viiRho12_ord, const int *vnConst_dev, float dc2, int n1, int nT, void *stream)
{
    const int CHUNK = 16, nC_max = 48;
    void *args[] = {&vrDelta1, &viNneigh1, &mrFet12, &viiSpk12_ord, &viiRho12_ord, &vnConst_dev, &dc2};
    return (int)launch(K_SDELTA, dim3(cdiv(n1, CHUNK * CHUNK), CHUNK), dim3(nT),
                       4 * CHUNK * (3 + nC_max + 2 * nT), (cudaStream_t)stream, args);
}

}  // extern "C"
