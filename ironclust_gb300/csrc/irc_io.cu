// irc_io.cu -- the on-disk formats on either side of the path, read into and
// written from device memory.  All files are raw little-endian arrays, as
// MATLAB's fwrite leaves them (write_bin_, matlab/irc2.m:6891-6920):
//
//   _fet_<load>.irc / _fet2_<load>.irc   (detect_paged_save_,
//       save_paged_fet_site_, matlab/irc2.m:4582-4618)  for every site in
//       turn, that site's spikes of the load as [nPc x nSites_spk] single
//       records (column-major, PC fastest).  irc_fet_load_site reads one
//       site's blocks of every load (load_fet_site_, matlab/irc2.m:4039-4135):
//       file reads into two pinned buffers alternate with asynchronous
//       copies to the device, then one kernel gathers the selected records
//       and applies the feature mask mlPc (get_mlPc_, matlab/irc2.m:3278).
//   _knn_<site>.irc   int64 [knn x n] global spike ids, appended page by
//       page (rho_paged_site_ + save_miKnn_site_, matlab/irc2.m:3670-3679,
//       :3355-3370).  irc_knn_save_site maps the device kNN (1-based
//       positions in the site feature matrix) to global ids, pads the rows
//       to knn by repeating the last, and writes or appends.
//   sort.irc   rho (single), delta (single), nneigh (int64), ordrho
//       (double) concatenated (sort_cache_ + struct_save_bin_,
//       matlab/irc2.m:356-391, :1733-1750).  irc_sort_save / irc_sort_load.
//
// irc_f16_to_f32 widens features kept as FP16 in host memory (streamed in
// half the bytes) after their copy to the device.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <vector>

#include "ircgb300.h"
#include "irc_common.cuh"

namespace {

constexpr size_t kStageBytes = 32u << 20;          // one pinned staging buffer

struct Pinned {
    void *p[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t init(size_t bytes)
    {
        cudaError_t e = cudaSuccess;
        for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
            e = cudaMallocHost(&p[i], bytes);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
        }
        return e;
    }
    ~Pinned()
    {
        for (int i = 0; i < 2; ++i) {
            if (ev[i]) {
                cudaEventSynchronize(ev[i]);
                cudaEventDestroy(ev[i]);
            }
            if (p[i]) cudaFreeHost(p[i]);
        }
    }
};

struct FileCloser {
    FILE *f = nullptr;
    ~FileCloser()
    {
        if (f) fclose(f);
    }
};

// F[k * nC + c] = records[viSel[k]][pcIdx[c]]  (the mask mlPc as a list of
// positions inside one [nPc x nSites_spk] record, in MATLAB's linear order)
__global__ void k_fet_gather(float *__restrict__ F, const float *__restrict__ rec, int recLen,
                             const int64_t *__restrict__ viSel, int64_t nOut, const int *__restrict__ pcIdx, int nC,
                             int64_t nRec, int *__restrict__ bad)
{
    const int64_t k = blockIdx.x * (int64_t)blockDim.y + threadIdx.y;
    if (k >= nOut) return;
    const int64_t r = viSel ? viSel[k] : k;
    if (r < 0 || r >= nRec) {
        if (threadIdx.x == 0) atomicOr(bad, 1);
        return;
    }
    const float *src = rec + r * recLen;
    for (int c = threadIdx.x; c < nC; c += blockDim.x) F[k * nC + c] = src[pcIdx[c]];
}

// rows of the saved kNN: global ids of the (1-based) positions, padded to
// knnOut rows by repeating the last
__global__ void k_knn_global(int64_t *__restrict__ out, const int32_t *__restrict__ miKnn, int knnIn, int knnOut,
                             int64_t n, const int64_t *__restrict__ viSpk, int64_t nF, int *__restrict__ bad)
{
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n * knnOut) return;
    const int64_t i = e / knnOut;
    const int k = (int)(e - i * knnOut);
    const int32_t pos = miKnn[(k < knnIn ? k : knnIn - 1) + (int64_t)knnIn * i];
    if (pos < 1 || pos > nF) {
        atomicOr(bad, 1);
        out[e] = 0;
        return;
    }
    out[e] = viSpk[pos - 1];
}

__global__ void k_i64_to_f64(double *__restrict__ out, const int64_t *__restrict__ in, int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

__global__ void k_f64_to_i64(int64_t *__restrict__ out, const double *__restrict__ in, int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int64_t)in[i];
}

unsigned grid_for(int64_t n, int per) { return (unsigned)((n + per - 1) / per > 0 ? (n + per - 1) / per : 1); }

// Read `bytes` from f at `offset` into dst (device), through the pinned
// buffers: a read into one buffer overlaps the copy out of the other.
int stream_to_device(FILE *f, int64_t offset, int64_t bytes, char *dst, Pinned &pin, cudaStream_t s,
                     const char *name)
{
    if (fseeko(f, (off_t)offset, SEEK_SET) != 0) {
        irc_host::set_error("%s: seek to %lld failed", name, (long long)offset);
        return IRC_E_INVAL;
    }
    int b = 0;
    for (int64_t done = 0; done < bytes; b ^= 1) {
        const size_t n = (size_t)((bytes - done) < (int64_t)kStageBytes ? (bytes - done) : (int64_t)kStageBytes);
        cudaError_t e = cudaEventSynchronize(pin.ev[b]);  // the copy that last used this buffer is done
        if (e != cudaSuccess) return irc_host::cuda_status(e, name);
        if (fread(pin.p[b], 1, n, f) != n) {
            irc_host::set_error("%s: short read at byte %lld", name, (long long)(offset + done));
            return IRC_E_INVAL;
        }
        e = cudaMemcpyAsync(dst + done, pin.p[b], n, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaEventRecord(pin.ev[b], s);
        if (e != cudaSuccess) return irc_host::cuda_status(e, name);
        done += (int64_t)n;
    }
    return IRC_OK;
}

// Write `bytes` of device memory src to f (appending at its position),
// through the pinned buffers.
int stream_from_device(FILE *f, const char *src, int64_t bytes, Pinned &pin, cudaStream_t s, const char *name)
{
    for (int64_t done = 0; done < bytes;) {
        const size_t n = (size_t)((bytes - done) < (int64_t)kStageBytes ? (bytes - done) : (int64_t)kStageBytes);
        cudaError_t e = cudaMemcpyAsync(pin.p[0], src + done, n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return irc_host::cuda_status(e, name);
        if (fwrite(pin.p[0], 1, n, f) != n) {
            irc_host::set_error("%s: write failed", name);
            return IRC_E_INVAL;
        }
        done += (int64_t)n;
    }
    return IRC_OK;
}

}  // namespace

extern "C" int irc_fet_load_site(float *F, int *nC_out, const char *const *files, int nLoads,
                                 const int64_t *vnSpkBefore, const int64_t *vnSpkSite, int nPc, int nSitesSpk,
                                 const uint8_t *mlPc, const int64_t *viSel, int64_t nOut, void *stream)
{
    const char *name = "irc_fet_load_site";
    cudaStream_t s = (cudaStream_t)stream;
    if (!F || !nC_out || !files || nLoads < 1 || !vnSpkBefore || !vnSpkSite || nPc < 1 || nSitesSpk < 1 || nOut < 0) {
        irc_host::set_error("%s: bad arguments", name);
        return IRC_E_INVAL;
    }
    const int recLen = nPc * nSitesSpk;
    const int64_t recBytes = (int64_t)recLen * 4;
    std::vector<int> pcIdx;
    for (int i = 0; i < recLen; ++i)
        if (!mlPc || mlPc[i]) pcIdx.push_back(i);
    const int nC = (int)pcIdx.size();
    *nC_out = nC;
    int64_t nRec = 0;
    for (int l = 0; l < nLoads; ++l) {
        if (vnSpkBefore[l] < 0 || vnSpkSite[l] < 0) {
            irc_host::set_error("%s: negative spike count in load %d", name, l);
            return IRC_E_INVAL;
        }
        nRec += vnSpkSite[l];
    }
    if (!viSel && nOut != nRec) {
        irc_host::set_error("%s: without viSel nOut must be the site's %lld records", name, (long long)nRec);
        return IRC_E_INVAL;
    }
    if (nOut == 0 || nC == 0) return IRC_OK;
    char *rec = nullptr;
    int *dev = nullptr;                                // [0] bad flag, [1..] pcIdx
    cudaError_t e = cudaMallocAsync((void **)&rec, (size_t)(nRec > 0 ? nRec : 1) * recBytes, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&dev, sizeof(int) * (size_t)(nC + 1), s);
    if (e != cudaSuccess) {
        if (rec) cudaFreeAsync(rec, s);
        return irc_host::cuda_status(e, name);
    }
    int rc = IRC_OK;
    {
        Pinned pin;
        e = pin.init(kStageBytes);
        if (e != cudaSuccess) rc = irc_host::cuda_status(e, name);
        int64_t at = 0;
        for (int l = 0; l < nLoads && rc == IRC_OK; ++l) {
            if (vnSpkSite[l] == 0) continue;
            FileCloser fc;
            fc.f = fopen(files[l], "rb");
            if (!fc.f) {
                irc_host::set_error("%s: cannot open %s", name, files[l]);
                rc = IRC_E_INVAL;
                break;
            }
            rc = stream_to_device(fc.f, vnSpkBefore[l] * recBytes, vnSpkSite[l] * recBytes, rec + at * recBytes,
                                  pin, s, name);
            at += vnSpkSite[l];
        }
        if (rc == IRC_OK) {
            const int zero = 0;
            e = cudaMemcpyAsync(dev, &zero, sizeof(int), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(dev + 1, pcIdx.data(), sizeof(int) * (size_t)nC, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) {
                const dim3 blk(32, 8);
                k_fet_gather<<<grid_for(nOut, 8), blk, 0, s>>>(F, (const float *)rec, recLen, viSel, nOut, dev + 1,
                                                              nC, nRec, dev);
                e = cudaGetLastError();
            }
            int bad = 0;
            if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, dev, sizeof(int), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);   // also keeps pcIdx / zero alive for the copies
            if (e != cudaSuccess) rc = irc_host::cuda_status(e, name);
            else if (bad) {
                irc_host::set_error("%s: a viSel entry is outside the site's %lld records", name, (long long)nRec);
                rc = IRC_E_INVAL;
            }
        }
    }                                                  // pinned buffers released after their copies
    cudaFreeAsync(rec, s);
    cudaFreeAsync(dev, s);
    return rc;
}

extern "C" int irc_knn_save_site(const char *path, int append, const int32_t *miKnn, int knnIn, int knnOut, int64_t n,
                                 const int64_t *viSpk, int64_t nF, void *stream)
{
    const char *name = "irc_knn_save_site";
    cudaStream_t s = (cudaStream_t)stream;
    if (!path || !miKnn || !viSpk || knnIn < 1 || knnOut < knnIn || n < 0 || nF < 1) {
        irc_host::set_error("%s: bad arguments (need 1 <= knnIn <= knnOut)", name);
        return IRC_E_INVAL;
    }
    FileCloser fc;
    fc.f = fopen(path, append ? "ab" : "wb");
    if (!fc.f) {
        irc_host::set_error("%s: cannot open %s", name, path);
        return IRC_E_INVAL;
    }
    if (n == 0) return IRC_OK;
    int64_t *out = nullptr;
    int *bad = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&out, sizeof(int64_t) * (size_t)(n * knnOut), s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&bad, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), s);
    if (e != cudaSuccess) {
        if (out) cudaFreeAsync(out, s);
        return irc_host::cuda_status(e, name);
    }
    k_knn_global<<<grid_for(n * knnOut, 256), 256, 0, s>>>(out, miKnn, knnIn, knnOut, n, viSpk, nF, bad);
    int rc = IRC_OK;
    int hbad = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = irc_host::cuda_status(e, name);
    else if (hbad) {
        irc_host::set_error("%s: a kNN position is outside 1..%lld", name, (long long)nF);
        rc = IRC_E_INVAL;
    } else {
        Pinned pin;
        e = pin.init(kStageBytes);
        rc = e != cudaSuccess ? irc_host::cuda_status(e, name)
                              : stream_from_device(fc.f, (const char *)out, (int64_t)sizeof(int64_t) * n * knnOut,
                                                   pin, s, name);
    }
    cudaFreeAsync(out, s);
    cudaFreeAsync(bad, s);
    return rc;
}

extern "C" int irc_sort_save(const char *path, const float *rho, const float *delta, const int64_t *nneigh,
                             const int64_t *ordrho, int64_t nSpk, void *stream)
{
    const char *name = "irc_sort_save";
    cudaStream_t s = (cudaStream_t)stream;
    if (!path || !rho || !delta || !nneigh || !ordrho || nSpk < 0) {
        irc_host::set_error("%s: bad arguments", name);
        return IRC_E_INVAL;
    }
    FileCloser fc;
    fc.f = fopen(path, "wb");
    if (!fc.f) {
        irc_host::set_error("%s: cannot open %s", name, path);
        return IRC_E_INVAL;
    }
    if (nSpk == 0) return IRC_OK;
    double *ord = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&ord, sizeof(double) * (size_t)nSpk, s);
    if (e != cudaSuccess) return irc_host::cuda_status(e, name);
    k_i64_to_f64<<<grid_for(nSpk, 256), 256, 0, s>>>(ord, ordrho, nSpk);
    int rc = IRC_OK;
    e = cudaGetLastError();
    if (e != cudaSuccess) rc = irc_host::cuda_status(e, name);
    {
        Pinned pin;
        if (rc == IRC_OK && (e = pin.init(kStageBytes)) != cudaSuccess) rc = irc_host::cuda_status(e, name);
        if (rc == IRC_OK) rc = stream_from_device(fc.f, (const char *)rho, 4 * nSpk, pin, s, name);
        if (rc == IRC_OK) rc = stream_from_device(fc.f, (const char *)delta, 4 * nSpk, pin, s, name);
        if (rc == IRC_OK) rc = stream_from_device(fc.f, (const char *)nneigh, 8 * nSpk, pin, s, name);
        if (rc == IRC_OK) rc = stream_from_device(fc.f, (const char *)ord, 8 * nSpk, pin, s, name);
    }
    cudaFreeAsync(ord, s);
    return rc;
}

extern "C" int irc_sort_load(const char *path, float *rho, float *delta, int64_t *nneigh, int64_t *ordrho,
                             int64_t nSpk, void *stream)
{
    const char *name = "irc_sort_load";
    cudaStream_t s = (cudaStream_t)stream;
    if (!path || !rho || !delta || !nneigh || !ordrho || nSpk < 0) {
        irc_host::set_error("%s: bad arguments", name);
        return IRC_E_INVAL;
    }
    FileCloser fc;
    fc.f = fopen(path, "rb");
    if (!fc.f) {
        irc_host::set_error("%s: cannot open %s", name, path);
        return IRC_E_INVAL;
    }
    if (nSpk == 0) return IRC_OK;
    double *ord = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&ord, sizeof(double) * (size_t)nSpk, s);
    if (e != cudaSuccess) return irc_host::cuda_status(e, name);
    int rc = IRC_OK;
    {
        Pinned pin;
        if ((e = pin.init(kStageBytes)) != cudaSuccess) rc = irc_host::cuda_status(e, name);
        if (rc == IRC_OK) rc = stream_to_device(fc.f, 0, 4 * nSpk, (char *)rho, pin, s, name);
        if (rc == IRC_OK) rc = stream_to_device(fc.f, 4 * nSpk, 4 * nSpk, (char *)delta, pin, s, name);
        if (rc == IRC_OK) rc = stream_to_device(fc.f, 8 * nSpk, 8 * nSpk, (char *)nneigh, pin, s, name);
        if (rc == IRC_OK) rc = stream_to_device(fc.f, 16 * nSpk, 8 * nSpk, (char *)ord, pin, s, name);
        if (rc == IRC_OK) {
            k_f64_to_i64<<<grid_for(nSpk, 256), 256, 0, s>>>(ordrho, ord, nSpk);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) rc = irc_host::cuda_status(e, name);
        }
    }
    cudaFreeAsync(ord, s);
    return rc;
}

namespace {
__global__ void k_f16_to_f32(float *__restrict__ out, const __half *__restrict__ in, int64_t n)
{
    const int64_t i0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * 4;
    if (i0 + 3 < n) {
        const __half2 a = *reinterpret_cast<const __half2 *>(in + i0);
        const __half2 b = *reinterpret_cast<const __half2 *>(in + i0 + 2);
        const float2 fa = __half22float2(a), fb = __half22float2(b);
        *reinterpret_cast<float4 *>(out + i0) = make_float4(fa.x, fa.y, fb.x, fb.y);
    } else {
        for (int64_t i = i0; i < n; ++i) out[i] = __half2float(in[i]);
    }
}
}  // namespace

extern "C" int irc_f16_to_f32(float *out, const void *in, int64_t n, void *stream)
{
    if (!out || !in || n < 0 || (reinterpret_cast<uintptr_t>(in) & 3) || (reinterpret_cast<uintptr_t>(out) & 15)) {
        irc_host::set_error("irc_f16_to_f32: null or misaligned pointer (in: 4-byte, out: 16-byte alignment)");
        return IRC_E_INVAL;
    }
    if (n == 0) return IRC_OK;
    const int64_t threads = (n + 3) / 4;
    k_f16_to_f32<<<(unsigned)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(out, (const __half *)in, n);
    IRC_CHECK_LAUNCH("irc_f16_to_f32");
    return IRC_OK;
}
