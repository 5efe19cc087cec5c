// irc_dc2.cu -- the distance cut-off of the time-drift clustering mode
// (vcCluster = 'drift'): calc_dc2_drift_ (matlab/irc.m:24582-24608) on the
// device.
//
// For every site, up to dc_subsample of the window's own spikes on that site
// (the first n1, primary features) are the queries, and up to 4 dc_subsample
// window spikes with that primary site (primary features) plus up to
// 4 dc_subsample with that secondary site (secondary features) the
// candidates, each list thinned by subsample_vr_ (matlab/irc.m:11322-11337).
// Per query, the squared distances to the candidates in eucl2_dist_'s
// expansion form (matlab/irc.m:2387-2392), sorted ascending: the cut is entry
// ceil(n2 * dc_percent / 100).  The site's dc2 is the median of its queries'
// cuts, the window's the nanmedian over sites (sites without queries are NaN).
//
// Arithmetic (restated; MATLAB's own BLAS product is closed): sum(Y.^2) and
// sum(X.^2) as rounded squares added in feature order, X'Y as fused
// multiply-adds in feature order, d = yy + (xx - 2 xy) in single precision.
// The median of an even count is a + (b - a) / 2 of the two middle values
// ((a + b) / 2 when their signs differ), as MATLAB's median computes it.
//
// Device work: one CTA per (site, query) computes its candidates' distances
// into shared memory and selects the cut by a radix search over
// order-preserving keys (NaN after +inf, as MATLAB's sort places it).
#include <algorithm>
#include <cmath>
#include <vector>

#include "irc_common.cuh"

namespace {

constexpr int kDc2Threads = 256;

__device__ __forceinline__ unsigned order_key(float v)
{
    const unsigned b = __float_as_uint(v);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ float key_value(unsigned k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Block q: query spike qidx[q] of site qsite[q]; candidates cidx[c_off[s] ..
// c_off[s] + n21[s] + n22[s]), the first n21[s] with primary features
// (mrFet1), the rest with secondary features (mrFet2); cut[s] (1-based).
__global__ void __launch_bounds__(kDc2Threads)
k_dc2_cut(const float *__restrict__ mrFet1, const float *__restrict__ mrFet2, int nC, const int32_t *__restrict__ qidx,
          const int32_t *__restrict__ qsite, const int32_t *__restrict__ c_off, const int32_t *__restrict__ n21,
          const int32_t *__restrict__ n22, const int32_t *__restrict__ cut, const int32_t *__restrict__ cidx,
          float *__restrict__ out)
{
    extern __shared__ float dyn_dc2[];
    __shared__ float sy[IRC_NC_MAX];
    __shared__ float s_yy;
    __shared__ unsigned s_cnt[kDc2Threads / 32];
    const int q = blockIdx.x, s = qsite[q];
    const float *y = mrFet1 + (size_t)qidx[q] * nC;
    for (int c = threadIdx.x; c < nC; c += blockDim.x) sy[c] = y[c];
    __syncthreads();
    if (threadIdx.x == 0) {
        float yy = 0.0f;
        for (int c = 0; c < nC; ++c) yy = __fadd_rn(yy, __fmul_rn(sy[c], sy[c]));
        s_yy = yy;
    }
    __syncthreads();
    const float yy = s_yy;
    const int a = n21[s], n2 = a + n22[s];
    const int32_t *ci = cidx + c_off[s];
    for (int j = threadIdx.x; j < n2; j += blockDim.x) {
        const float *x = (j < a ? mrFet1 : mrFet2) + (size_t)ci[j] * nC;
        float xx = 0.0f, xy = 0.0f;
        for (int c = 0; c < nC; ++c) {
            const float xc = __ldg(x + c);
            xx = __fadd_rn(xx, __fmul_rn(xc, xc));
            xy = __fmaf_rn(xc, sy[c], xy);
        }
        dyn_dc2[j] = __fadd_rn(yy, __fsub_rn(xx, __fmul_rn(2.0f, xy)));
    }
    __syncthreads();
    // the k-th smallest key: the largest t with fewer than k keys below it
    const unsigned k = (unsigned)cut[s];
    unsigned ans = 0u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b = 31; b >= 0; --b) {
        const unsigned t = ans | (1u << b);
        unsigned c = 0;
        for (int j = threadIdx.x; j < n2; j += blockDim.x) c += order_key(dyn_dc2[j]) < t;
        c = __reduce_add_sync(0xffffffffu, c);
        if (lane == 0) s_cnt[warp] = c;
        __syncthreads();
        unsigned tot = 0;
#pragma unroll
        for (int w = 0; w < kDc2Threads / 32; ++w) tot += s_cnt[w];
        __syncthreads();
        if (tot < k) ans = t;
    }
    if (threadIdx.x == 0) out[q] = key_value(ans);
}

// subsample_vr_ (matlab/irc.m:11322-11337): every nSkip-th entry, then the
// entries at round(linspace(1, n, nRemove)) removed (MATLAB's linspace:
// d1 + ((0:n1) * (d2 - d1)) / n1 with both ends set exactly).
std::vector<int32_t> subsample_vr(std::vector<int32_t> vi, int nMax)
{
    if ((int)vi.size() <= nMax) return vi;
    const int nSkip = (int)(vi.size() / (size_t)nMax);
    if (nSkip > 1) {
        std::vector<int32_t> t;
        for (size_t i = 0; i < vi.size(); i += (size_t)nSkip) t.push_back(vi[i]);
        vi.swap(t);
    }
    if ((int)vi.size() > nMax) {
        const int n = (int)vi.size(), nRemove = n - nMax;
        std::vector<char> rm(n, 0);
        const double d1 = 1.0, d2 = n, n1 = nRemove - 1;
        for (int i = 0; i < nRemove; ++i) {
            double y = (i == 0) ? d1 : (i == nRemove - 1) ? d2 : d1 + ((double)i * (d2 - d1)) / n1;
            if (nRemove == 1) y = d2;            // a one-point linspace is its end point
            long r = std::lround(y);             // round half away from zero, as MATLAB's round
            r = std::min<long>(std::max<long>(r, 1), n);
            rm[r - 1] = 1;
        }
        std::vector<int32_t> t;
        for (int i = 0; i < n; ++i)
            if (!rm[i]) t.push_back(vi[i]);
        vi.swap(t);
    }
    return vi;
}

// MATLAB's median of single values: NaN when any value is NaN or there are
// none, else the middle value, or a + (b - a) / 2 of the two middle ones
// ((a + b) / 2 when their signs differ or one is infinite).
float matlab_median(std::vector<float> v)
{
    if (v.empty()) return NAN;
    for (float x : v)
        if (std::isnan(x)) return NAN;
    std::sort(v.begin(), v.end());
    const size_t n = v.size();
    if (n & 1) return v[n / 2];
    const float a = v[n / 2 - 1], b = v[n / 2];
    if (std::signbit(a) != std::signbit(b) || std::isinf(a) || std::isinf(b)) return (a + b) / 2.0f;
    return a + (b - a) / 2.0f;
}

}  // namespace

extern "C" int irc_calc_dc2_drift(float *dc2, float *dc2_site, int n1, int n12, int nC, const int32_t *viSite1,
                                  const int32_t *viSite2, const float *mrFet1, const float *mrFet2, int nSites,
                                  int dc_subsample, double dc_percent, void *stream)
{
    const char *me = "irc_calc_dc2_drift";
    if (!dc2 || !viSite1 || !viSite2 || !mrFet1 || !mrFet2 || n1 <= 0 || n12 < n1 || nC <= 0 || nSites <= 0) {
        irc_host::set_error("%s: null pointer or bad sizes", me);
        return IRC_E_INVAL;
    }
    if (nC > IRC_NC_MAX) { irc_host::set_error("%s: nC=%d > %d", me, nC, IRC_NC_MAX); return IRC_E_NC; }
    if (dc_subsample <= 0 || !(dc_percent > 0.0) || dc_percent > 100.0) {
        irc_host::set_error("%s: dc_subsample must be positive and dc_percent in (0, 100]", me);
        return IRC_E_INVAL;
    }
    const int n1s = dc_subsample, n2s = 4 * dc_subsample;
    const size_t smem = (size_t)2 * n2s * sizeof(float);
    if (smem > 200 * 1024) {
        irc_host::set_error("%s: dc_subsample %d too large (at most %d)", me, dc_subsample, 200 * 1024 / 32);
        return IRC_E_INVAL;
    }
    // per-site query / candidate lists (0-based positions in the window)
    std::vector<int32_t> qidx, qsite, c_off(nSites), n21(nSites), n22(nSites), cut(nSites), cidx;
    std::vector<int> nq(nSites);
    for (int s = 0; s < nSites; ++s) {
        const int site = s + 1;
        std::vector<int32_t> v11, v21, v22;
        for (int i = 0; i < n12; ++i) {
            if (i < n1 && viSite1[i] == site) v11.push_back(i);
            if (viSite1[i] == site) v21.push_back(i);
            if (viSite2[i] == site) v22.push_back(i);
        }
        v11 = subsample_vr(v11, n1s);
        v21 = subsample_vr(v21, n2s);
        v22 = subsample_vr(v22, n2s);
        c_off[s] = (int32_t)cidx.size();
        n21[s] = (int32_t)v21.size();
        n22[s] = (int32_t)v22.size();
        cidx.insert(cidx.end(), v21.begin(), v21.end());
        cidx.insert(cidx.end(), v22.begin(), v22.end());
        const int n2 = n21[s] + n22[s];
        cut[s] = (int32_t)std::ceil((double)n2 * dc_percent / 100.0);
        nq[s] = n2 > 0 ? (int)v11.size() : 0;
        for (int k = 0; k < nq[s]; ++k) {
            qidx.push_back(v11[k]);
            qsite.push_back(s);
        }
    }
    const int nQ = (int)qidx.size();
    std::vector<float> cuts(nQ);
    if (nQ > 0) {
        cudaStream_t st = (cudaStream_t)stream;
        const size_t ni = 5 * (size_t)nSites + 2 * (size_t)nQ + cidx.size();
        int32_t *d = nullptr;
        cudaError_t e = cudaMalloc(&d, ni * 4 + (size_t)nQ * 4);
        if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_calc_dc2_drift: cudaMalloc");
        std::vector<int32_t> img;
        img.reserve(ni);
        auto put = [&](const std::vector<int32_t> &v) { img.insert(img.end(), v.begin(), v.end()); };
        put(qidx); put(qsite); put(c_off); put(n21); put(n22); put(cut); put(cidx);
        int32_t *p = d;
        const int32_t *dq = p; p += nQ;
        const int32_t *ds = p; p += nQ;
        const int32_t *dco = p; p += nSites;
        const int32_t *d21 = p; p += nSites;
        const int32_t *d22 = p; p += nSites;
        const int32_t *dcut = p; p += nSites;
        const int32_t *dci = p; p += cidx.size();
        float *dout = reinterpret_cast<float *>(p);
        e = cudaMemcpyAsync(d, img.data(), img.size() * 4, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_dc2_cut, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(n2s * 4 * 2));
        if (e == cudaSuccess) {
            int mx = 0;
            for (int s = 0; s < nSites; ++s) mx = std::max(mx, n21[s] + n22[s]);
            k_dc2_cut<<<nQ, kDc2Threads, (size_t)mx * 4, st>>>(mrFet1, mrFet2, nC, dq, ds, dco, d21, d22, dcut, dci,
                                                             dout);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(cuts.data(), dout, (size_t)nQ * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaFree(d);
        if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_calc_dc2_drift");
    }
    // median per site, nanmedian over sites
    std::vector<float> site_dc2;
    for (int s = 0, k = 0; s < nSites; ++s) {
        std::vector<float> v(cuts.begin() + k, cuts.begin() + k + nq[s]);
        k += nq[s];
        const float m = matlab_median(v);
        if (dc2_site) dc2_site[s] = m;
        if (!std::isnan(m)) site_dc2.push_back(m);
    }
    *dc2 = matlab_median(site_dc2);
    return IRC_OK;
}
