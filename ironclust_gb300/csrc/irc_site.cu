// irc_site.cu -- fused per-site path, REF mode, and plan management.
//
// The MATLAB host launches search_min_drift once per drift chunk, gathers the
// [nT x nA] per-bin minima to the host and sorts every column there
// (matlab/irc2.m:3764-3788); search_delta_drift is handled the same way with
// a column `min` (:3829-3858).  Here one launch covers every chunk of a site:
// a CTA owns a tile of up to QB queries of one chunk, evaluates every bin of
// the chunk into shared memory, and performs the MATLAB sort/min on the
// device with warp arg-min reductions over (value, bin) keys -- the stable
// ascending order of MATLAB's sort.  Results equal the reference kernels +
// MATLAB post-processing bit for bit.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "irc_common.cuh"
#include "irc_plan.cuh"
#include "irc_scan.cuh"
#include "irc_tc.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kKnnQB = 16;     // queries per CTA, kNN kernel (bin table 16 x nT in smem)
constexpr int kDeltaQB = 16;   // queries per CTA, delta kernel

// kNN (search_min_drift + sort): bin table sV/sI [QB][nT] in dynamic smem.
__global__ void __launch_bounds__(kThreads)
k_site_knn_ref(irc::PlanDev p, const float *__restrict__ F, int nC, int nT, int knn,
               float *__restrict__ vrKnn, float *__restrict__ rho, int *__restrict__ miKnn)
{
    constexpr int QB = kKnnQB;
    __shared__ __align__(16) float sA[IRC_NC_MAX * QB];
    extern __shared__ __align__(16) unsigned char dyn[];
    float *sV = reinterpret_cast<float *>(dyn);            // [QB][nT]  sqrt(|bin min|)
    int *sI = reinterpret_cast<int *>(sV + QB * nT);       // [QB][nT]  1-based index
    int chunk, qs, n;
    irc::tile_lookup<QB>(p, blockIdx.x, chunk, qs, n);
    const int r0 = __ldg(p.roffr + chunk), nBB = __ldg(p.roffr + chunk + 1) - r0;
    irc::stage_queries<QB>(F, nC, qs, n, sA);
    __syncthreads();
    const int nT0 = nT / nBB;
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
        const int b = t % nBB;
        const int ib0 = __ldg(p.rsr + r0 + b), nb0 = __ldg(p.rnr + r0 + b);
        float mn[QB];
        int mi[QB];
#pragma unroll
        for (int q = 0; q < QB; ++q) { mn[q] = IRC_SINGLE_INF_F; mi[q] = qs + min(q, n - 1); }
        irc::scan_bin<QB, false>(F, nullptr, nC, ib0 + t / nBB, ib0 + nb0, nT0, sA, nullptr, mn, mi);
#pragma unroll
        for (int q = 0; q < QB; ++q) { sV[q * nT + t] = irc::ref_sqrt_abs(mn[q]); sI[q * nT + t] = mi[q] + 1; }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const float kTaken = -1.0f;
    for (int q = warp; q < n; q += nw) {
        float *v = sV + q * nT;
        const int *ix = sI + q * nT;
        const size_t o = (size_t)(qs + q - p.q_base);
        float last = 0.0f;
        for (int k = 0; k < knn; ++k) {
            unsigned long long best = ~0ull;
            for (int t = lane; t < nT; t += 32) {
                const float x = v[t];
                const unsigned long long key = (x == kTaken) ? ~0ull : irc::sort_key(x, t);
                best = key < best ? key : best;
            }
            best = irc::warp_min_u64(best);
            const int t = (int)(best & 0xffffffffu);
            last = v[t];
            __syncwarp();
            if (lane == 0) {
                miKnn[(size_t)k + (size_t)knn * o] = ix[t];
                v[t] = kTaken;
            }
            __syncwarp();
        }
        if (lane == 0) {
            vrKnn[o] = last;
            if (rho) rho[o] = __fdiv_rn(1.0f, last);
        }
    }
}

// delta (search_delta_drift + min): thread-local arg-min over its bins, then a
// block reduction of (value, bin) keys per query.
__global__ void __launch_bounds__(kThreads)
k_site_delta_ref(irc::PlanDev p, const float *__restrict__ F, const float *__restrict__ R, int nC,
                 int nT, float *__restrict__ delta, int *__restrict__ nneigh)
{
    constexpr int QB = kDeltaQB;
    __shared__ __align__(16) float sA[IRC_NC_MAX * QB];
    __shared__ float sRA[QB];
    __shared__ unsigned long long sKey[QB][kThreads / 32];
    __shared__ int sIdx[QB][kThreads / 32];
    int chunk, qs, n;
    irc::tile_lookup<QB>(p, blockIdx.x, chunk, qs, n);
    const int r0 = __ldg(p.roffr + chunk), nBB = __ldg(p.roffr + chunk + 1) - r0;
    irc::stage_queries<QB>(F, nC, qs, n, sA);
    if (threadIdx.x < QB) sRA[threadIdx.x] = __ldg(R + qs + min((int)threadIdx.x, n - 1));
    __syncthreads();
    const int nT0 = nT / nBB;
    unsigned long long bk[QB];
    int bi[QB];
#pragma unroll
    for (int q = 0; q < QB; ++q) { bk[q] = ~0ull; bi[q] = 0; }
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
        const int b = t % nBB;
        const int ib0 = __ldg(p.rsr + r0 + b), nb0 = __ldg(p.rnr + r0 + b);
        float mn[QB];
        int mi[QB];
#pragma unroll
        for (int q = 0; q < QB; ++q) { mn[q] = IRC_SINGLE_INF_F; mi[q] = qs + min(q, n - 1); }
        irc::scan_bin<QB, true>(F, R, nC, ib0 + t / nBB, ib0 + nb0, nT0, sA, sRA, mn, mi);
#pragma unroll
        for (int q = 0; q < QB; ++q) {
            const unsigned long long key = irc::sort_key(irc::ref_sqrt_abs(mn[q]), t);
            if (key < bk[q]) { bk[q] = key; bi[q] = mi[q]; }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < QB; ++q) {
        unsigned long long k = bk[q];
        int idx = bi[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ok = __shfl_xor_sync(0xffffffffu, k, o);
            const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
            if (ok < k) { k = ok; idx = oi; }
        }
        if (lane == 0) { sKey[q][warp] = k; sIdx[q][warp] = idx; }
    }
    __syncthreads();
    if (threadIdx.x < n) {
        const int q = threadIdx.x;
        unsigned long long k = sKey[q][0];
        int idx = sIdx[q][0];
        for (int w = 1; w < kThreads / 32; ++w)
            if (sKey[q][w] < k) { k = sKey[q][w]; idx = sIdx[q][w]; }
        const float v = __uint_as_float((unsigned)(k >> 32));
        const size_t o = (size_t)(qs + q - p.q_base);
        delta[o] = __fmul_rn(v, sRA[q]);
        nneigh[o] = idx + 1;
    }
}

inline int tiles_for(const irc_plan *pl, int qb) { return pl->ntiles[irc::tile_slot(qb)]; }

struct Slot {
    int chunk, qs, nq, nt;
};

// Work items of the tensor-core kNN (see irc_tc.cu).  Cost of an item: the
// largest candidate-tile count among its slots (its slots run side by side).
// Layout: chunks with more than 64 queries (more than 0 with max_slots == 1)
// are cut into 128-row single-slot items; the remainders are packed two
// (64-row slots) or four (32-row slots) per item, at most max_slots, slots of
// similar tile counts together.  order 0: items by cost, largest first, the
// items of one chunk adjacent (they stream the same candidate tiles and share
// them in L2); order 1: chunk order.
std::vector<irc::TcItem> build_tc_items(const int32_t *q0, const int32_t *nq, const int32_t *roff,
                                        const int32_t *rn, int nChunks, int max_slots, int order_mode,
                                        int *n_one, int *n_wide)
{
    std::vector<irc::TcItem> items;
    std::vector<int> cost;
    std::vector<Slot> s2, s1;
    auto push = [&](int nslot, const Slot *sl, int n) {
        irc::TcItem it;
        memset(&it, 0, sizeof(it));
        it.nslot = nslot;
        int c = 0;
        for (int s = 0; s < 4; ++s) {
            it.chunk[s] = s < n ? sl[s].chunk : -1;
            it.qs[s] = s < n ? sl[s].qs : 0;
            it.nq[s] = s < n ? sl[s].nq : 0;
            if (s < n) c = std::max(c, sl[s].nt);
        }
        items.push_back(it);
        cost.push_back(c);
    };
    const int big = max_slots == 1 ? 0 : 64;         // remainders up to this many rows are packed
    for (int i = 0; i < nChunks; ++i) {
        int nt = 0;
        for (int r = roff[i]; r < roff[i + 1]; ++r) nt += (rn[r] + 127) / 128;
        int q = q0[i], R = nq[i];
        while (R > big) {
            const Slot s{i, q, std::min(128, R), nt};
            push(1, &s, 1);
            q += s.nq;
            R -= s.nq;
        }
        if (R > 32 || (R > 0 && max_slots == 2)) s2.push_back(Slot{i, q, R, nt});
        else if (R > 0) s1.push_back(Slot{i, q, R, nt});
    }
    auto by_nt = [](const Slot &a, const Slot &b) { return a.nt > b.nt || (a.nt == b.nt && a.chunk < b.chunk); };
    std::sort(s2.begin(), s2.end(), by_nt);
    std::sort(s1.begin(), s1.end(), by_nt);
    for (size_t k = 0; k < s2.size(); k += 2) push(2, &s2[k], (int)std::min<size_t>(2, s2.size() - k));
    for (size_t k = 0; k < s1.size(); k += 4) push(4, &s1[k], (int)std::min<size_t>(4, s1.size() - k));
    std::vector<int> order(items.size());
    for (size_t k = 0; k < order.size(); ++k) order[k] = (int)k;
    if (order_mode == 0)
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            if (cost[a] != cost[b]) return cost[a] > cost[b];
            return items[a].chunk[0] < items[b].chunk[0];
        });
    else
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return items[a].chunk[0] < items[b].chunk[0]; });
    // one persistent launch per packing class: one-slot items, then two-slot
    // items (both on 256-candidate units, two 256-column accumulators), then
    // four-slot items (128-candidate units, one accumulator per slot), each
    // class in the order chosen above
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return items[a].nslot < items[b].nslot; });
    std::vector<irc::TcItem> out;
    out.reserve(items.size());
    int n1 = 0, nw = 0;
    for (int k : order) {
        out.push_back(items[k]);
        n1 += items[k].nslot == 1;
        nw += items[k].nslot <= 2;
    }
    *n_one = n1;
    *n_wide = nw;
    return out;
}

// Adjacent runs of a chunk merged into candidate intervals (same candidate set).
void merge_runs(const int32_t *roff, const int32_t *rs, const int32_t *rn, int nChunks, std::vector<int32_t> &moff,
                std::vector<int32_t> &ms, std::vector<int32_t> &mn)
{
    moff.assign(1, 0);
    ms.clear();
    mn.clear();
    for (int i = 0; i < nChunks; ++i) {
        for (int r = roff[i]; r < roff[i + 1]; ++r) {
            if ((int)ms.size() > moff.back() && ms.back() + mn.back() == rs[r]) mn.back() += rn[r];
            else { ms.push_back(rs[r]); mn.push_back(rn[r]); }
        }
        moff.push_back((int32_t)ms.size());
    }
}

}  // namespace

// Tensor-core operand rows (two [nF x row_bytes] matrices) followed by the
// re-rank's FP32 rows padded to 16-byte multiples ([nF x fp_row_bytes]) and
// extra_bytes of working space (256-byte aligned);
// allocated on the first tensor-core call of a plan, grown when a call
// needs more, kept until irc_plan_destroy.
int irc_plan_tc_buffers(irc_plan *pl, void **fq, void **fc, void **fp, void **extra, size_t row_bytes,
                        size_t fp_row_bytes, size_t extra_bytes)
{
    const size_t one = (size_t)pl->dev.nF * row_bytes;
    const size_t fpb = ((size_t)pl->dev.nF * fp_row_bytes + 255) & ~(size_t)255;
    const size_t need = 2 * one + fpb + extra_bytes;
    if (pl->tc_external) {
        if (pl->tc_bytes < need) {
            irc_host::set_error("irc_site_knn: the shared operand buffer holds %zu bytes, %zu needed",
                                pl->tc_bytes, need);
            return IRC_E_INVAL;
        }
        pl->tc_row_bytes = row_bytes;
    } else if (!pl->tc_buf || pl->tc_bytes < need || pl->tc_row_bytes != row_bytes) {
        if (pl->tc_buf) cudaFree(pl->tc_buf);
        pl->tc_buf = nullptr;
        pl->tc_bytes = 0;
        cudaError_t e = cudaMalloc(&pl->tc_buf, need);
        if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn: operand buffers");
        pl->tc_row_bytes = row_bytes;
        pl->tc_bytes = need;
    }
    *fq = pl->tc_buf;
    *fc = (char *)pl->tc_buf + one;
    *fp = (char *)pl->tc_buf + 2 * one;
    *extra = (char *)pl->tc_buf + 2 * one + fpb;
    return IRC_OK;
}

namespace {

// [nT x nA] search_min_drift output holding the exact kNN in rows 0..knn-1
// (ascending) and the no-candidate sentinel in the others, so the unchanged
// MATLAB post-processing (stable sort, first knn rows) returns the exact kNN.
__global__ void k_expand_exact(float *__restrict__ D, int *__restrict__ I, const int *__restrict__ miKnn,
                               const float *__restrict__ d2Knn, int nA, int nT, int knn, int iA0)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)nA * nT) return;
    const int a = (int)(i / nT), t = (int)(i % nT);
    if (t < knn) {
        D[i] = irc::ref_sqrt_abs(d2Knn[(size_t)a * knn + t]);
        I[i] = miKnn[(size_t)a * knn + t];
    } else {
        D[i] = irc::ref_sqrt_abs(IRC_SINGLE_INF_F);
        I[i] = iA0 + a + 1;
    }
}

}  // namespace

// IRC_MODE_EXACT of the search_min_drift drop-in: a one-chunk plan through the
// EXACT site kernel, then the expansion above.  The drop-in receives IBB/NBB
// on the device, so they are read back first; the plan and the temporaries
// are created and released per call (stream-ordered allocation).
int irc_exact_chunk_fill(float *D, int32_t *I, const float *F, const int32_t *IBB, const int32_t *NBB, int nC,
                         int nBB, int iA0, int nA, int nT, int knn, int nF, cudaStream_t s)
{
    std::vector<int32_t> rs(nBB), rn(nBB);
    cudaError_t e = cudaMemcpyAsync(rs.data(), IBB, 4 * (size_t)nBB, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rn.data(), NBB, 4 * (size_t)nBB, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_search_min_drift(EXACT): read IBB/NBB");
    const int32_t q0[1] = {iA0}, nq[1] = {nA}, roff[2] = {0, nBB};
    irc_plan *pl = nullptr;
    int rc = irc_plan_create(&pl, q0, nq, roff, rs.data(), rn.data(), 1, iA0, nA, nF);
    if (rc != IRC_OK) return rc;
    float *vr = nullptr, *d2 = nullptr;
    int32_t *mi = nullptr;
    e = cudaMallocAsync(&vr, sizeof(float) * (size_t)nA, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&d2, sizeof(float) * (size_t)nA * knn, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&mi, sizeof(int32_t) * (size_t)nA * knn, s);
    if (e == cudaSuccess) {
        rc = irc_site_knn(pl, F, nC, knn, nT, IRC_MODE_EXACT, vr, nullptr, mi, d2, s);
        if (rc == IRC_OK) {
            const size_t n = (size_t)nA * nT;
            k_expand_exact<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(D, I, mi, d2, nA, nT, knn, iA0);
            e = cudaGetLastError();
            if (e != cudaSuccess) rc = irc_host::cuda_status(e, "irc_search_min_drift(EXACT): expand");
        }
    } else {
        rc = irc_host::cuda_status(e, "irc_search_min_drift(EXACT): temporaries");
    }
    if (vr) cudaFreeAsync(vr, s);
    if (d2) cudaFreeAsync(d2, s);
    if (mi) cudaFreeAsync(mi, s);
    cudaStreamSynchronize(s);                    // the plan's image is released with the call
    irc_plan_destroy(pl);
    return rc;
}

// Exact / tensor-core site kernels (irc_exact.cu, irc_tc.cu).
int irc_site_knn_exact(irc_plan *plan, const float *F, int nC, int knn, float *vrKnn, float *rho,
                       int32_t *miKnn, float *d2Knn, cudaStream_t s);
int irc_site_knn_tc(irc_plan *plan, const float *F, int nC, int knn, int mode, float *vrKnn,
                    float *rho, int32_t *miKnn, float *d2Knn, cudaStream_t s);
int irc_site_delta_list(irc_plan *plan, const float *F, int nC, const float *R, int knn,
                        const int32_t *miKnn, const float *d2Knn, float *delta, int32_t *nneigh,
                        cudaStream_t s);

// Rows of F a plan reads (its queries and candidate runs) as merged [lo, hi)
// intervals; more than 8 collapse to their hull.  Operand preparation runs
// over these rows only (a streaming ring holds rows no plan of the moment
// reads).
static void row_intervals(const int32_t *q0, const int32_t *nq, const int32_t *rs, const int32_t *rn, int nChunks,
                          int nRuns, irc_plan *pl)
{
    std::vector<std::pair<int, int>> iv;
    iv.reserve((size_t)nChunks + nRuns);
    for (int i = 0; i < nChunks; ++i) iv.emplace_back(q0[i], q0[i] + nq[i]);
    for (int r = 0; r < nRuns; ++r) iv.emplace_back(rs[r], rs[r] + rn[r]);
    std::sort(iv.begin(), iv.end());
    std::vector<std::pair<int, int>> m;
    for (const auto &x : iv) {
        if (!m.empty() && x.first <= m.back().second) m.back().second = std::max(m.back().second, x.second);
        else m.push_back(x);
    }
    if (m.size() > 8) m.assign(1, std::make_pair(m.front().first, m.back().second));
    pl->n_row_iv = (int)m.size();
    for (size_t k = 0; k < m.size(); ++k) {
        pl->row_iv[2 * k] = m[k].first;
        pl->row_iv[2 * k + 1] = m[k].second;
    }
}

extern "C" {

int irc_plan_create(irc_plan **out, const int32_t *q0, const int32_t *nq, const int32_t *roff,
                    const int32_t *rs, const int32_t *rn, int nChunks, int q_base, int n_out, int nF)
{
    if (!out) {
        irc_host::set_error("irc_plan_create: null pointer or empty plan");
        return IRC_E_INVAL;
    }
    *out = nullptr;
    long long pairs = 0;
    int max_nq = 0;
    const int vrc = irc_host::check_plan("irc_plan_create", q0, nq, roff, rs, rn, nChunks, q_base, n_out, nF,
                                         &pairs, &max_nq);
    if (vrc != IRC_OK) return vrc;
    const int nRuns = roff[nChunks];
    irc_plan *pl = (irc_plan *)calloc(1, sizeof(irc_plan));
    if (!pl) return IRC_E_NOMEM;
    // host copies
    const size_t nCh = (size_t)nChunks;
    pl->h_q0 = (int32_t *)malloc(4 * nCh);
    pl->h_nq = (int32_t *)malloc(4 * nCh);
    pl->h_roff = (int32_t *)malloc(4 * (nCh + 1));
    pl->h_rs = (int32_t *)malloc(4 * (size_t)nRuns);
    pl->h_rn = (int32_t *)malloc(4 * (size_t)nRuns);
    memcpy(pl->h_q0, q0, 4 * nCh);
    memcpy(pl->h_nq, nq, 4 * nCh);
    memcpy(pl->h_roff, roff, 4 * (nCh + 1));
    memcpy(pl->h_rs, rs, 4 * (size_t)nRuns);
    memcpy(pl->h_rn, rn, 4 * (size_t)nRuns);
    // device image: q0 | nq | roff | rs | rn | tile_off x 5
    std::vector<int32_t> img;
    img.reserve(4 * nCh + 2 * nRuns + irc::kNumTileSizes * (nCh + 1) + 8);
    size_t off_q0 = img.size(); img.insert(img.end(), q0, q0 + nCh);
    size_t off_nq = img.size(); img.insert(img.end(), nq, nq + nCh);
    // candidate intervals: adjacent runs of a chunk merged (same candidate set)
    std::vector<int32_t> moff, ms, mn;
    merge_runs(roff, rs, rn, nChunks, moff, ms, mn);
    size_t off_roff = img.size(); img.insert(img.end(), moff.begin(), moff.end());
    size_t off_rs = img.size(); img.insert(img.end(), ms.begin(), ms.end());
    size_t off_rn = img.size(); img.insert(img.end(), mn.begin(), mn.end());
    size_t off_roffr = img.size(); img.insert(img.end(), roff, roff + nCh + 1);
    size_t off_rsr = img.size(); img.insert(img.end(), rs, rs + nRuns);
    size_t off_rnr = img.size(); img.insert(img.end(), rn, rn + nRuns);
    size_t off_ncand = img.size();
    for (int i = 0; i < nChunks; ++i) {
        int32_t c = 0;
        for (int r = roff[i]; r < roff[i + 1]; ++r) c += rn[r];
        img.push_back(c);
    }
    // tensor-core tiles: every chunk's intervals cut into 128-row tiles,
    // each chunk's list padded to an even length
    const size_t off_toff = img.size();
    std::vector<int32_t> tiles;
    for (int i = 0; i < nChunks; ++i) {
        img.push_back((int32_t)(tiles.size() / 2));
        for (int r = moff[i]; r < moff[i + 1]; ++r)
            for (int t = 0; t < mn[r]; t += 128) {
                tiles.push_back(ms[r] + t);
                tiles.push_back(std::min(128, mn[r] - t));
            }
        if ((tiles.size() / 2) & 1) { tiles.push_back(0); tiles.push_back(0); }
    }
    img.push_back((int32_t)(tiles.size() / 2));
    while (img.size() % 4) img.push_back(0);          // 16-byte aligned
    const size_t off_tiles = img.size();
    img.insert(img.end(), tiles.begin(), tiles.end());
    size_t off_tile[irc::kNumTileSizes];
    for (int k = 0; k < irc::kNumTileSizes; ++k) {
        const int qb = irc::kTileSizes[k];
        off_tile[k] = img.size();
        int acc = 0;
        img.push_back(0);
        for (int i = 0; i < nChunks; ++i) { acc += (nq[i] + qb - 1) / qb; img.push_back(acc); }
        pl->ntiles[k] = acc;
    }
    // tensor-core work items: 128-row tiles of large chunks, then the 33-64 and
    // 1-32 row remainders packed two and four per item (similar tile counts
    // together), all ordered by cost, largest first
    int n_one = 0, n_wide = 0;
    std::vector<irc::TcItem> items = build_tc_items(q0, nq, moff.data(), mn.data(), nChunks, 4, 0, &n_one, &n_wide);
    while (img.size() % 16) img.push_back(0);
    const size_t off_items = img.size();
    for (const irc::TcItem &it : items) {
        const int32_t *w = reinterpret_cast<const int32_t *>(&it);
        img.insert(img.end(), w, w + 16);
    }
    cudaGetDevice(&pl->device);
    if (img.size() & 1) img.push_back(0);          // scratch starts 8-byte aligned (int2 items)
    // 4 words, two query lists of n_out, and the (chunk, tile) items of the
    // delta fallback: at most n_out/16 + nChunks pairs
    // counters, two query lists, the delta fallback's (tile, part) units (up to 8 parts per
    // 16-query tile) and its per-query 64-bit best keys (8-byte aligned: every term before
    // them is even)
    const size_t scratch_ints = irc::kScratchLists + 2 * (size_t)n_out +
                                16 * ((size_t)n_out / 16 + nChunks + 1) + 2 * (size_t)n_out;
    cudaError_t e = cudaMalloc(&pl->dmem, (img.size() + scratch_ints) * sizeof(int32_t));
    if (e != cudaSuccess) {
        free(pl->h_q0); free(pl->h_nq); free(pl->h_roff); free(pl->h_rs); free(pl->h_rn); free(pl);
        irc_host::cuda_status(e, "irc_plan_create: cudaMalloc");
        return IRC_E_NOMEM;
    }
    e = cudaMemcpy(pl->dmem, img.data(), img.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cudaFree(pl->dmem); free(pl); return irc_host::cuda_status(e, "irc_plan_create: upload"); }
    const int32_t *base = (const int32_t *)pl->dmem;
    pl->dev.q0 = base + off_q0;
    pl->dev.nq = base + off_nq;
    pl->dev.roff = base + off_roff;
    pl->dev.rs = base + off_rs;
    pl->dev.rn = base + off_rn;
    pl->dev.roffr = base + off_roffr;
    pl->dev.rsr = base + off_rsr;
    pl->dev.rnr = base + off_rnr;
    pl->dev.ncand = base + off_ncand;
    pl->dev.tc_toff = base + off_toff;
    pl->dev.tc_tiles = reinterpret_cast<const int2 *>(base + off_tiles);
    for (int k = 0; k < irc::kNumTileSizes; ++k) pl->dev.tile_off[k] = base + off_tile[k];
    pl->scratch = (int32_t *)pl->dmem + img.size();
    pl->tc_items = reinterpret_cast<const irc::TcItem *>((const int32_t *)pl->dmem + off_items);
    pl->n_tc_items = (int)items.size();
    pl->n_tc_one = n_one;
    pl->n_tc_wide = n_wide;
    e = cudaMemset(pl->scratch, 0, irc::kScratchLists * sizeof(int32_t));      // counters and error word
    if (e != cudaSuccess) { cudaFree(pl->dmem); free(pl); return irc_host::cuda_status(e, "irc_plan_create: clear"); }
    pl->dev.nChunks = nChunks;
    pl->dev.q_base = q_base;
    pl->dev.n_out = n_out;
    pl->dev.nF = nF;
    pl->dev.nRuns = (int)ms.size();
    pl->max_nq = max_nq;
    pl->pairs = pairs;
    row_intervals(q0, nq, rs, rn, nChunks, nRuns, pl);
    *out = pl;
    return IRC_OK;
}

int irc_plan_destroy(irc_plan *pl)
{
    if (!pl) return IRC_OK;
    cudaError_t e = cudaFree(pl->dmem);
    if (pl->tc_buf && !pl->tc_external) cudaFree(pl->tc_buf);
    if (pl->tc_items_buf) cudaFree(pl->tc_items_buf);
    if (pl->row_dims) cudaFree(pl->row_dims);
    free(pl->h_q0); free(pl->h_nq); free(pl->h_roff); free(pl->h_rs); free(pl->h_rn);
    free(pl);
    return e == cudaSuccess ? IRC_OK : irc_host::cuda_status(e, "irc_plan_destroy");
}

size_t irc_plan_tc_bytes(const irc_plan *pl, int nC)
{
    if (!pl || nC < 1) return 0;
    const size_t one = (size_t)pl->dev.nF * 128;
    const size_t fpb = ((size_t)pl->dev.nF * (size_t)irc_tc::fp_row4(nC) * 16 + 255) & ~(size_t)255;
    return 2 * one + fpb + (size_t)256 * 64 * 4 + 256 + irc_tc::list_area_bytes(pl->dev.n_out);
}

int irc_plan_set_tc_buffer(irc_plan *pl, void *buf, size_t bytes)
{
    if (!pl || !buf) {
        irc_host::set_error("irc_plan_set_tc_buffer: null plan or buffer");
        return IRC_E_INVAL;
    }
    if (pl->tc_buf && !pl->tc_external) cudaFree(pl->tc_buf);
    pl->tc_buf = buf;
    pl->tc_bytes = bytes;
    pl->tc_row_bytes = 0;
    pl->tc_external = 1;
    return IRC_OK;
}

int irc_plan_tc_layout(irc_plan *pl, int max_slots, int order)
{
    if (!pl || (max_slots != 1 && max_slots != 2 && max_slots != 4) || (order != 0 && order != 1)) {
        irc_host::set_error("irc_plan_tc_layout: need a plan, max_slots in {1, 2, 4} and order in {0, 1}");
        return IRC_E_INVAL;
    }
    const int nChunks = pl->dev.nChunks;
    std::vector<int32_t> moff, ms, mn;
    merge_runs(pl->h_roff, pl->h_rs, pl->h_rn, nChunks, moff, ms, mn);
    int n_one = 0, n_wide = 0;
    std::vector<irc::TcItem> items = build_tc_items(pl->h_q0, pl->h_nq, moff.data(), mn.data(), nChunks, max_slots,
                                                    order, &n_one, &n_wide);
    void *buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, sizeof(irc::TcItem) * (items.size() ? items.size() : 1));
    if (e == cudaSuccess)
        e = cudaMemcpy(buf, items.data(), sizeof(irc::TcItem) * items.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        if (buf) cudaFree(buf);
        return irc_host::cuda_status(e, "irc_plan_tc_layout");
    }
    if (pl->tc_items_buf) cudaFree(pl->tc_items_buf);   // synchronises the device: no launch still reads it
    pl->tc_items_buf = buf;
    pl->tc_items = reinterpret_cast<const irc::TcItem *>(buf);
    pl->n_tc_items = (int)items.size();
    pl->n_tc_one = n_one;
    pl->n_tc_wide = n_wide;
    return IRC_OK;
}

int irc_plan_set_site_dims(irc_plan *pl, int nSites, const int64_t *row_base, const int32_t *dims)
{
    if (!pl) { irc_host::set_error("irc_plan_set_site_dims: null plan"); return IRC_E_INVAL; }
    if (nSites == 0) {                            // clear
        if (pl->row_dims) cudaFree(pl->row_dims);
        pl->row_dims = nullptr;
        return IRC_OK;
    }
    const int nF = pl->dev.nF;
    if (nSites < 0 || !row_base || !dims || row_base[0] != 0 || row_base[nSites] != nF) {
        irc_host::set_error("irc_plan_set_site_dims: need row_base[0] = 0 and row_base[nSites] = nF (%d)", nF);
        return IRC_E_INVAL;
    }
    for (int k = 0; k < nSites; ++k)
        if (row_base[k + 1] < row_base[k] || dims[k] < 1 || dims[k] > IRC_NC_MAX) {
            irc_host::set_error("irc_plan_set_site_dims: site %d: bad rows or dims", k);
            return IRC_E_INVAL;
        }
    // every chunk's queries and candidate runs lie in one site (the site of
    // its first query): the site's width then bounds every distance it needs
    auto site_of = [&](long long r) {
        return (int)(std::upper_bound(row_base, row_base + nSites + 1, (int64_t)r) - row_base) - 1;
    };
    for (int i = 0; i < pl->dev.nChunks; ++i) {
        if (pl->h_nq[i] <= 0) continue;
        const int st = site_of(pl->h_q0[i]);
        bool ok = site_of((long long)pl->h_q0[i] + pl->h_nq[i] - 1) == st;
        for (int r = pl->h_roff[i]; ok && r < pl->h_roff[i + 1]; ++r)
            ok = pl->h_rn[r] <= 0 || (site_of(pl->h_rs[r]) == st && site_of((long long)pl->h_rs[r] + pl->h_rn[r] - 1) == st);
        if (!ok) {
            irc_host::set_error("irc_plan_set_site_dims: chunk %d reaches outside the site of its queries", i);
            return IRC_E_INVAL;
        }
    }
    std::vector<uint8_t> h((size_t)nF);
    for (int k = 0; k < nSites; ++k)
        for (long long r = row_base[k]; r < row_base[k + 1]; ++r) h[(size_t)r] = (uint8_t)dims[k];
    if (!pl->row_dims) {
        cudaError_t e = cudaMalloc(&pl->row_dims, h.size() ? h.size() : 1);
        if (e != cudaSuccess) { pl->row_dims = nullptr; return irc_host::cuda_status(e, "irc_plan_set_site_dims"); }
    }
    cudaError_t e = cudaMemcpy(pl->row_dims, h.data(), h.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_plan_set_site_dims: upload");
    return IRC_OK;
}

int irc_plan_tc_units(irc_plan *pl, int width)
{
    if (!pl || (width != 128 && width != 256)) {
        irc_host::set_error("irc_plan_tc_units: need a plan and a width of 128 or 256");
        return IRC_E_INVAL;
    }
    pl->tc_wide_bn = width;
    return IRC_OK;
}

int irc_plan_check(irc_plan *pl, void *stream)
{
    if (!pl) { irc_host::set_error("irc_plan_check: null plan"); return IRC_E_INVAL; }
    int word = 0;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(&word, pl->scratch + irc::kScratchErr, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_plan_check");
    if (word) {
        cudaMemsetAsync(pl->scratch + irc::kScratchErr, 0, sizeof(int), s);
        irc_host::set_error("a device-side wait of the plan's kernels timed out");
        return IRC_E_TIMEOUT;
    }
    return IRC_OK;
}

int irc_site_knn(irc_plan *pl, const float *F, int nC, int knn, int nThreads, int mode,
                 float *vrKnn, float *rho, int32_t *miKnn, float *d2Knn, void *stream)
{
    if (!pl || !F || !vrKnn || !miKnn) { irc_host::set_error("irc_site_knn: null pointer"); return IRC_E_INVAL; }
    if (nC > IRC_NC_MAX) { irc_host::set_error("irc_site_knn: nC=%d > %d", nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0 || knn <= 0) { irc_host::set_error("irc_site_knn: bad nC/knn"); return IRC_E_INVAL; }
    cudaStream_t s = (cudaStream_t)stream;
    if (mode == IRC_MODE_REF) {
        if (nThreads <= 0 || nThreads > 1024 || knn > nThreads) {
            irc_host::set_error("irc_site_knn: bad nThreads=%d / knn=%d", nThreads, knn);
            return IRC_E_INVAL;
        }
        for (int i = 0; i < pl->dev.nChunks; ++i)
            if (pl->h_roff[i + 1] - pl->h_roff[i] > nThreads) {
                irc_host::set_error("irc_site_knn: chunk %d has more runs than bins", i);
                return IRC_E_INVAL;
            }
        const size_t smem = (size_t)kKnnQB * nThreads * 8;
        cudaError_t e = cudaFuncSetAttribute(k_site_knn_ref, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_site_knn: smem attribute");
        k_site_knn_ref<<<tiles_for(pl, kKnnQB), kThreads, smem, s>>>(pl->dev, F, nC, nThreads, knn, vrKnn, rho, miKnn);
        IRC_CHECK_LAUNCH("irc_site_knn(REF)");
        return IRC_OK;
    }
    if (mode == IRC_MODE_EXACT) return irc_site_knn_exact(pl, F, nC, knn, vrKnn, rho, miKnn, d2Knn, s);
    if (mode == IRC_MODE_BF16 || mode == IRC_MODE_FP8)
        return irc_site_knn_tc(pl, F, nC, knn, mode, vrKnn, rho, miKnn, d2Knn, s);
    irc_host::set_error("irc_site_knn: unknown mode %d", mode);
    return IRC_E_INVAL;
}

int irc_site_delta(irc_plan *pl, const float *F, int nC, const float *R, int nThreads, int mode,
                   int knn, const int32_t *miKnn, const float *d2Knn, float *delta, int32_t *nneigh,
                   void *stream)
{
    if (!pl || !F || !R || !delta || !nneigh) { irc_host::set_error("irc_site_delta: null pointer"); return IRC_E_INVAL; }
    if (nC > IRC_NC_MAX) { irc_host::set_error("irc_site_delta: nC=%d > %d", nC, IRC_NC_MAX); return IRC_E_NC; }
    if (nC <= 0) { irc_host::set_error("irc_site_delta: bad nC"); return IRC_E_INVAL; }
    cudaStream_t s = (cudaStream_t)stream;
    if (mode == IRC_MODE_REF) {
        if (nThreads <= 0 || nThreads > 1024) { irc_host::set_error("irc_site_delta: bad nThreads"); return IRC_E_INVAL; }
        for (int i = 0; i < pl->dev.nChunks; ++i)
            if (pl->h_roff[i + 1] - pl->h_roff[i] > nThreads) {
                irc_host::set_error("irc_site_delta: chunk %d has more runs than bins", i);
                return IRC_E_INVAL;
            }
        k_site_delta_ref<<<tiles_for(pl, kDeltaQB), kThreads, 0, s>>>(pl->dev, F, R, nC, nThreads, delta, nneigh);
        IRC_CHECK_LAUNCH("irc_site_delta(REF)");
        return IRC_OK;
    }
    if (mode == IRC_MODE_EXACT || mode == IRC_MODE_BF16 || mode == IRC_MODE_FP8) {
        if (!miKnn || !d2Knn || knn <= 0) { irc_host::set_error("irc_site_delta: kNN list required"); return IRC_E_INVAL; }
        return irc_site_delta_list(pl, F, nC, R, knn, miKnn, d2Knn, delta, nneigh, s);
    }
    irc_host::set_error("irc_site_delta: unknown mode %d", mode);
    return IRC_E_INVAL;
}

// kNN, rho and delta of a plan in one call: irc_site_knn with the 1024 bins
// of search_knn_drift_ and irc_site_delta with the 512 of
// search_delta_drift_ (the counts MATLAB sets, matlab/irc2.m:3755, :3819;
// only the REF mode depends on them), stream-ordered.  R = rho of every
// column of F; NULL uses the rho computed here, which needs a plan whose
// queries are all of F.
int irc_knn_rho_delta_site(irc_plan *pl, const float *F, int nC, const float *R, int knn, int mode,
                           float *vrKnn, float *rho, int32_t *miKnn, float *d2Knn, float *delta, int32_t *nneigh,
                           void *stream)
{
    if (!pl || !rho) { irc_host::set_error("irc_knn_rho_delta_site: null plan or rho"); return IRC_E_INVAL; }
    if (!R && (pl->dev.q_base != 0 || pl->dev.n_out != pl->dev.nF)) {
        irc_host::set_error("irc_knn_rho_delta_site: R is required when the plan's queries are not all of F "
                            "(q_base %d, n_out %d, nF %d)", pl->dev.q_base, pl->dev.n_out, pl->dev.nF);
        return IRC_E_INVAL;
    }
    int rc = irc_site_knn(pl, F, nC, knn, 1024, mode, vrKnn, rho, miKnn, d2Knn, stream);
    if (rc != IRC_OK) return rc;
    return irc_site_delta(pl, F, nC, R ? R : rho, 512, mode, knn, miKnn, d2Knn, delta, nneigh, stream);
}

// One plan for a batch of sites stacked row-wise (site s at rows
// row_base[s] .. row_base[s+1]-1 of one feature matrix): the sites' plans
// (site-local rows) are concatenated with their rows offset, q_base 0 and
// every row a query.  Per-site arrays are given back to back: q0/nq hold
// nChunks[s] entries per site, roff nChunks[s]+1 (site-local, from 0), rs/rn
// roff_s[nChunks[s]] entries.  Candidate runs must stay inside their site.
int irc_batch_plan_create(irc_plan **out, int nSites, const int32_t *nChunks, const int64_t *row_base,
                          const int32_t *q0, const int32_t *nq, const int32_t *roff, const int32_t *rs,
                          const int32_t *rn)
{
    if (!out || nSites <= 0 || !nChunks || !row_base || !q0 || !nq || !roff || !rs || !rn) {
        irc_host::set_error("irc_batch_plan_create: null pointer or no site");
        return IRC_E_INVAL;
    }
    *out = nullptr;
    if (row_base[0] != 0 || row_base[nSites] > INT32_MAX) {
        irc_host::set_error("irc_batch_plan_create: row_base must start at 0 and end below 2^31");
        return IRC_E_INVAL;
    }
    std::vector<int32_t> Q0, NQ, ROFF(1, 0), RS, RN;
    size_t c0 = 0, f0 = 0, r0 = 0;
    for (int st = 0; st < nSites; ++st) {
        const int64_t base = row_base[st], n = row_base[st + 1] - row_base[st];
        const int nc = nChunks[st];
        if (n < 0 || nc < 0) { irc_host::set_error("irc_batch_plan_create: site %d: bad sizes", st); return IRC_E_INVAL; }
        const int32_t *ro = roff + f0;
        if (ro[0] != 0) { irc_host::set_error("irc_batch_plan_create: site %d: roff must start at 0", st); return IRC_E_INVAL; }
        for (int i = 0; i < nc; ++i) {
            const int32_t a = q0[c0 + i], m = nq[c0 + i];
            if (a < 0 || m <= 0 || a + (int64_t)m > n || ro[i + 1] < ro[i]) {
                irc_host::set_error("irc_batch_plan_create: site %d chunk %d out of range", st, i);
                return IRC_E_INVAL;
            }
            Q0.push_back((int32_t)(a + base));
            NQ.push_back(m);
            for (int r = ro[i]; r < ro[i + 1]; ++r) {
                const int32_t b = rs[r0 + r], k = rn[r0 + r];
                if (b < 0 || k <= 0 || b + (int64_t)k > n) {
                    irc_host::set_error("irc_batch_plan_create: site %d run %d leaves its site", st, r);
                    return IRC_E_INVAL;
                }
                RS.push_back((int32_t)(b + base));
                RN.push_back(k);
            }
            ROFF.push_back((int32_t)RS.size());
        }
        c0 += nc;
        f0 += nc + 1;
        r0 += ro[nc];
    }
    const int nRows = (int)row_base[nSites];
    return irc_plan_create(out, Q0.data(), NQ.data(), ROFF.data(), RS.data(), RN.data(), (int)Q0.size(), 0, nRows,
                           nRows);
}

// Site feature matrices (device, site s [n_s x nC_s] row-major) stacked into
// one [row_base[nSites] x nCmax] matrix zero-padded to nCmax columns: a
// padded feature adds exactly 0 to every fused accumulate, so results on the
// stack equal the per-site results bit for bit.  F_sites is a host array of
// device pointers.
int irc_batch_stack(float *F, int nCmax, const float *const *F_sites, const int32_t *nC_sites, const int64_t *row_base,
                    int nSites, void *stream)
{
    if (!F || !F_sites || !nC_sites || !row_base || nSites <= 0 || nCmax <= 0) {
        irc_host::set_error("irc_batch_stack: null pointer or empty batch");
        return IRC_E_INVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const size_t pitch = (size_t)nCmax * sizeof(float);
    for (int st = 0; st < nSites; ++st) {
        const int64_t n = row_base[st + 1] - row_base[st];
        const int nc = nC_sites[st];
        if (n < 0 || nc < 0 || nc > nCmax || (n > 0 && nc > 0 && !F_sites[st])) {
            irc_host::set_error("irc_batch_stack: site %d: bad size or pointer", st);
            return IRC_E_INVAL;
        }
        if (n == 0) continue;
        float *dst = F + (size_t)row_base[st] * nCmax;
        cudaError_t e = cudaSuccess;
        if (nc > 0)
            e = cudaMemcpy2DAsync(dst, pitch, F_sites[st], (size_t)nc * sizeof(float), (size_t)nc * sizeof(float),
                                  (size_t)n, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess && nc < nCmax)
            e = cudaMemset2DAsync(dst + nc, pitch, 0, (size_t)(nCmax - nc) * sizeof(float), (size_t)n, s);
        if (e != cudaSuccess) return irc_host::cuda_status(e, "irc_batch_stack");
    }
    return IRC_OK;
}

}  // extern "C"

