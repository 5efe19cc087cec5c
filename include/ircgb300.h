/*
 * ircgb300.h -- C ABI of the GB300 (sm_103a) IronClust clustering hot path.
 *
 * The library replaces the CUDA kernels IronClust's MATLAB host launches
 * through parallel.gpu.CUDAKernel + feval on the clustering path (the drift
 * kNN / rho / delta kernels and their irc.m variants), keeping their
 * argument order, array shapes and outputs; adds fused per-site entry points
 * that run a whole site (every drift chunk) per call; and runs the
 * clustering step that consumes their outputs (sort_'s normalisation,
 * postCluster_'s cluster assignment).
 *
 * Conventions (identical to the reference):
 *   - feature matrices are MATLAB column-major [nC x n] float32, i.e. the nC
 *     features of one spike are contiguous;
 *   - 2-D outputs are column-major ([nT x nA] means element (t, a) at
 *     t + nT*a);
 *   - returned spike indices are 1-based;
 *   - SINGLE_INF = (float)3.402E+38 marks "no candidate".
 * All array arguments are DEVICE pointers unless a comment says "host".
 * vnConst arrays are read on the host (MATLAB builds them on the host before
 * uploading them as gpuArrays; the MEX gateway passes the host copy).
 * `stream` is a cudaStream_t (NULL = legacy default stream).  Every call is
 * asynchronous with respect to the host and returns IRC_OK or a negative
 * IRC_E* status; irc_last_error() describes the last failure of the calling
 * thread.  Kernels never trap: a failed call leaves the context usable.
 */
#ifndef IRCGB300_H
#define IRCGB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define IRC_OK 0
#define IRC_E_INVAL (-1)   /* bad pointer, size or argument combination   */
#define IRC_E_NC (-2)      /* feature count above the kernel's maximum      */
#define IRC_E_CUDA (-3)    /* a CUDA runtime call or launch failed          */
#define IRC_E_NOMEM (-4)   /* device allocation failed                      */
#define IRC_E_TIMEOUT (-5) /* a bounded device-side wait gave up            */
#define IRC_E_UNSUPPORTED (-6) /* mode not available on this device        */

/* precision / search modes of the kNN entry points */
#define IRC_MODE_REF 0   /* bit-exact with the reference binned-minimum kernels */
#define IRC_MODE_EXACT 1 /* true top-k, reference FP32 arithmetic, (d2, index) ties */
#define IRC_MODE_BF16 2  /* tcgen05 BF16 distance filter + exact FP32 re-rank   */
#define IRC_MODE_FP8 3   /* tcgen05 FP8-e4m3 filter (plan-wide scale) + re-rank */

int irc_version(void);                 /* 10000*major + 100*minor + patch */
const char *irc_last_error(void);      /* message of the calling thread's last failure */
const char *irc_status_string(int status);

/* ---------------------------------------------------------------------------
 * Drop-in kernels (one call == one MATLAB feval of the reference kernel).
 * Output arrays are fully written (the reference relies on pre-zeroed
 * outputs only for entries it does not write; these write every entry).
 * ------------------------------------------------------------------------ */

/* Replaces search_min_drift (matlab/search_min_drift.cu:24; launched from
 * matlab/irc2.m:3793).  vnConst (host) = {nC, nF, nBB, iA0, nA}.
 * D, I: [nThreads x nA].  IBB/NBB: [nBB] 0-based run starts / run lengths.
 * mode IRC_MODE_REF: per-thread-bin minima exactly as the reference.
 * mode IRC_MODE_EXACT: rows 0..knn-1 hold the true k nearest (distance > 0)
 * in ascending (distance, index) order, the remaining rows hold
 * sqrt(SINGLE_INF) and the query's own index, so the unchanged MATLAB
 * post-processing (sort, first knn rows) returns the exact kNN. */
int irc_search_min_drift(float *D, int32_t *I, const float *F, const int32_t *IBB,
                         const int32_t *NBB, const int32_t *vnConst, int nThreads,
                         int mode, int knn, void *stream);

/* Replaces search_delta_drift (matlab/search_delta_drift.cu:24; launched
 * from matlab/irc2.m:3846).  R: [nF] rho.  D, I: [nThreads x nA]. */
int irc_search_delta_drift(float *D, int32_t *I, const float *F, const float *R,
                           const int32_t *IBB, const int32_t *NBB, const int32_t *vnConst,
                           int nThreads, void *stream);

/* Replaces cuda_knn_index (matlab/cuda_knn_index.cu:27; launched from
 * matlab/irc.m:24389).  vnConst (host) = {nB, nA, nC, knn}.  B: [nC x nB],
 * A: [nC x nA].  K: [nA], I: [knn x nA].  nThreads = the reference block
 * size (512). */
int irc_cuda_knn_index(float *K, int32_t *I, const float *B, const float *A,
                       const int32_t *vnConst, int nThreads, void *stream);

/* Replaces cuda_delta_knn (matlab/cuda_delta_knn.cu:19; launched from
 * matlab/irc.m:24541).  vnConst (host) = {nB, nA, nC}.  D: [nA], N: [nA]
 * (1-based into B; falls back to the query's own A-space index, as the
 * reference does).  nThreads = the reference block size (128). */
int irc_cuda_delta_knn(float *D, uint32_t *N, const float *B, const float *A,
                       const float *R_B, const float *R_A, const int32_t *vnConst,
                       int nThreads, void *stream);

/* Replaces jrc3_cuda_rho_drift (matlab/irc_cuda_rho_drift.cu:28; launched
 * from matlab/irc.m:24635).  vnConst (host) = {n1, n12, nC}.  miSite12:
 * [n12 x 2] int32 (primary, secondary site), mrFet1/mrFet2: [nC x n12].
 * vrRho1: [n1]. */
int irc_rho_drift(float *vrRho1, const int32_t *miSite12, const float *mrFet1,
                  const float *mrFet2, const int32_t *vnConst, float dc2, void *stream);

/* Replaces jrc3_cuda_delta_drift (matlab/irc_cuda_delta_drift.cu:28; launched
 * from matlab/irc.m:24663).  vnConst (host) = {n1, n12, nC}; vrRho1: [n12].
 * vrDelta1 [n1] = sqrt(min d2 / dc2) over site-matched candidates with
 * strictly higher rho; viNneigh1 [n1] 1-based (the query itself when none). */
int irc_delta_drift(float *vrDelta1, uint32_t *viNneigh1, const int32_t *miSite12, const float *mrFet1,
                    const float *mrFet2, const float *vrRho1, const int32_t *vnConst, float dc2,
                    void *stream);

/* The distance cut-off of the time-drift clustering mode, calc_dc2_drift_
 * (matlab/irc.m:24582-24608; cluster_drift_ computes it on its first drift
 * window, :24095-24097, and passes it to every irc_rho_drift /
 * irc_delta_drift call).  A window of n12 spikes, the own chunk's n1 first:
 * viSite1 / viSite2 (HOST, [n12], 1-based primary / secondary sites, 0 =
 * none), mrFet1 / mrFet2 (device, [nC x n12], primary / secondary features).
 * Per site s = 1..nSites: up to dc_subsample own spikes on s (queries) and up
 * to 4*dc_subsample window spikes with primary site s plus 4*dc_subsample with
 * secondary site s (candidates), thinned by subsample_vr_; each query's
 * squared distances (eucl2_dist_'s expansion form) sorted, entry
 * ceil(n2 * dc_percent / 100) kept; the site's value is their median.  dc2
 * (HOST) = the median over sites with queries (nanmedian); dc2_site (HOST,
 * [nSites], may be NULL) = the per-site values, NaN for a site without
 * queries.  dc_subsample <= 6400.  Synchronises the stream. */
int irc_calc_dc2_drift(float *dc2, float *dc2_site, int n1, int n12, int nC, const int32_t *viSite1,
                       const int32_t *viSite2, const float *mrFet1, const float *mrFet2, int nSites, int dc_subsample,
                       double dc_percent, void *stream);

/* The binned-minimum kNN variants of cuda_knn_index (same scan and selection
 * sort, so results depend on nThreads the same way).  vnConst (host) =
 * {nB, nA, nC, knn}; B: [nC x nB], A: [nC x nA]; knn <= nThreads.
 *
 * Replaces cuda_knn (matlab/cuda_knn.cu:24; launched from matlab/irc.m:24456
 * with nThreads = 2 * P.nThreads = 256): K [nA] = the knn-th distance. */
int irc_cuda_knn(float *K, const float *B, const float *A, const int32_t *vnConst, int nThreads,
                 void *stream);

/* Replaces cuda_knn_full (matlab/cuda_knn_full.cu:27; no call site in the
 * reference's MATLAB code; its block size is 512): K [knn x nA] = every
 * sorted distance, I [knn x nA] 1-based (1 for a bin that saw no candidate). */
int irc_cuda_knn_full(float *K, int32_t *I, const float *B, const float *A, const int32_t *vnConst,
                      int nThreads, void *stream);

/* Replaces cuda_knn_ib (matlab/cuda_knn_ib.cu:27; no call site; block size
 * 512): candidates are the B columns IB[0..nB-1] (1-based; B has nF
 * columns), K [nA], I [knn x nA] = 1-based B columns.  IB entries outside
 * 1..nF, which the reference would read out of bounds, are skipped and
 * reported as IRC_E_INVAL (the call synchronises the stream to check). */
int irc_cuda_knn_ib(float *K, int32_t *I, const float *B, const float *A, const int32_t *IB, int nF,
                    const int32_t *vnConst, int nThreads, void *stream);

/* Replaces jrc3_cuda_rho (matlab/irc_cuda_rho.cu:24; launched from
 * matlab/irc.m:2551, the time-window "spacetime" clustering mode).
 * vnConst (host) = {n1, n12, nC, dn_max, fDc_spk}; mrFet12 [nC x n12] with
 * the n1 queries first; viiSpk12_ord [n12] time order.  vrRho1 [n1] =
 * (candidates within |ord_i - ord_j| <= dn_max at d2 <= dc2) / (candidates
 * within the window); fDc_spk = 1 uses d2 < dc2 * |query|^2 instead.
 * fDc_spk must be 0 or 1 (the reference leaves its cut-off uninitialised
 * otherwise). */
int irc_cuda_rho(float *vrRho1, const float *mrFet12, const int32_t *viiSpk12_ord, const int32_t *vnConst,
                 float dc2, void *stream);

/* Replaces jrc3_cuda_delta (matlab/irc_cuda_delta.cu:26; irc.m's cuda_delta_,
 * matlab/irc.m:2651-2676, names it 'iron_cuda_delta', a file the reference
 * does not ship, so there it always falls back to the CPU).  vnConst as
 * irc_cuda_rho; viiRho12_ord [n12] = rank in descending rho.  vrDelta1 [n1]
 * = sqrt(min d2 / dc2) over window candidates ranked before the query (cut
 * dc2 * |query|^2 with fDc_spk = 1); viNneigh1 [n1] 1-based into the window
 * (the query itself when none).  nThreads = the reference block size
 * (P.nThreads, 128): ties go to the lowest of nThreads bins; a multiple of
 * 32 up to 128. */
int irc_cuda_delta(float *vrDelta1, uint32_t *viNneigh1, const float *mrFet12, const int32_t *viiSpk12_ord,
                   const int32_t *viiRho12_ord, const int32_t *vnConst, float dc2, int nThreads, void *stream);

/* ---------------------------------------------------------------------------
 * Fused per-site path.  A plan describes every launch the MATLAB chunk loop
 * of search_knn_drift_ / search_delta_drift_ (matlab/irc2.m:3764-3788,
 * :3829-3864) would make for one site: query chunk i covers queries
 * [q0[i], q0[i]+nq[i]) of the site feature matrix (0-based) and candidate
 * runs rs[roff[i] .. roff[i+1]-1] / rn[...] (the IBB/NBB of that launch).
 * Outputs are indexed by q - q_base (n_out entries).  Plan arrays are host
 * pointers; the plan keeps device copies until irc_plan_destroy.
 * ------------------------------------------------------------------------ */
typedef struct irc_plan irc_plan;

int irc_plan_create(irc_plan **out, const int32_t *q0, const int32_t *nq, const int32_t *roff,
                    const int32_t *rs, const int32_t *rn, int nChunks, int q_base, int n_out,
                    int nF);
int irc_plan_destroy(irc_plan *plan);

/* Synchronises `stream` and reports IRC_E_TIMEOUT if a bounded device-side
 * wait in one of the plan's kernels gave up since the last check (the
 * kernel then returned early and its outputs are incomplete); clears the
 * flag.  No reference counterpart: the reference kernels have no waits. */
int irc_plan_check(irc_plan *plan, void *stream);

/* Layout of the plan's tensor-core work items (IRC_MODE_BF16 / FP8): chunks
 * with more than 64 queries run as 128-query CTAs; the remaining queries of
 * each chunk are packed up to max_slots chunks per CTA (1, 2 or 4; default
 * 4); order 0 = costliest first with a chunk's CTAs adjacent (default),
 * 1 = chunk order.  Results do not depend on the layout, only speed does
 * (ironclust_gb300.autotune picks it by timing).  Synchronises the device;
 * call it outside stream capture.  No reference counterpart. */
int irc_plan_tc_layout(irc_plan *plan, int max_slots, int order);

/* Candidate-unit width of the plan's one- and two-slot tensor-core work items
 * (IRC_MODE_BF16 / FP8): 256 (default: one N = 256 MMA per K slice, two
 * 256-column accumulators, the threshold folded into the MMA for BF16) or 128
 * (N = 128, four 128-column accumulators, the threshold compared in the
 * epilogue).  Four-slot items always use 128.  Results do not depend on it,
 * only speed does (ironclust_gb300.autotune picks it with the layout).  No
 * reference counterpart. */
int irc_plan_tc_units(irc_plan *plan, int width);

/* Site widths of a plan over stacked sites (host arrays): rows
 * row_base[k] .. row_base[k+1]-1 of F belong to site k, whose features past
 * dims[k] are zero in every row (as irc_batch_stack writes them); row_base
 * spans the plan's nF rows, and every chunk's queries and candidates must lie
 * in one site (checked).  The tensor-core re-rank and the delta fallback
 * scan then skip each query's zero features: same results, less work.
 * nSites = 0 clears it.  No reference counterpart. */
int irc_plan_set_site_dims(irc_plan *plan, int nSites, const int64_t *row_base, const int32_t *dims);

/* Working memory of the tensor-core modes: bytes a plan needs for nC
 * features (operand rows of all nF columns + their padded FP32 copy).  By
 * default a plan allocates it on its first tensor-core call and keeps it;
 * irc_plan_set_tc_buffer hands it caller-owned device memory of `bytes`
 * instead, which several plans can share when their calls are serialised on
 * one stream (the plans of consecutive pages, for instance).  No reference
 * counterpart. */
size_t irc_plan_tc_bytes(const irc_plan *plan, int nC);
int irc_plan_set_tc_buffer(irc_plan *plan, void *buf, size_t bytes);

/* Poll limit of the tensor-core filter's pipeline waits on the current
 * device: polls > 0 sets it, polls <= 0 restores the default (2^22 polls,
 * a few seconds).  A poll is a suspending try_wait; below 64 polls every poll
 * is a non-blocking test instead.  A wait that runs out makes its CTA stop,
 * let its own copies and MMAs land, free its TMEM and set the plan's error
 * word, which irc_plan_check reports as IRC_E_TIMEOUT; a small limit
 * exercises that path.  Applies to later calls; not during stream capture.
 * No reference counterpart (the reference kernels have no waits). */
int irc_set_wait_limit(int polls);

/* Kernel timing of the tensor-core modes.  Between irc_profile_begin and
 * irc_profile_end every tensor-core irc_site_knn call (up to max_calls)
 * records CUDA events on its stream around its filter kernel and around its
 * re-rank kernel; irc_profile_end waits for them and returns the summed
 * milliseconds of each and the number of calls timed.  Host-side bookkeeping
 * only; no reference counterpart. */
int irc_profile_begin(int max_calls);
int irc_profile_end(float *filter_ms, float *rerank_ms, int *calls);

/* kNN + rho of every query of the plan (rho_paged_site_ up to the global-id
 * mapping, matlab/irc2.m:3645-3670).
 * vrKnn [n_out]: distance of the knn-th neighbour; rho [n_out] (optional) =
 * 1 ./ vrKnn; miKnn [knn x n_out]: 1-based indices into F; d2Knn
 * [knn x n_out] (optional, not in REF mode): squared distances.
 * REF mode = search_min_drift with nThreads bins + MATLAB sort, bit-exact. */
int irc_site_knn(irc_plan *plan, const float *F, int nC, int knn, int nThreads, int mode,
                 float *vrKnn, float *rho, int32_t *miKnn, float *d2Knn, void *stream);

/* delta + nearest higher-rho neighbour of every query of the plan
 * (delta_paged_site_ up to the global-id mapping, matlab/irc2.m:3697-3720).
 * R: [nF] rho of every column of F.  Outputs delta [n_out] =
 * (distance to the nearest higher-rho spike) .* R(query), nneigh [n_out]
 * (1-based into F).
 * REF mode = search_delta_drift with nThreads bins + MATLAB min, bit-exact.
 * Other modes need miKnn/d2Knn of irc_site_knn (same plan and mode): delta
 * comes from the kNN list when it holds a higher-rho spike, else from a full
 * drift-window scan; ties are broken by (distance, index). */
int irc_site_delta(irc_plan *plan, const float *F, int nC, const float *R, int nThreads,
                   int mode, int knn, const int32_t *miKnn, const float *d2Knn,
                   float *delta, int32_t *nneigh, void *stream);

/* kNN, rho and delta of a plan in one stream-ordered call (the fused entry
 * of the new host path; replaces the search_knn_drift_ -> rho_paged_site_ ->
 * search_delta_drift_ -> delta_paged_site_ sequence of one page,
 * matlab/irc2.m:3635-3726, up to the global-id mapping): irc_site_knn with
 * 1024 bins, then irc_site_delta with 512 (the counts MATLAB sets).  R = rho
 * of every column of F, or NULL to use the rho computed here (then the
 * plan's queries must be all of F: q_base 0, n_out = nF).  d2Knn is needed
 * in every mode but IRC_MODE_REF.  A batch plan (below) runs a whole probe in
 * one call. */
int irc_knn_rho_delta_site(irc_plan *plan, const float *F, int nC, const float *R, int knn, int mode,
                           float *vrKnn, float *rho, int32_t *miKnn, float *d2Knn, float *delta, int32_t *nneigh,
                           void *stream);

/* Batches: the sites of a probe (processed one by one in the reference's
 * parfor, matlab/irc2.m:3539-3561) as one plan over one feature matrix.
 * irc_batch_plan_create concatenates per-site plans (site-local rows; per
 * site, nChunks[s] entries of q0/nq, nChunks[s]+1 of roff starting at 0,
 * roff_s[nChunks[s]] of rs/rn, back to back) with site s at rows
 * row_base[s] .. row_base[s+1]-1 (row_base[0] = 0, nSites+1 entries); every
 * row is a query.  irc_batch_stack copies the sites' device feature matrices
 * (F_sites: host array of device pointers, site s [n_s x nC_s]) into one
 * [row_base[nSites] x nCmax] matrix, zero-padded: a padded feature adds
 * exactly 0 to every distance, so batch results equal per-site results bit
 * for bit.  No reference counterpart. */
int irc_batch_plan_create(irc_plan **out, int nSites, const int32_t *nChunks, const int64_t *row_base,
                          const int32_t *q0, const int32_t *nq, const int32_t *roff, const int32_t *rs,
                          const int32_t *rn);
int irc_batch_stack(float *F, int nCmax, const float *const *F_sites, const int32_t *nC_sites,
                    const int64_t *row_base, int nSites, void *stream);

/* irc_site_knn in IRC_MODE_EXACT for callers that cannot allocate device
 * memory -- hosts whose device memory is reserved up front by their own pool
 * (a MATLAB gpuArray workspace, a real-time acquisition loop that must not
 * hit the device-wide synchronisation of cudaMalloc/cudaFree), or code
 * running where allocation is not allowed.  No counterpart in the reference.
 * It takes the plan arrays as HOST pointers (same meaning as
 * irc_plan_create) plus the inputs and outputs of irc_site_knn, and calls no
 * cudaMalloc/cudaFree or other allocating routine: the device copy of the
 * plan, its tile table and the overflow queue live in one fixed 8 MiB array
 * inside the library, held by every GPU that loads it until the process
 * exits.  The plan must fit that array: 4 + 2*n_out + 4*nChunks + 2 +
 * 2*nRuns int32 words <= 2^21 (about a million queries); larger plans are
 * rejected with IRC_E_INVAL and a message, as are plans irc_plan_create
 * rejects.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current and keeps it; make that
 * first call before any stream capture, and do not call the entry point on a
 * device after cudaDeviceReset (the kept address is then stale).  Every call
 * shares the array and overwrites it, so calls that overlap on the GPU (two
 * streams, two host threads) race: serialise them on one stream.  Outputs
 * equal those of irc_site_knn(IRC_MODE_EXACT) bit for bit. */
int irc_site_knn_exact_noalloc(const float *F, int nC, const int32_t *q0, const int32_t *nq,
                               const int32_t *roff, const int32_t *rs, const int32_t *rn, int nChunks,
                               int q_base, int n_out, int nF, int knn, float *vrKnn, float *rho,
                               int32_t *miKnn, float *d2Knn, void *stream);

/* ---------------------------------------------------------------------------
 * Clustering after the path: the consumers of rho, delta, nneigh and kNN.
 * ------------------------------------------------------------------------ */

/* ---------------------------------------------------------------------------
 * On-disk formats on either side of the path (raw little-endian arrays, as
 * MATLAB's fwrite writes them).  Paths are host strings.
 * ------------------------------------------------------------------------ */

/* load_fet_site_ (matlab/irc2.m:4039-4135) into device memory.  files
 * [nLoads]: the per-load feature files (_fet_<load>.irc, or _fet2_ for the
 * secondary-site features), each holding, site after site, that site's
 * spikes as [nPc x nSitesSpk] single records (save_paged_fet_site_,
 * matlab/irc2.m:4612-4618).  vnSpkBefore[l] / vnSpkSite[l] (host): records
 * of the sites before this one / of this site in load l.  The site's records
 * of all loads, concatenated in load order, are the "site records"; viSel
 * [nOut] (DEVICE, 0-based into them; NULL = all of them in order, then nOut
 * must equal their count) picks the output spikes.  mlPc [nPc x nSitesSpk]
 * (host, column-major 0/1 bytes; NULL = all) selects the features, in
 * MATLAB's linear order.  F [nC x nOut] (device, column-major) receives
 * them; nC_out (host) = the number of selected features.  File reads are
 * staged through pinned buffers and overlap the copies to the device.
 * Synchronises the stream. */
int irc_fet_load_site(float *F, int *nC_out, const char *const *files, int nLoads, const int64_t *vnSpkBefore,
                      const int64_t *vnSpkSite, int nPc, int nSitesSpk, const uint8_t *mlPc, const int64_t *viSel,
                      int64_t nOut, void *stream);

/* The kNN file of rho_paged_site_ / save_miKnn_site_ (matlab/irc2.m:3670-3679,
 * :3355-3370): miKnn [knnIn x n] (device, 1-based positions into the site
 * feature matrix, as irc_site_knn returns them), viSpk [nF] (device, int64
 * global spike ids of the feature-matrix columns) -> int64 [knnOut x n]
 * global ids, rows padded to knnOut by repeating the last, written to path
 * (append != 0: appended, as for every page after the first).  Synchronises
 * the stream. */
int irc_knn_save_site(const char *path, int append, const int32_t *miKnn, int knnIn, int knnOut, int64_t n,
                      const int64_t *viSpk, int64_t nF, void *stream);

/* The sort result file of sort_cache_ / struct_save_bin_ (matlab/irc2.m:356-391,
 * :1733-1750): rho, delta (single), nneigh (int64), ordrho (written as
 * double, as MATLAB's sort returns it) concatenated; device arrays of nSpk.
 * irc_sort_load reads the same layout back (ordrho to int64).  Both
 * synchronise the stream. */
int irc_sort_save(const char *path, const float *rho, const float *delta, const int64_t *nneigh,
                  const int64_t *ordrho, int64_t nSpk, void *stream);
int irc_sort_load(const char *path, float *rho, float *delta, int64_t *nneigh, int64_t *ordrho, int64_t nSpk,
                  void *stream);

/* out[i] = (float)in[i] for n FP16 values (device pointers; in 4-byte and out
 * 16-byte aligned): features streamed from host memory as FP16 are widened
 * to the FP32 the kernels read.  No reference counterpart. */
int irc_f16_to_f32(float *out, const void *in, int64_t n, void *stream);

/* The drift linkage of calc_drift_ (matlab/irc2.m:6373-6465) on the device.
 * vrAmp, vrPos [nSpk] (device): spike amplitudes and positions (second
 * column of mrPos_spk).  Chunks of equal spike counts, viLim [n+1] int64
 * (device, 0-based: chunk c = spikes viLim[c] .. viLim[c+1]-1); per chunk a
 * histcounts2 of (amplitude, position) over the quantile_vr_ edges
 * ((0:nQuantile)/nQuantile of the amplitudes, (0:nSites)/nSites of the
 * positions); miDrift [nTime_batch x n] int32 (device, 0-based): column j =
 * the nTime_batch chunks whose count columns are nearest chunk j's
 * (Euclidean, ties by chunk index), over all chunks when n <=
 * nTime_max_drift, else over calc_drift_'s band of |i - j| <=
 * nTime_max_drift/4 widened at both ends.  mlDrift(i, j) of the reference
 * is "i is listed in column j".  nDrift_out (HOST) = n; with nTime_batch >=
 * nTime_drift (the reference's single-chunk branch) n = 1, viLim = {0,
 * nSpk} and column 0 lists chunk 0.  nTime_max_drift must be a multiple of
 * 4.  Synchronises the stream. */
int irc_calc_drift(int32_t *miDrift, int64_t *viLim, int *nDrift_out, const float *vrAmp, const float *vrPos,
                   int64_t nSpk, int nSites, int nTime_drift, int nTime_batch, int nTime_max_drift, int nQuantile,
                   void *stream);

/* The output normalisation of sort_ (matlab/irc2.m:3263-3264):
 *   vrRho = vrRho / max(vrRho);  [~, ordrho] = sort(vrRho, 'descend')
 * rho [nSpk] is normalised in place (max skips NaN; single division);
 * ordrho [nSpk] receives 1-based spike ids in MATLAB's descending order
 * (NaN first, equal values in index order).  Device pointers. */
int irc_sort_rho(float *rho, int64_t *ordrho, int64_t nSpk, void *stream);

/* Largest number of peaks (spikes with delta >= delta_cut) accepted by
 * irc_assign_cluster_knn; more returns IRC_E_UNSUPPORTED. */
#define IRC_CLUSTER_MAX_PEAKS 131072

/* The cluster assignment of postCluster_ (matlab/irc2.m:6520-6535):
 * assignCluster_knn_ (:6640-6694) -- peaks = delta >= delta_cut in
 * descending rho order, peaks merged where their kNN lists share a spike
 * (cell2map_, :6754-6805, including its ten-repeat cap and overwrite
 * order), labels propagated to the other spikes along nneigh in ordrho
 * order (at most ten in-place passes) -- then dpclus_remove_count_
 * (:6735-6750), which drops clusters with fewer than min_count spikes.
 *
 * Device pointers: rho, delta [nSpk] (normalised, as sort_ leaves them);
 * ordrho, nneigh [nSpk] 1-based spike ids; miKnn [knn x nSpk] int64
 * column-major, the kNN list of every spike (only equality between the
 * values matters; the reference reads the peaks' columns from its
 * _knn_<site>.irc files).  Outputs: viClu [nSpk] int32 labels (0 = none);
 * icl [cap] 1-based centre spike ids and vnSpk_clu [cap] spikes per cluster,
 * first nClu entries.  counts (HOST, 3 entries) = { nClu, nClu_pre (peaks),
 * nClu_post (clusters after the merge, before dpclus_remove_count_) }.
 * delta_cut is compared in single precision.  Synchronises the stream.
 *
 * Errors: IRC_E_INVAL where MATLAB would raise an index error (an ordrho or
 * nneigh entry it reads outside 1..nSpk), when ordrho is not a permutation
 * of 1..nSpk (sort_ always gives one; the reference would run on without
 * an error), or when nClu > cap (counts still filled). */
int irc_assign_cluster_knn(int32_t *viClu, int64_t *icl, int32_t *vnSpk_clu, int64_t cap, int64_t *counts,
                           const float *rho, const float *delta, const int64_t *ordrho,
                           const int64_t *nneigh, const int64_t *miKnn, int knn, int64_t nSpk,
                           float delta_cut, int min_count, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* IRCGB300_H */
