// irc_capi.cu -- error reporting and version of the C ABI.
#include <cstdarg>
#include <cstdio>

#include "irc_common.cuh"

namespace {
thread_local char g_err[512] = "";
}

namespace irc_host {

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char *where)
{
    set_error("%s: %s (%s)", where, cudaGetErrorName(e), cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? IRC_E_NOMEM : IRC_E_CUDA;
}

int check_plan(const char *who, const int32_t *q0, const int32_t *nq, const int32_t *roff, const int32_t *rs,
               const int32_t *rn, int nChunks, int q_base, int n_out, int nF, long long *pairs, int *max_nq)
{
    if (!q0 || !nq || !roff || !rs || !rn || nChunks <= 0 || n_out <= 0 || nF <= 0) {
        set_error("%s: null pointer or empty plan", who);
        return IRC_E_INVAL;
    }
    if (nChunks >= (1 << 28)) {                       // chunk ids share a word with a 3-bit part number
        set_error("%s: %d chunks (at most 2^28 - 1)", who, nChunks);
        return IRC_E_INVAL;
    }
    const long long nRuns = roff[nChunks];
    if (roff[0] != 0 || nRuns <= 0) {
        set_error("%s: bad roff (roff[0] = %d, roff[nChunks] = %lld)", who, roff[0], nRuns);
        return IRC_E_INVAL;
    }
    const long long qlo = q_base, qhi = (long long)q_base + n_out;
    long long np = 0;
    int mq = 0;
    for (int i = 0; i < nChunks; ++i) {
        const long long a = q0[i], b = (long long)q0[i] + nq[i];
        if (nq[i] <= 0 || a < 0 || b > nF || a < qlo || b > qhi || roff[i + 1] <= roff[i] || roff[i + 1] > nRuns) {
            set_error("%s: chunk %d out of range", who, i);
            return IRC_E_INVAL;
        }
        long long cand = 0;
        for (int r = roff[i]; r < roff[i + 1]; ++r) {
            if (rs[r] < 0 || rn[r] <= 0 || (long long)rs[r] + rn[r] > nF) {
                set_error("%s: run %d out of range", who, r);
                return IRC_E_INVAL;
            }
            cand += rn[r];
        }
        np += cand * nq[i];
        mq = nq[i] > mq ? nq[i] : mq;
    }
    if (pairs) *pairs = np;
    if (max_nq) *max_nq = mq;
    return IRC_OK;
}

}  // namespace irc_host

extern "C" {

int irc_version(void) { return 1 * 10000 + 0 * 100 + 0; }

const char *irc_last_error(void) { return g_err; }

const char *irc_status_string(int status)
{
    switch (status) {
    case IRC_OK: return "ok";
    case IRC_E_INVAL: return "invalid argument";
    case IRC_E_NC: return "feature count above the kernel maximum";
    case IRC_E_CUDA: return "CUDA error";
    case IRC_E_NOMEM: return "device allocation failed";
    case IRC_E_TIMEOUT: return "device-side wait timed out";
    case IRC_E_UNSUPPORTED: return "mode not supported";
    default: return "unknown status";
    }
}

}  // extern "C"
