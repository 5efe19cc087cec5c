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
