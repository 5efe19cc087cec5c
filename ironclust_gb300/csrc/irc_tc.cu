// irc_tc.cu -- tensor-core (tcgen05) site kNN: placeholder until the kernel lands.
#include "irc_common.cuh"
#include "irc_plan.cuh"

int irc_site_knn_tc(irc_plan *, const float *, int, int, int, float *, float *, int32_t *, float *,
                    cudaStream_t)
{
    irc_host::set_error("irc_site_knn: tensor-core modes not built");
    return IRC_E_UNSUPPORTED;
}
