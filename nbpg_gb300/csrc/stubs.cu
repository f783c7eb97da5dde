// Entry points whose kernels are not in this build yet.
#include "internal.h"
using namespace nbpg;
extern "C" nbpg_status nbpg_build(nbpg_index *, const nbpg_build_params *, nbpg_build_stats *, uint32_t *, uint32_t *)
{
    set_error("nbpg_build: not built");
    return NBPG_ERR_UNSUPPORTED;
}
