// fmm.cu -- fast multipole method on GB300 (pending).
#include "sv_internal.cuh"

namespace sv {
sv_status fmm_accel(sv_ctx *c) { return set_error(c, SV_ERR_UNSUPPORTED, "FMM not built yet"); }
void fmm_free(sv_ctx *) {}
}  // namespace sv
