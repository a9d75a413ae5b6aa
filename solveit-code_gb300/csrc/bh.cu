// bh.cu -- Barnes-Hut treecode on GB300 (pending).
#include "sv_internal.cuh"

namespace sv {
sv_status bh_accel(sv_ctx *c) { return set_error(c, SV_ERR_UNSUPPORTED, "Barnes-Hut not built yet"); }
}  // namespace sv
