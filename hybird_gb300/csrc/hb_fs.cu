// hb_fs.cu -- free-surface phase (placeholder until the kernels land).
#include "hb_common.cuh"
#include "hb_ctx.h"

namespace hb {
int fs_init(hb_ctx* c) { (void)c; return HB_ERR_UNSUPPORTED; }
void launch_fs_step(hb_ctx* c, int cur) { (void)c; (void)cur; }
}  // namespace hb
