// tcgen05 (UMMA) pipeline for 64-row blocks. Placeholder until the kernel lands:
// reports "unsupported" so the dispatcher uses the mma.sync pipeline.
#include "internal.h"

namespace spmm {
spmm_status launch_tc(const LaunchRequest& r) {
  (void)r;
  return fail(SPMM_ERR_UNSUPPORTED, "tcgen05 pipeline not built");
}
}  // namespace spmm
