// Shared by the host-only translation units.
#pragma once
#include <string>
#include "../../../include/bcsr_spmm.h"

namespace spmm {
// Records msg as the calling thread's last error (same slot spmm_last_error reads).
spmm_status host_fail(spmm_status st, const std::string& msg);
}  // namespace spmm
