// Host-side status plumbing shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include "../../include/madi_gb300.h"

namespace madi {
namespace host {
void clear_error();
madi_status fail(madi_status code, const char* fmt, ...);
madi_status cuda_fail(cudaError_t e, const char* what);
}  // namespace host
}  // namespace madi
