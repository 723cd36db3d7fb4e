// hlbl_internal.h -- declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

namespace hg {

// Record a message for hlbl_last_error() and return `code`.
int fail(int code, const char* fmt, ...);
// Record a CUDA error for hlbl_last_error() and return HLBL_ECUDA.
int cuda_fail(cudaError_t e, const char* what);

}  // namespace hg
