// sim_internal.h -- helpers shared by the translation units of liblbx_cuda.so.
#pragma once
#include <cuda_runtime.h>

namespace lbx {
// map a CUDA error to an lbx status code
int status_from_cuda(cudaError_t e);
// remember the last CUDA error text (reported by lbx_status_string)
void note_error(const char* where, cudaError_t e);
}  // namespace lbx
