// sim_internal.h -- helpers shared by the translation units of liblbx_cuda.so.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

namespace lbx {
// map a CUDA error to an lbx status code
int status_from_cuda(cudaError_t e);
// remember the last CUDA error text (reported by lbx_status_string)
void note_error(const char* where, cudaError_t e);

// Copy a caller's host buffer to device memory and wait for it on `st`;
// large copies are read by a kernel over the host's page tables where the
// device allows it, else go through pinned staging buffers (transfer.cu).
cudaError_t upload_host(void* dst, const void* src, size_t bytes, cudaStream_t st);
// Copy device memory into a caller's host buffer after the work queued on
// `st`, and wait for it; large copies are written by a kernel, else go
// through the same staging buffers.
cudaError_t download_host(void* dst, const void* src, size_t bytes, cudaStream_t st);

// Named host range for profilers (NVTX; a no-op unless a tool is attached).
// Every C-ABI call that launches work opens one, so a timeline shows which
// API call issued which kernels.
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range&) = delete;
  Range& operator=(const Range&) = delete;
};
}  // namespace lbx
