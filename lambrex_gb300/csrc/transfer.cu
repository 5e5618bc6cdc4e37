// transfer.cu -- host -> device upload of a caller's (pageable) buffer.
//
// On the Grace host a direct cudaMemcpy from pageable memory runs at up to
// ~190 GB/s over NVLink-C2C when the buffer's pages were used recently, but
// from memory backed by transparent huge pages (numpy's large arrays) it can
// drop to 2-10 GB/s after the process was idle for a few seconds.  Copying
// through pinned staging buffers keeps the GPU out of the caller's page
// tables: CPU threads copy a chunk into one of two pinned buffers while the
// copy engine moves the previous chunk, at a steady ~60 GB/s.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "sim_internal.h"

namespace lbx {

namespace {

constexpr size_t kStageChunk = (size_t)64 << 20;     // bytes per staging buffer
constexpr size_t kStageMin = (size_t)64 << 20;       // smaller copies go direct
constexpr unsigned kMaxCopyThreads = 8;

// process-wide staging area (allocated on first use, kept until exit)
struct Stage {
  std::mutex mu;
  char* buf[2] = {nullptr, nullptr};
  cudaEvent_t free_ev[2] = {nullptr, nullptr};  // buffer b may be refilled
  int device = -1;
};
Stage& stage() {
  static Stage s;
  return s;
}

cudaError_t stage_setup(Stage& S) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (S.buf[0] && S.device == dev) return cudaSuccess;
  if (S.buf[0]) {  // another device: pinned memory is portable, events are not
    for (int b = 0; b < 2; ++b) {
      cudaEventSynchronize(S.free_ev[b]);
      cudaEventDestroy(S.free_ev[b]);
      S.free_ev[b] = nullptr;
    }
  } else {
    for (int b = 0; b < 2; ++b) {
      e = cudaHostAlloc(&S.buf[b], kStageChunk, cudaHostAllocPortable);
      if (e != cudaSuccess) return e;
    }
  }
  for (int b = 0; b < 2; ++b) {
    e = cudaEventCreateWithFlags(&S.free_ev[b], cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
  }
  S.device = dev;
  return cudaSuccess;
}

void parallel_copy(char* dst, const char* src, size_t len, unsigned threads) {
  if (threads <= 1 || len < ((size_t)4 << 20)) {
    std::memcpy(dst, src, len);
    return;
  }
  std::vector<std::thread> ts;
  const size_t part = (len + threads - 1) / threads;
  for (unsigned t = 1; t < threads; ++t) {
    const size_t o = t * part;
    if (o >= len) break;
    const size_t l = std::min(part, len - o);
    ts.emplace_back([=] { std::memcpy(dst + o, src + o, l); });
  }
  std::memcpy(dst, src, std::min(part, len));
  for (auto& t : ts) t.join();
}

}  // namespace

cudaError_t upload_host(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (bytes < kStageMin) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    return e == cudaSuccess ? cudaStreamSynchronize(st) : e;
  }
  Stage& S = stage();
  std::lock_guard<std::mutex> lock(S.mu);
  cudaError_t e = stage_setup(S);
  if (e != cudaSuccess) return e;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const unsigned threads = std::min(kMaxCopyThreads, std::max(1u, hw / 2));
  size_t off = 0;
  int b = 0;
  while (off < bytes) {
    const size_t len = std::min(kStageChunk, bytes - off);
    e = cudaEventSynchronize(S.free_ev[b]);  // its previous copy is done
    if (e != cudaSuccess) return e;
    parallel_copy(S.buf[b], static_cast<const char*>(src) + off, len, threads);
    e = cudaMemcpyAsync(static_cast<char*>(dst) + off, S.buf[b], len, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    e = cudaEventRecord(S.free_ev[b], st);
    if (e != cudaSuccess) return e;
    off += len;
    b ^= 1;
  }
  return cudaStreamSynchronize(st);
}

}  // namespace lbx
