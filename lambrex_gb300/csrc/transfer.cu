// transfer.cu -- copies between a caller's (pageable) host buffer and the
// device.
//
// On the Grace host a direct cudaMemcpy between pageable memory and the
// device runs at ~200 GB/s over NVLink-C2C when the buffer's pages were used
// recently, but with memory backed by transparent huge pages (numpy's large
// arrays) it fell to 30-60 GB/s in either direction after the process had
// been idle for a few seconds, and page-locking the caller's buffer for the
// copy (cudaHostRegister) varied as much.  Large copies therefore go direct
// chunk by chunk while each chunk runs at the link rate, and the rest goes
// through pinned staging buffers as soon as one does not: a persistent pool
// of CPU threads moves one 64 MB chunk between the caller's buffer and a
// staging buffer while the copy engine moves others.  Measured on the GB300
// host: memcpy into pinned memory ~14 GB/s per thread, ~125 GB/s with 12
// threads; the copy engine ~210 GB/s; the staged upload of 4.3 GB ~48 ms in
// every state tried, the direct one 22 ms with recently used pages.
//
// Where the device reads and writes pageable host memory through the host's
// page tables (cudaDevAttrPageableMemoryAccess: Grace over NVLink-C2C), a
// copy kernel instead moves the caller's buffer at the link rate whatever
// the state of its pages: measured on the GB300 host 198 GB/s host -> device
// and 170 GB/s device -> host, on warm, cold and freshly written buffers
// alike, against 78-178 and 50-154 GB/s for cudaMemcpy from the same
// pageable buffers; on memory backed by transparent huge pages (numpy marks
// its large arrays for them) it ran at 3-9 GB/s.  Large copies of anonymous
// memory (the caller's arrays and vectors) therefore start with a small
// timed kernel chunk and keep the kernel while it runs at the link rate;
// otherwise, and for file-backed mappings, they take the copy-engine path
// above.  LBX_HOST_ACCESS=copy selects that path for every copy.
// Page-locked buffers (cudaHostAlloc, cudaHostRegister) go to the copy
// engine in one piece.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "sim_internal.h"

namespace lbx {

namespace {

// ---- copies by a kernel that dereferences the host pointer ----------------
constexpr size_t kKernelProbeChunk = (size_t)4 << 20;  // first kernel chunk of a copy
// B/s below which the kernel hands a copy to the copy engine: a 4 MB chunk
// at the link rate measures ~100 GB/s with its launch and wait, on huge-page
// memory 3-9 GB/s
constexpr double kKernelMinRate = 50e9;
constexpr int kMaxDev = 64;

template <typename W>
__global__ void k_copy_words(const W* __restrict__ src, W* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

template <typename W>
cudaError_t launch_copy_words(const void* src, void* dst, size_t n, int sms, cudaStream_t st) {
  if (!n) return cudaSuccess;
  const size_t want = (n + 255) / 256;
  const unsigned grid = (unsigned)std::min<size_t>(want, (size_t)sms * 16);
  k_copy_words<W><<<grid, 256, 0, st>>>(static_cast<const W*>(src), static_cast<W*>(dst), n);
  return cudaGetLastError();
}

// whole copy: 16-byte words when both ends allow, else 8-byte, else bytes
cudaError_t kernel_copy(void* dst, const void* src, size_t bytes, int sms, cudaStream_t st) {
  const uintptr_t a = (uintptr_t)dst | (uintptr_t)src;
  size_t done = 0;
  cudaError_t e = cudaSuccess;
  if ((a & 15) == 0) {
    e = launch_copy_words<uint4>(src, dst, bytes / 16, sms, st);
    done = bytes / 16 * 16;
  } else if ((a & 7) == 0) {
    e = launch_copy_words<uint2>(src, dst, bytes / 8, sms, st);
    done = bytes / 8 * 8;
  }
  if (e == cudaSuccess && done < bytes)
    e = launch_copy_words<unsigned char>(static_cast<const char*>(src) + done,
                                         static_cast<char*>(dst) + done, bytes - done, sms, st);
  return e;
}

// SM count of the current device when its kernels may dereference pageable
// host memory, 0 otherwise (asked once per device)
int host_access_sms() {
  static std::atomic<int> cache[kMaxDev];
  static std::once_flag once;
  static bool forced_off = false;
  std::call_once(once, [] {
    for (auto& c : cache) c.store(-1);
    const char* v = std::getenv("LBX_HOST_ACCESS");
    forced_off = v && std::strcmp(v, "copy") == 0;
  });
  if (forced_off) return 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return 0;
  int c = cache[dev].load();
  if (c < 0) {
    int pma = 0, pht = 0, sms = 0;
    if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pht, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) !=
            cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      pma = 0;
    c = (pma && pht) ? sms : 0;
    cache[dev].store(c);
  }
  return c;
}

// Whether [p, p + bytes) lies in anonymous mappings of this process (inode 0,
// no backing file) that allow reading, and writing when `write`: the lines
// of /proc/self/maps covering the range, which must be contiguous.
bool anonymous_range(const void* p, size_t bytes, bool write) {
  FILE* fp = std::fopen("/proc/self/maps", "r");
  if (!fp) return false;
  uintptr_t lo = (uintptr_t)p;
  const uintptr_t hi = lo + bytes;
  char line[512];
  bool ok = false;
  while (std::fgets(line, sizeof line, fp)) {
    unsigned long long a = 0, b = 0, off = 0, inode = 0;
    char perm[5] = {0};
    unsigned dmaj = 0, dmin = 0;
    int path = 0;
    if (std::sscanf(line, "%llx-%llx %4s %llx %x:%x %llu %n", &a, &b, perm, &off, &dmaj, &dmin,
                    &inode, &path) < 7)
      continue;
    if (b <= lo || a > lo) continue;  // not the mapping that holds lo
    const char* name = line + path;
    const bool special = name[0] == '[' && std::strncmp(name, "[heap]", 6) != 0 &&
                         std::strncmp(name, "[stack]", 7) != 0;
    if (inode != 0 || special || perm[0] != 'r' || (write && perm[1] != 'w')) break;
    if (b >= hi) {
      ok = true;
      break;
    }
    lo = b;  // the rest of the range must start in the next mapping
  }
  std::fclose(fp);
  return ok;
}

constexpr size_t kStageChunk = (size_t)64 << 20;  // bytes per staging buffer
constexpr size_t kStageMin = (size_t)64 << 20;    // smaller copies go direct
constexpr size_t kProbeChunk = (size_t)16 << 20;  // first direct chunk of a large copy
constexpr double kDirectMinRate = 100e9;          // B/s below which the rest is staged
constexpr int kBufs = 4;                          // staging buffers
constexpr unsigned kMaxCopyThreads = 12;          // memcpy saturates near 12

// Persistent copy threads: copy() splits one memcpy over all of them (the
// caller takes part 0) and returns when every part is done.  The threads
// sleep on a condition variable between copies.
class CopyPool {
 public:
  explicit CopyPool(unsigned threads) : T_(threads) {
    for (unsigned i = 1; i < T_; ++i) ts_.emplace_back([this, i] { worker(i); });
  }
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> l(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : ts_) t.join();
  }
  void copy(char* dst, const char* src, size_t len) {
    {
      std::lock_guard<std::mutex> l(mu_);
      dst_ = dst;
      src_ = src;
      len_ = len;
      left_.store(T_ - 1);
      ++gen_;
    }
    cv_.notify_all();
    part(0);
    while (left_.load() > 0) std::this_thread::yield();
  }

 private:
  void part(unsigned i) {
    const size_t p = (len_ + T_ - 1) / T_, o = (size_t)i * p;
    if (o < len_) std::memcpy(dst_ + o, src_ + o, std::min(p, len_ - o));
  }
  void worker(unsigned i) {
    long seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> l(mu_);
        cv_.wait(l, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
      }
      part(i);
      left_.fetch_sub(1);
    }
  }
  const unsigned T_;
  std::vector<std::thread> ts_;
  std::mutex mu_;
  std::condition_variable cv_;
  long gen_ = 0;
  bool stop_ = false;
  char* dst_ = nullptr;
  const char* src_ = nullptr;
  size_t len_ = 0;
  std::atomic<unsigned> left_{0};
};

// process-wide staging area (allocated on first use, kept until exit)
struct Stage {
  std::mutex mu;
  char* buf[kBufs] = {};
  cudaEvent_t ev[kBufs] = {};  // the copy engine is done with buffer b
  int device = -1;
  CopyPool* pool = nullptr;
};
Stage& stage() {
  static Stage s;
  return s;
}

// Events belong to the device that made them; wait for and drop them.
void stage_drop_events(Stage& S) {
  for (int b = 0; b < kBufs; ++b)
    if (S.ev[b]) {
      cudaEventSynchronize(S.ev[b]);
      cudaEventDestroy(S.ev[b]);
      S.ev[b] = nullptr;
    }
}

// All-or-nothing set-up: the pinned buffers and the copy pool once per
// process (S.pool is set only when every buffer exists), the events once per
// device (S.device is set only when every event exists).  A failure part-way
// leaves nothing half made, so the next call starts over.
cudaError_t stage_setup(Stage& S) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (S.pool && S.device == dev) return cudaSuccess;
  if (!S.pool) {
    for (int b = 0; b < kBufs; ++b) {
      e = cudaHostAlloc(&S.buf[b], kStageChunk, cudaHostAllocPortable);
      if (e != cudaSuccess) {
        S.buf[b] = nullptr;
        for (int c = 0; c < b; ++c) {
          cudaFreeHost(S.buf[c]);
          S.buf[c] = nullptr;
        }
        return e;
      }
    }
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    static CopyPool pool(std::min(kMaxCopyThreads, hw));
    S.pool = &pool;
  }
  stage_drop_events(S);
  S.device = -1;
  for (int b = 0; b < kBufs; ++b) {
    e = cudaEventCreateWithFlags(&S.ev[b], cudaEventDisableTiming);
    if (e != cudaSuccess) {
      S.ev[b] = nullptr;
      stage_drop_events(S);
      return e;
    }
  }
  S.device = dev;
  return cudaSuccess;
}

// Direct copies chunk by chunk, each timed (after the stream's earlier work
// is done, so that only the copy is timed): while they run at the link rate
// they continue; the first chunk below kDirectMinRate stops them and the
// caller stages the rest.  `done` returns the bytes copied.  The chunks are
// moved by the copy kernel where the device reads pageable memory and the
// host range (`host`, written when host_write) is anonymous memory, and by
// the copy engine otherwise; a kernel chunk that runs slowly hands the rest
// to copy-engine chunks first.  (Measured on the GB300 host: the kernel
// reads and writes plain anonymous pages at 198 / 170 GB/s, but memory that
// numpy backs with transparent huge pages ran at 3-9 GB/s that way, so the
// kernel's first chunk is small.)
cudaError_t copy_direct_while_fast(char* dst, const char* src, size_t bytes, cudaMemcpyKind kind,
                                   cudaStream_t st, size_t& done, const void* host,
                                   bool host_write) {
  done = 0;
  cudaError_t e = cudaStreamSynchronize(st);
  int sms = host_access_sms();
  if (sms && !anonymous_range(host, bytes, host_write)) sms = 0;
  size_t chunk = sms ? kKernelProbeChunk : kProbeChunk;
  while (e == cudaSuccess && done < bytes) {
    const size_t len = std::min(chunk, bytes - done);
    const auto t0 = std::chrono::steady_clock::now();
    e = sms ? kernel_copy(dst + done, src + done, len, sms, st)
            : cudaMemcpyAsync(dst + done, src + done, len, kind, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) break;
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    done += len;
    if ((double)len < (sms ? kKernelMinRate : kDirectMinRate) * dt) {
      if (!sms) break;
      sms = 0;  // the kernel is slow on this memory: try the copy engine
      chunk = kProbeChunk;
      continue;
    }
    chunk = kStageChunk;
  }
  return e;
}

}  // namespace

// whether p is page-locked host memory known to CUDA (cudaHostAlloc,
// cudaHostRegister, or pinned by another user of the same context): the copy
// engine moves it at the link rate (211 GB/s measured for 4.3 GB), while a
// kernel reading it over the mapping is slower
static bool pinned_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the error of an unknown pointer
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

cudaError_t upload_host(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (bytes < kStageMin || pinned_host(src)) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    return e == cudaSuccess ? cudaStreamSynchronize(st) : e;
  }
  size_t off = 0;
  cudaError_t e = copy_direct_while_fast(static_cast<char*>(dst), static_cast<const char*>(src),
                                         bytes, cudaMemcpyHostToDevice, st, off, src, false);
  if (e != cudaSuccess || off == bytes) return e;
  Stage& S = stage();
  std::lock_guard<std::mutex> lock(S.mu);
  e = stage_setup(S);
  if (e != cudaSuccess) return e;
  int b = 0;
  while (off < bytes) {
    const size_t len = std::min(kStageChunk, bytes - off);
    e = cudaEventSynchronize(S.ev[b]);  // its previous copy is done
    if (e != cudaSuccess) return e;
    S.pool->copy(S.buf[b], static_cast<const char*>(src) + off, len);
    e = cudaMemcpyAsync(static_cast<char*>(dst) + off, S.buf[b], len, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    e = cudaEventRecord(S.ev[b], st);
    if (e != cudaSuccess) return e;
    off += len;
    b = (b + 1) % kBufs;
  }
  return cudaStreamSynchronize(st);
}

cudaError_t download_host(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (bytes < kStageMin || pinned_host(dst)) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
    return e == cudaSuccess ? cudaStreamSynchronize(st) : e;
  }
  size_t base = 0;
  cudaError_t e = copy_direct_while_fast(static_cast<char*>(dst), static_cast<const char*>(src),
                                         bytes, cudaMemcpyDeviceToHost, st, base, dst, true);
  if (e != cudaSuccess || base == bytes) return e;
  Stage& S = stage();
  std::lock_guard<std::mutex> lock(S.mu);
  e = stage_setup(S);
  if (e != cudaSuccess) return e;
  const size_t rest = bytes - base;
  const size_t chunks = (rest + kStageChunk - 1) / kStageChunk;
  auto issue = [&](size_t c) {  // device -> staging buffer c % kBufs
    const size_t off = base + c * kStageChunk, len = std::min(kStageChunk, bytes - off);
    const int b = (int)(c % kBufs);
    // a copy into b left in flight by an earlier call that failed part-way
    // (possibly on another stream) must land before this one
    cudaError_t r = cudaEventSynchronize(S.ev[b]);
    if (r != cudaSuccess) return r;
    r = cudaMemcpyAsync(S.buf[b], static_cast<const char*>(src) + off, len,
                        cudaMemcpyDeviceToHost, st);
    return r == cudaSuccess ? cudaEventRecord(S.ev[b], st) : r;
  };
  for (size_t c = 0; c < chunks && c < (size_t)kBufs; ++c)
    if ((e = issue(c)) != cudaSuccess) return e;
  for (size_t c = 0; c < chunks; ++c) {
    const int b = (int)(c % kBufs);
    const size_t off = base + c * kStageChunk, len = std::min(kStageChunk, bytes - off);
    e = cudaEventSynchronize(S.ev[b]);  // chunk c has arrived
    if (e != cudaSuccess) return e;
    S.pool->copy(static_cast<char*>(dst) + off, S.buf[b], len);
    if (c + kBufs < chunks && (e = issue(c + kBufs)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace lbx
