// reduce_noalloc.cu -- mass/momentum reduction that allocates nothing.
//
// lbx_reduce_mass_momentum_f64 obtains its partial-sum scratch with
// cudaMalloc on first use.  Some callers cannot let a library allocate device
// memory at that point: an application that hands all of HBM to its own pool
// at start-up, or a latency-bound loop that must not take the allocator's
// locks.  This variant keeps its scratch in the file-scope array below.
//
// Facts a caller relies on:
//  * the array holds kReduceBlocks x 8 doubles (32 KiB); every GPU that
//    loads the library holds it until the process exits;
//  * the first call on a device (with that device current) looks up the
//    array's device address with cudaGetSymbolAddress and caches it; make
//    that first call before any stream capture;
//  * all calls share the array.  Each call's first pass writes every partial
//    slot that its second pass reads, so nothing has to start at zero, but
//    calls that overlap on the GPU (for example on two streams) race on it;
//  * inputs of more than kNoAllocMaxCells cells are rejected with
//    LBX_ERR_ARG before any GPU work.
#include <atomic>
#include <mutex>

#include "kernels.cuh"
#include "lbx.h"
#include "sim_internal.h"

namespace {

constexpr size_t kNoAllocScratch = (size_t)lbx::kReduceBlocks * 8;  // doubles
constexpr size_t kNoAllocMaxCells = 0x7fffffff;  // cell index range of the kernel
constexpr int kMaxDevices = 64;

// Host code must not pass this symbol to a kernel: on the host it names a
// stand-in object, not device memory.  Its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratch];

std::mutex g_setup_mu;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// device address of the scratch array on the current device (set up once)
int scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    lbx::note_error("cudaGetDevice", e);
    return lbx::status_from_cuda(e);
  }
  if (dev < 0 || dev >= kMaxDevices) return LBX_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> g(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      lbx::note_error("cudaGetSymbolAddress", e);
      return lbx::status_from_cuda(e);
    }
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return LBX_OK;
}

}  // namespace

extern "C" int lbx_reduce_mass_momentum_f64_noalloc(const double* f, size_t ncells, double* out4,
                                                    void* stream) {
  if (!f || !out4 || ncells == 0) return LBX_ERR_ARG;
  if (ncells > kNoAllocMaxCells) return LBX_ERR_ARG;  // beyond the stated maximum
  static_assert(kNoAllocScratch == (size_t)lbx::kReduceBlocks * 8,
                "scratch must hold one partial set per first-pass block");
  double* scratch = nullptr;
  const int rc = scratch_address(&scratch);
  if (rc != LBX_OK) return rc;
  const lbx::Box3 b = lbx::make_box((int)ncells, 1, 1, 0);
  const cudaError_t e = lbx::launch_reduce<double>(f, b, lbx::empty_ibox(), 0.0, scratch, out4,
                                                   (cudaStream_t)stream);
  if (e != cudaSuccess) {
    lbx::note_error("lbx_reduce_mass_momentum_f64_noalloc", e);
    return lbx::status_from_cuda(e);
  }
  return LBX_OK;
}
