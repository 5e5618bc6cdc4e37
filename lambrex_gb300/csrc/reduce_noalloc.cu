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
//    that first call before any stream capture.  The cache is keyed by the
//    device's current context, so after a context is destroyed and made
//    anew (cudaDeviceReset) the next call looks the address up again; make
//    that call before any capture too;
//  * all calls share the array.  Each call's first pass writes every partial
//    slot that its second pass reads, so nothing has to start at zero, but
//    calls that overlap on the GPU (for example on two streams) race on it;
//  * inputs of more than kNoAllocMaxCells cells are rejected with
//    LBX_ERR_ARG before any GPU work.
#include <cuda.h>  // CUcontext / CUresult types; entry points resolved at run time

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
struct ScratchSlot {
  unsigned long long ctx_id = 0;  // context the address belongs to (0: unknown)
  double* addr = nullptr;
};
ScratchSlot g_scratch_addr[kMaxDevices];

// Unique id of the calling thread's current context (cuCtxGetId), through
// the driver entry points the runtime exposes; 0 if the driver lacks them.
unsigned long long current_context_id() {
  typedef CUresult (*GetCurrentFn)(CUcontext*);
  typedef CUresult (*GetIdFn)(CUcontext, unsigned long long*);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrentFn>(p);
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetIdFn>(p);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  return get_id(ctx, &id) == CUDA_SUCCESS ? id : 0;
}

// device address of the scratch array in the current context (set up once
// per device, again whenever the device's context has been re-created)
int scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    lbx::note_error("cudaGetDevice", e);
    return lbx::status_from_cuda(e);
  }
  if (dev < 0 || dev >= kMaxDevices) return LBX_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> g(g_setup_mu);
  ScratchSlot& slot = g_scratch_addr[dev];
  const unsigned long long ctx = current_context_id();
  if (!slot.addr || ctx == 0 || ctx != slot.ctx_id) {  // no context yet: the lookup makes it
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      lbx::note_error("cudaGetSymbolAddress", e);
      return lbx::status_from_cuda(e);
    }
    slot.addr = static_cast<double*>(p);
    slot.ctx_id = current_context_id();  // the lookup creates the context if needed
  }
  *out = slot.addr;
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
