// checked.cuh -- global-memory accessors with the bounds checks of the debug
// build.
//
// Every kernel reads and writes population stores and per-cell fields
// through ld_pop / st_pop / ld_cell / st_cell.  In the release library they
// are plain (read-only cached) loads and stores.  Built with LBX_CHECKED
// (liblbx_cuda_checked.so) each access first tests its element index against
// the extent of the array it addresses -- NV * sq elements for a population
// store of box b, the cell count for a per-cell field -- and on a miss counts
// it in a device counter of the translation unit, remembers the first bad
// index and skips the access (loads return 0).  Nothing traps; the host reads
// and clears the counters with lbx_debug_bounds().
#pragma once
#include <cuda_runtime.h>

#include "d3q15.cuh"

namespace lbx {

#ifdef LBX_CHECKED
// [0] = number of out-of-range accesses, [1] = first bad index (as written)
static __device__ unsigned long long g_oob[2];

__host__ __device__ __forceinline__ bool idx_ok(long long i, long long n) {
  if (i >= 0 && i < n) return true;
#ifdef __CUDA_ARCH__
  if (atomicAdd(&g_oob[0], 1ull) == 0ull) g_oob[1] = (unsigned long long)i;
#endif
  return false;
}

// Each translation unit that includes this header registers a reader of its
// own counters; lbx_debug_bounds() sums them.
using OobReader = int (*)(unsigned long long* count, long long* first, bool reset);
int register_oob_reader(OobReader r);

static int read_unit_oob(unsigned long long* count, long long* first, bool reset) {
  unsigned long long h[2] = {0ull, 0ull};
  if (cudaMemcpyFromSymbol(h, g_oob, sizeof h) != cudaSuccess) return -1;
  *count = h[0];
  *first = (long long)h[1];
  if (reset) {
    const unsigned long long z[2] = {0ull, 0ull};
    if (cudaMemcpyToSymbol(g_oob, z, sizeof z) != cudaSuccess) return -1;
  }
  return 0;
}
static const int g_oob_unit_registered = register_oob_reader(&read_unit_oob);
#else
__host__ __device__ __forceinline__ constexpr bool idx_ok(long long, long long) { return true; }
#endif

// read-only cached load on the device (a plain load in a host build, which
// runs the per-cell code off the GPU in the tests)
template <typename T>
__host__ __device__ __forceinline__ T ld_ro(const T* p) {
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}

// population store of box b: element index i = q * sq + cell (I: the
// index type of the caller, 64-bit or, for the batch engine's small boxes,
// 32-bit)
template <typename T, typename I>
__host__ __device__ __forceinline__ T ld_pop(const T* __restrict__ p, I i, const Box3& b) {
  return idx_ok((long long)i, NV * b.sq) ? ld_ro(p + i) : T(0);
}
// load of an entry the same kernel may also write (no read-only cache)
template <typename T, typename I>
__host__ __device__ __forceinline__ T ld_pop_rw(const T* p, I i, const Box3& b) {
  return idx_ok((long long)i, NV * b.sq) ? p[i] : T(0);
}
template <typename T, typename I>
__host__ __device__ __forceinline__ void st_pop(T* __restrict__ p, I i, const Box3& b, T v) {
  if (idx_ok((long long)i, NV * b.sq)) p[i] = v;
}

// per-cell field of n elements (density, velocity components, partial sums)
template <typename T>
__host__ __device__ __forceinline__ T ld_cell(const T* __restrict__ p, long long i, long long n) {
  return idx_ok(i, n) ? ld_ro(p + i) : T(0);
}
template <typename T>
__host__ __device__ __forceinline__ void st_cell(T* __restrict__ p, long long i, long long n, T v) {
  if (idx_ok(i, n)) p[i] = v;
}

}  // namespace lbx
