// kernels_step.cu -- single-box kernels: fused periodic step, equilibrium,
// hydrodynamic fields, FP64 import/export and compensated reductions.
#include <algorithm>

#include "cells.cuh"

namespace lbx {

namespace {

// Fused collide + push-stream over a periodic valid region
// (src/AmrSim.cpp:25-135; include/component.h:22-29 written as a push:
// f_new(x + c_q, q) = C(f)(x, q) is the same map as the reference's pull
// f_new(x, q) = C(f)(x - c_q, q)).
template <typename T, bool COVER, bool PAIRED>
__global__ void __launch_bounds__(256) k_step_periodic(const T* __restrict__ fin,
                                                       T* __restrict__ fout, Box3 b, IBox cov,
                                                       T om_s, T om_b, T rho0, DfRates r) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  cell_step_periodic<T, COVER, PAIRED>(fin, fout, b, cov, x, y, z, om_s, om_b, rho0, r);
}

// pull-form step P -> C(S(P)) (see cells.cuh); I = int when every element
// index of the store fits in 31 bits (up to 15 x 2^27 elements: 512^3)
template <typename T, bool PAIRED, typename I>
__global__ void __launch_bounds__(256) k_step_pull(const T* __restrict__ fin, T* __restrict__ fout,
                                                   Box3 b, T om_s, T om_b, T rho0, DfRates r) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  cell_step_pull<T, PAIRED, I>(fin, fout, b, x, y, z, om_s, om_b, rho0, r);
}

// the pull-form step with CalcHydroVars fused in (cell_step_pull_hydro)
template <typename T, bool PAIRED, typename I>
__global__ void __launch_bounds__(256) k_step_pull_hydro(const T* __restrict__ fin,
                                                         T* __restrict__ fout, Box3 b, T om_s,
                                                         T om_b, T rho0, DfRates r, double rho0_d,
                                                         double* __restrict__ rho,
                                                         double* __restrict__ u) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  cell_step_pull_hydro<T, PAIRED, I>(fin, fout, b, x, y, z, om_s, om_b, rho0, r, rho0_d, rho, u);
}

// FP64 store, periodic push step with the paired collision in its one-cell
// scalar form (collide_f64_via_df, no packed instructions): the form the
// packed collision reproduces bit for bit, kept for the device-pointer entry
// lbx_step_periodic_f64p so that the two can be compared.
__global__ void __launch_bounds__(256) k_step_periodic_pairs_scalar(const double* __restrict__ fin,
                                                                    double* __restrict__ fout,
                                                                    Box3 b, DfRates r) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  const long long c = b.at(x, y, z);
  double f[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) f[q] = ld_pop(fin, q * b.sq + c, b);
  collide_f64_via_df(f, r);
  push_periodic<double>(fout, b, x, y, z, f);
}

// Q -> R = S(Q) (SIGN = +1, leaving the pull form) or R -> Q = S^-1(R)
// (SIGN = -1, entering it): a pure shift of each population
template <typename T, int SIGN>
__global__ void k_shift(const T* __restrict__ fin, T* __restrict__ fout, Box3 b) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  T v[NV];
  gather_periodic<T, SIGN>(fin, b, x, y, z, v);
  const long long c = b.at(x, y, z);
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(fout, q * b.sq + c, b, v[q]);
}

template <typename T>
__global__ void k_equilibrium(const double* __restrict__ rho, const double* __restrict__ u,
                              T* __restrict__ f, Box3 b, double rho0) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  const long long n = (long long)b.n[0] * b.n[1] * b.n[2];
  const long long v = ((long long)z * b.n[1] + y) * b.n[0] + x;
  const double r = ld_cell(rho, v, n), ux = ld_cell(u, v, 3 * n), uy = ld_cell(u, n + v, 3 * n),
               uz = ld_cell(u, 2 * n + v, 3 * n);
  const long long c = b.at(x, y, z);
  if constexpr (sizeof(T) == 4) {
    float g[NV];
    equilibrium_shifted(r, ux, uy, uz, rho0, g);
#pragma unroll
    for (int q = 0; q < NV; ++q) st_pop(f, q * b.sq + c, b, g[q]);
  } else {
    double e[NV];
    equilibrium(r, ux, uy, uz, e);
#pragma unroll
    for (int q = 0; q < NV; ++q) st_pop(f, q * b.sq + c, b, (T)(e[q] - W(q) * rho0));
  }
}

// equilibrium of rho = 1 + amplitude on the plane coord[axis] == index, u = 0
template <typename T>
__global__ void k_init_pulse(T* __restrict__ f, Box3 b, int axis, int index, double amplitude,
                             double rho0) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  const int c[3] = {x, y, z};
  const double rho = 1.0 + (c[axis] == index ? amplitude : 0.0);
  const long long s = b.at(x, y, z);
  if constexpr (sizeof(T) == 4) {
    float g[NV];
    equilibrium_shifted(rho, 0.0, 0.0, 0.0, rho0, g);
#pragma unroll
    for (int q = 0; q < NV; ++q) st_pop(f, q * b.sq + s, b, g[q]);
  } else {
    double e[NV];
    equilibrium(rho, 0.0, 0.0, 0.0, e);
#pragma unroll
    for (int q = 0; q < NV; ++q) st_pop(f, q * b.sq + s, b, (T)(e[q] - W(q) * rho0));
  }
}

template <typename T, bool GATHER>
__global__ void k_hydro(const T* __restrict__ f, Box3 b, double rho0, double* __restrict__ rho,
                        double* __restrict__ u) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  cell_hydro<T, GATHER>(f, b, rho0, rho, u, x, y, z);
}

template <typename T, bool GATHER>
__global__ void k_copy_out(const T* __restrict__ f, Box3 b, double rho0, double* __restrict__ out) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  const long long n = (long long)b.n[0] * b.n[1] * b.n[2];
  const long long v = ((long long)z * b.n[1] + y) * b.n[0] + x;
  const long long c = b.at(x, y, z);
  T p[NV];
  if (GATHER) {
    gather_periodic<T>(f, b, x, y, z, p);
  } else {
#pragma unroll
    for (int q = 0; q < NV; ++q) p[q] = ld_pop(f, q * b.sq + c, b);
  }
#pragma unroll
  for (int q = 0; q < NV; ++q) st_cell(out, q * n + v, NV * n, (double)p[q] + W(q) * rho0);
}

template <typename T>
__global__ void k_copy_in(const double* __restrict__ in, T* __restrict__ f, Box3 b, double rho0) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  const long long n = (long long)b.n[0] * b.n[1] * b.n[2];
  const long long v = ((long long)z * b.n[1] + y) * b.n[0] + x;
  const long long c = b.at(x, y, z);
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(f, q * b.sq + c, b, (T)(ld_cell(in, q * n + v, NV * n) - W(q) * rho0));
}

// valid region of a store <-> packed FAB order in the storage type (raw, no
// shift applied): checkpoints keep the exact stored values
template <typename T>
__global__ void k_pack(const T* __restrict__ f, Box3 b, T* __restrict__ out) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  const long long n = (long long)b.n[0] * b.n[1] * b.n[2];
  const long long v = ((long long)z * b.n[1] + y) * b.n[0] + x;
  const long long c = b.at(x, y, z);
#pragma unroll
  for (int q = 0; q < NV; ++q) st_cell(out, q * n + v, NV * n, ld_pop(f, q * b.sq + c, b));
}
template <typename T>
__global__ void k_unpack(const T* __restrict__ in, T* __restrict__ f, Box3 b) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  const long long n = (long long)b.n[0] * b.n[1] * b.n[2];
  const long long v = ((long long)z * b.n[1] + y) * b.n[0] + x;
  const long long c = b.at(x, y, z);
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(f, q * b.sq + c, b, ld_cell(in, q * n + v, NV * n));
}

// Neumaier-compensated pair (s, e): value = s + e.
struct Comp {
  double s, e;
};
__device__ __forceinline__ void comp_add(Comp& a, double v) {
  const double t = a.s + v;
  if (fabs(a.s) >= fabs(v))
    a.e += (a.s - t) + v;
  else
    a.e += (v - t) + a.s;
  a.s = t;
}
__device__ __forceinline__ void comp_merge(Comp& a, const Comp& b) {
  comp_add(a, b.s);
  a.e += b.e;
}

// Block-level reduction of four compensated sums with warp shuffles.
__device__ __forceinline__ void block_reduce4(Comp* acc, double* out8) {
  __shared__ double sh[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      Comp other{__shfl_down_sync(0xffffffffu, acc[k].s, o),
                 __shfl_down_sync(0xffffffffu, acc[k].e, o)};
      comp_merge(acc[k], other);
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      sh[2 * k][warp] = acc[k].s;
      sh[2 * k + 1][warp] = acc[k].e;
    }
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      Comp c{lane < nw ? sh[2 * k][lane] : 0.0, lane < nw ? sh[2 * k + 1][lane] : 0.0};
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        Comp other{__shfl_down_sync(0xffffffffu, c.s, o), __shfl_down_sync(0xffffffffu, c.e, o)};
        comp_merge(c, other);
      }
      if (lane == 0) {
        out8[2 * k] = c.s;
        out8[2 * k + 1] = c.e;
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) k_reduce(const T* __restrict__ f, Box3 b,
                                                           IBox skip, double rho0,
                                                           double* __restrict__ partials) {
  if (!idx_ok(blockIdx.x, kReduceBlocks)) return;  // partials hold kReduceBlocks blocks
  Comp acc[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  // cell counts of every caller are below 2^31 (checked on the host), so the
  // index arithmetic stays in 32 bits
  const unsigned n = (unsigned)((long long)b.n[0] * b.n[1] * b.n[2]);
  const unsigned n0 = (unsigned)b.n[0], n1 = (unsigned)b.n[1];
  if constexpr (sizeof(T) == 4) {
    // the FP32 store's shifted populations are small: each cell's sums in
    // FP32 (rounding ~1e-9 of the fluctuations), a thread's few hundred
    // cells summed plainly in FP64 (~1e-14), the threads' and blocks' sums
    // merged compensated; the mass is rho0 per cell plus the fluctuations
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    unsigned cells = 0;
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
      const unsigned r = v / n0;
      const int x = (int)(v - r * n0);
      const int y = (int)(r % n1);
      const int z = (int)(r / n1);
      if (skip.contains(x, y, z)) continue;
      const long long c = b.at(x, y, z);
      float s = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const float fq = (float)ld_pop(f, q * b.sq + c, b);
        s += fq;
        if (CX(q)) sx += CX(q) * fq;
        if (CY(q)) sy += CY(q) * fq;
        if (CZ(q)) sz += CZ(q) * fq;
      }
      t[0] += (double)s;
      t[1] += (double)sx;
      t[2] += (double)sy;
      t[3] += (double)sz;
      ++cells;
    }
    acc[0].s = rho0 * (double)cells;
    comp_add(acc[0], t[0]);
    for (int k = 1; k < 4; ++k) acc[k].s = t[k];
  } else {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
      const unsigned r = v / n0;
      const int x = (int)(v - r * n0);
      const int y = (int)(r % n1);
      const int z = (int)(r / n1);
      if (skip.contains(x, y, z)) continue;
      const long long c = b.at(x, y, z);
      double m = rho0, jx = 0, jy = 0, jz = 0;
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const double fq = (double)ld_pop(f, q * b.sq + c, b);
        m += fq;
        if (CX(q)) jx += CX(q) * fq;
        if (CY(q)) jy += CY(q) * fq;
        if (CZ(q)) jz += CZ(q) * fq;
      }
      comp_add(acc[0], m);
      comp_add(acc[1], jx);
      comp_add(acc[2], jy);
      comp_add(acc[3], jz);
    }
  }
  block_reduce4(acc, partials + 8 * blockIdx.x);
}

__global__ void k_reduce_final(const double* __restrict__ partials, int nblocks,
                               double* __restrict__ out4) {
  Comp acc[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
#pragma unroll
    for (int k = 0; k < 4; ++k) comp_merge(acc[k], Comp{partials[8 * i + 2 * k], partials[8 * i + 2 * k + 1]});
  }
  __shared__ double res[8];
  block_reduce4(acc, res);
  __syncthreads();
  if (threadIdx.x < 4) out4[threadIdx.x] = res[2 * threadIdx.x] + res[2 * threadIdx.x + 1];
}

// sum of n doubles (the mean density that shifts an FP32 store): each
// thread adds its strided values with one FP64 addition each (n / 131,072
// values, ~1e-13 relative), the threads' and blocks' sums merge compensated;
// the order is fixed, so the sum is the same on every run
__global__ void __launch_bounds__(kReduceThreads) k_sum(const double* __restrict__ x, size_t n,
                                                       double* __restrict__ partials) {
  if (!idx_ok(blockIdx.x, kReduceBlocks)) return;
  double t = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    t += ld_cell(x, (long long)i, (long long)n);
  Comp acc[4] = {{t, 0}, {0, 0}, {0, 0}, {0, 0}};
  block_reduce4(acc, partials + 8 * blockIdx.x);
}

__global__ void k_fill(double* __restrict__ p, size_t n, double v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    st_cell(p, (long long)i, (long long)n, v);
}

// C-order user vectors -> FAB order (InitDensity/InitVelocity,
// src/AmrSim.cpp:138-295): rho(i,j,k) = rho_c[(i*ny + j)*nz + k],
// u(i,j,k,n) = u_c[((i*ny + j)*nz + k)*3 + n].  For each j this is a
// transpose of the (i, k) plane: a block stages a 32 x 32 tile through
// shared memory, reading it with k contiguous (C order; the three velocity
// components of a tile row are 96 contiguous values) and writing it with i
// contiguous (FAB order), so both sides are coalesced.  A null source leaves
// its field alone (a scalar initial value was filled separately).
constexpr int kTT = 32;  // tile edge
constexpr int kTR = 8;   // rows of threads (blockDim = kTT x kTR)
__global__ void __launch_bounds__(kTT * kTR)
    k_c_to_fab(const double* __restrict__ rho_c, const double* __restrict__ u_c,
               double* __restrict__ rho, double* __restrict__ u, int nx, int ny, int nz) {
  __shared__ double tr[kTT][kTT + 1];     // [i][k]
  __shared__ double tu[3][kTT][kTT + 1];  // [component][i][k]
  const int k0 = blockIdx.x * kTT, i0 = blockIdx.y * kTT, j = blockIdx.z;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long long n = (long long)nx * ny * nz;
  const int kn = min(kTT, nz - k0), in = min(kTT, nx - i0);
  for (int r = ty; r < in; r += kTR) {
    const long long row = ((long long)(i0 + r) * ny + j) * nz + k0;  // C index of (i, j, k0)
    if (rho_c && tx < kn) tr[r][tx] = ld_cell(rho_c, row + tx, n);
    if (u_c)
      for (int e = tx; e < 3 * kn; e += kTT) tu[e % 3][r][e / 3] = ld_cell(u_c, 3 * row + e, 3 * n);
  }
  __syncthreads();
  for (int r = ty; r < kn; r += kTR) {
    if (tx >= in) continue;
    const long long v = ((long long)(k0 + r) * ny + j) * nx + i0 + tx;  // FAB index of (i, j, k)
    if (rho_c) st_cell(rho, v, n, tr[tx][r]);
    if (u_c) {
      st_cell(u, v, 3 * n, tu[0][tx][r]);
      st_cell(u, n + v, 3 * n, tu[1][tx][r]);
      st_cell(u, 2 * n + v, 3 * n, tu[2][tx][r]);
    }
  }
}


}  // namespace

cudaError_t launch_c_to_fab(const double* rho_c, const double* u_c, double* rho, double* u,
                            int nx, int ny, int nz, cudaStream_t st) {
  const dim3 grid((unsigned)((nz + kTT - 1) / kTT), (unsigned)((nx + kTT - 1) / kTT), (unsigned)ny);
  k_c_to_fab<<<grid, dim3(kTT, kTR, 1), 0, st>>>(rho_c, u_c, rho, u, nx, ny, nz);
  return cudaGetLastError();
}

cudaError_t launch_sum(const double* x, size_t n, double* partials, double* out4, cudaStream_t st) {
  k_sum<<<kReduceBlocks, kReduceThreads, 0, st>>>(x, n, partials);
  k_reduce_final<<<1, kReduceThreads, 0, st>>>(partials, kReduceBlocks, out4);
  return cudaGetLastError();
}

cudaError_t launch_fill(double* p, size_t n, double v, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const size_t blocks = (n + 255) / 256;
  k_fill<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, st>>>(p, n, v);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_step_periodic(const T* fin, T* fout, const Box3& b, IBox covered, double om_s,
                                 double om_b, double rho0, cudaStream_t st, int block,
                                 bool paired) {
  const bool cov = covered.hi[0] >= covered.lo[0] && covered.hi[1] >= covered.lo[1] &&
                   covered.hi[2] >= covered.lo[2];
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], block);
  const dim3 grid = rl.grid;
  if constexpr (sizeof(T) == 8) {
    if (paired) {
      const DfRates r = df_rates(om_s, om_b);
      if (cov)
        k_step_periodic<double, true, true><<<grid, rl.block, 0, st>>>(fin, fout, b, covered, om_s,
                                                                    om_b, 0.0, r);
      else
        k_step_periodic<double, false, true><<<grid, rl.block, 0, st>>>(fin, fout, b, covered, om_s,
                                                                     om_b, 0.0, r);
      return cudaGetLastError();
    }
  }
  if (cov)
    k_step_periodic<T, true, false><<<grid, rl.block, 0, st>>>(fin, fout, b, covered, (T)om_s,
                                                            (T)om_b, (T)rho0, DfRates{});
  else
    k_step_periodic<T, false, false><<<grid, rl.block, 0, st>>>(fin, fout, b, covered, (T)om_s,
                                                             (T)om_b, (T)rho0, DfRates{});
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_equilibrium(const double* rho, const double* u, T* f, const Box3& b,
                               double rho0, cudaStream_t st) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  k_equilibrium<T><<<rl.grid, rl.block, 0, st>>>(rho, u, f, b, rho0);
  return cudaGetLastError();
}

// one row of x per (blockIdx.y, blockIdx.z), a block's threads along it;
// each warp folds its tagged cells' box and count before one atomic each
__global__ void k_tag_density(const double* __restrict__ rho, int nx, int ny, int nz, double ref,
                              double threshold, int* __restrict__ box6,
                              unsigned long long* __restrict__ count) {
  const int y = blockIdx.y, z = blockIdx.z;
  const int lane = threadIdx.x & 31;
  int lo[3] = {nx, ny, nz}, hi[3] = {-1, -1, -1};
  unsigned k = 0;
  for (int x0 = blockIdx.x * blockDim.x; x0 < nx; x0 += gridDim.x * blockDim.x) {
    const int x = x0 + threadIdx.x;
    if (x < nx && fabs(rho[((long long)z * ny + y) * nx + x] - ref) > threshold) {
      lo[0] = min(lo[0], x);
      hi[0] = max(hi[0], x);
      lo[1] = hi[1] = y;
      lo[2] = hi[2] = z;
      ++k;
    }
  }
  const unsigned all = 0xffffffffu;
  for (int d = 0; d < 3; ++d) {
    lo[d] = __reduce_min_sync(all, lo[d]);
    hi[d] = __reduce_max_sync(all, hi[d]);
  }
  k = __reduce_add_sync(all, k);
  if (lane == 0 && k) {
    for (int d = 0; d < 3; ++d) {
      atomicMin(box6 + d, lo[d]);
      atomicMax(box6 + 3 + d, hi[d]);
    }
    atomicAdd(count, (unsigned long long)k);
  }
}

cudaError_t launch_tag_density(const double* rho, const int* n, double ref, double threshold,
                               int* box6, unsigned long long* count, cudaStream_t st) {
  const int threads = 256;
  const dim3 grid((unsigned)std::min((n[0] + threads - 1) / threads, 8), (unsigned)n[1],
                  (unsigned)n[2]);
  k_tag_density<<<grid, threads, 0, st>>>(rho, n[0], n[1], n[2], ref, threshold, box6, count);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_hydro(const T* f, const Box3& b, double rho0, double* rho, double* u,
                         cudaStream_t st, bool gather) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  if (gather)
    k_hydro<T, true><<<rl.grid, rl.block, 0, st>>>(f, b, rho0, rho, u);
  else
    k_hydro<T, false><<<rl.grid, rl.block, 0, st>>>(f, b, rho0, rho, u);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_copy_out(const T* f, const Box3& b, double rho0, double* out, cudaStream_t st,
                            bool gather) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  if (gather)
    k_copy_out<T, true><<<rl.grid, rl.block, 0, st>>>(f, b, rho0, out);
  else
    k_copy_out<T, false><<<rl.grid, rl.block, 0, st>>>(f, b, rho0, out);
  return cudaGetLastError();
}

template <typename T, typename I>
cudaError_t launch_step_pull_i(const T* fin, T* fout, const Box3& b, double om_s, double om_b,
                               double rho0, bool paired, cudaStream_t st, int block) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], block);
  if constexpr (sizeof(T) == 8) {
    if (paired) {
      // 52 registers: blocks of 128 threads fit nine per SM (36 warps)
      // against four of 256 (32 warps); measured 1 % faster at 512^3
      const RowLaunch rp = row_launch(b.n[0], b.n[1], b.n[2], block < 128 ? block : 128);
      k_step_pull<double, true, I><<<rp.grid, rp.block, 0, st>>>(fin, fout, b, om_s, om_b, 0.0,
                                                                 df_rates(om_s, om_b));
      return cudaGetLastError();
    }
  }
  k_step_pull<T, false, I><<<rl.grid, rl.block, 0, st>>>(fin, fout, b, (T)om_s, (T)om_b, (T)rho0,
                                                          DfRates{});
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_step_pull(const T* fin, T* fout, const Box3& b, double om_s, double om_b,
                             double rho0, bool paired, cudaStream_t st, int block) {
  // the FP64 store is instruction-bound: narrower index arithmetic pays
  // there (1,889 -> 1,786 instructions per cell, paired); the FP32 store is
  // bound by HBM and keeps the 64-bit form it was tuned with
  if (sizeof(T) == 8 && (long long)NV * b.sq < (1ll << 31))
    return launch_step_pull_i<T, int>(fin, fout, b, om_s, om_b, rho0, paired, st, block);
  return launch_step_pull_i<T, long long>(fin, fout, b, om_s, om_b, rho0, paired, st, block);
}

template <typename T, typename I>
cudaError_t launch_step_pull_hydro_i(const T* fin, T* fout, const Box3& b, double om_s,
                                     double om_b, double rho0, bool paired, double* rho,
                                     double* u, cudaStream_t st) {
  if constexpr (sizeof(T) == 8) {
    if (paired) {
      const RowLaunch rp = row_launch(b.n[0], b.n[1], b.n[2], 128);
      k_step_pull_hydro<double, true, I><<<rp.grid, rp.block, 0, st>>>(
          fin, fout, b, om_s, om_b, 0.0, df_rates(om_s, om_b), rho0, rho, u);
      return cudaGetLastError();
    }
  }
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 256);
  k_step_pull_hydro<T, false, I><<<rl.grid, rl.block, 0, st>>>(fin, fout, b, (T)om_s, (T)om_b,
                                                               (T)rho0, DfRates{}, rho0, rho, u);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_step_pull_hydro(const T* fin, T* fout, const Box3& b, double om_s, double om_b,
                                   double rho0, bool paired, double* rho, double* u,
                                   cudaStream_t st) {
  if (sizeof(T) == 8 && (long long)NV * b.sq < (1ll << 31))
    return launch_step_pull_hydro_i<T, int>(fin, fout, b, om_s, om_b, rho0, paired, rho, u, st);
  return launch_step_pull_hydro_i<T, long long>(fin, fout, b, om_s, om_b, rho0, paired, rho, u, st);
}

cudaError_t launch_step_periodic_pairs_scalar(const double* fin, double* fout, const Box3& b,
                                              double om_s, double om_b, cudaStream_t st) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  k_step_periodic_pairs_scalar<<<rl.grid, rl.block, 0, st>>>(fin, fout, b, df_rates(om_s, om_b));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_init_pulse(T* f, const Box3& b, int axis, int index, double amplitude,
                              double rho0, cudaStream_t st) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  k_init_pulse<T><<<rl.grid, rl.block, 0, st>>>(f, b, axis, index, amplitude, rho0);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_unstream(const T* fin, T* fout, const Box3& b, cudaStream_t st) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  k_shift<T, -1><<<rl.grid, rl.block, 0, st>>>(fin, fout, b);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_stream_gather(const T* fin, T* fout, const Box3& b, cudaStream_t st) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  k_shift<T, 1><<<rl.grid, rl.block, 0, st>>>(fin, fout, b);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_copy_in(const double* in, T* f, const Box3& b, double rho0, cudaStream_t st) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  k_copy_in<T><<<rl.grid, rl.block, 0, st>>>(in, f, b, rho0);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pack(const T* f, const Box3& b, T* out, cudaStream_t st) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  k_pack<T><<<rl.grid, rl.block, 0, st>>>(f, b, out);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_unpack(const T* in, T* f, const Box3& b, cudaStream_t st) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  k_unpack<T><<<rl.grid, rl.block, 0, st>>>(in, f, b);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reduce(const T* f, const Box3& b, IBox skip, double rho0, double* partials,
                          double* out4, cudaStream_t st) {
  k_reduce<T><<<kReduceBlocks, kReduceThreads, 0, st>>>(f, b, skip, rho0, partials);
  k_reduce_final<<<1, kReduceThreads, 0, st>>>(partials, kReduceBlocks, out4);
  return cudaGetLastError();
}

#define LBX_INST(T)                                                                             \
  template cudaError_t launch_step_periodic<T>(const T*, T*, const Box3&, IBox, double, double, \
                                               double, cudaStream_t, int, bool);                \
  template cudaError_t launch_equilibrium<T>(const double*, const double*, T*, const Box3&,     \
                                             double, cudaStream_t);                             \
  template cudaError_t launch_hydro<T>(const T*, const Box3&, double, double*, double*,         \
                                       cudaStream_t, bool);                                     \
  template cudaError_t launch_copy_out<T>(const T*, const Box3&, double, double*, cudaStream_t, \
                                          bool);                                                \
  template cudaError_t launch_step_pull_hydro<T>(const T*, T*, const Box3&, double, double,    \
                                                 double, bool, double*, double*, cudaStream_t);  \
  template cudaError_t launch_step_pull<T>(const T*, T*, const Box3&, double, double, double,  \
                                           bool, cudaStream_t, int);                            \
  template cudaError_t launch_unstream<T>(const T*, T*, const Box3&, cudaStream_t);             \
  template cudaError_t launch_init_pulse<T>(T*, const Box3&, int, int, double, double,          \
                                            cudaStream_t);                                      \
  template cudaError_t launch_stream_gather<T>(const T*, T*, const Box3&, cudaStream_t);        \
  template cudaError_t launch_copy_in<T>(const double*, T*, const Box3&, double, cudaStream_t);  \
  template cudaError_t launch_reduce<T>(const T*, const Box3&, IBox, double, double*, double*,  \
                                        cudaStream_t);                                          \
  template cudaError_t launch_pack<T>(const T*, const Box3&, T*, cudaStream_t);                 \
  template cudaError_t launch_unpack<T>(const T*, T*, const Box3&, cudaStream_t);
LBX_INST(double)
LBX_INST(float)
#undef LBX_INST

}  // namespace lbx
