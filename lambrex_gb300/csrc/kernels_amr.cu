// kernels_amr.cu -- coarse/fine coupling kernels.
//
// Three schemes share these files.  The reference-faithful one restates the
// Rohde cycle of src/AmrSim.cpp:430-631 as separate FP64 passes over
// ghost-cell boxes (fill patch, collide, stream, zero invalid, sum from fine).
// The conservative one is the library's volumetric scheme: the coarse
// post-collision populations that head into the patch are exploded onto the
// fine ghost shell (constant over the coarse step, so no time interpolation
// is needed), the fine level sub-cycles twice, and every population that left
// the patch is coalesced back with volume weight 1/8; total mass is conserved
// to round-off.  The rescaled one keeps the covered coarse cells active,
// refills the fine ghost shell before every sub-step from the parents
// interpolated in time, with the non-equilibrium part rescaled between the
// levels, and restricts the covered cells after the two sub-steps.
#include "cells.cuh"
#include "faithful.cuh"

namespace lbx {

namespace {

// storage coordinates of a grown box: (sx, sy, sz) in [0, n + 2g).  Storage
// rows (n + 4 cells) are never a multiple of a warp, so each x-y plane is
// flattened over blocks of `threads` (grid.x) and z is grid.y (grown_launch);
// one 32-bit division per thread recovers (sx, sy).
struct GIdx {
  int x, y, z;
};
__device__ __forceinline__ bool grown_index(const Box3& b, GIdx& s) {
  const int SX = b.n[0] + 2 * b.g;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= SX * (b.n[1] + 2 * b.g)) return false;
  s.y = t / SX;
  s.x = t - s.y * SX;
  s.z = blockIdx.y;
  return true;
}
inline RowLaunch grown_launch(const Box3& b, int threads) {
  const int plane = (b.n[0] + 2 * b.g) * (b.n[1] + 2 * b.g);
  return RowLaunch{dim3((unsigned)((plane + threads - 1) / threads), (unsigned)(b.n[2] + 2 * b.g), 1),
                   dim3((unsigned)threads, 1, 1)};
}
// ------------------------------------------------------------------ conservative

template <typename T, bool PAIRED>
__global__ void k_explode(const T* __restrict__ coarse, T* __restrict__ fine, Coupling c, T om_s,
                          T om_b, T rho0, DfRates r) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int s[3];
  if (t >= ghost_cells_of(c.fb) || !ghost_coords(c.fb, (int)t, s)) return;
  cell_explode<T, PAIRED>(coarse, fine, c, s[0], s[1], s[2], om_s, om_b, rho0, r);
}

template <typename T, bool COVER, bool PAIRED>
__global__ void k_step_patch(const T* __restrict__ fin, T* __restrict__ fout, Box3 b, IBox cov,
                             T om_s, T om_b, T rho0, DfRates r) {
  GIdx s;
  if (!grown_index(b, s)) return;
  cell_step_patch<T, COVER, PAIRED>(fin, fout, b, cov, s.x, s.y, s.z, om_s, om_b, rho0, r);
}

template <typename T>
__global__ void k_coalesce(const T* __restrict__ fine, T* __restrict__ coarse, Coupling c, T rho0) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;  // (ring cell, q)
  const long long cell = t / NV;
  const int q = (int)(t - cell * NV);
  int r[3];
  if (cell >= ring_cells_of(c) || !ring_coords(c, (int)cell, r)) return;
  cell_coalesce_q<T>(fine, coarse, c, r[0], r[1], r[2], q, rho0);
}

template <typename T>
__global__ void k_restrict(const T* __restrict__ fine, T* __restrict__ coarse, Coupling c) {
  const int ex = c.fb.n[0] / 2, ey = c.fb.n[1] / 2, ez = c.fb.n[2] / 2;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)ex * ey * ez) return;
  const int rx = (int)(t % ex), ry = (int)((t / ex) % ey), rz = (int)(t / ((long long)ex * ey));
  cell_restrict<T>(fine, coarse, c, rx, ry, rz);
}

template <typename T, bool PAIRED>
__global__ void k_explode_resc(const T* __restrict__ cprev, const T* __restrict__ cnow,
                               T* __restrict__ fine, Coupling c, T om_s, T om_b, T rho0, T wp, T wn,
                               DfRates r) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int s[3];
  if (t >= ghost_cells_of(c.fb) || !ghost_coords(c.fb, (int)t, s)) return;
  cell_explode_resc<T, PAIRED>(cprev, cnow, fine, c, s[0], s[1], s[2], om_s, om_b, rho0, wp, wn, r);
}

template <typename T, bool PAIRED>
__global__ void k_restrict_resc(const T* __restrict__ fine, T* __restrict__ coarse, Coupling c,
                                T om_s, T om_b, T rho0, DfRates r) {
  const int ex = c.fb.n[0] / 2, ey = c.fb.n[1] / 2, ez = c.fb.n[2] / 2;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)ex * ey * ez) return;
  const int rx = (int)(t % ex), ry = (int)((t / ex) % ey), rz = (int)(t / ((long long)ex * ey));
  cell_restrict_resc<T, PAIRED>(fine, coarse, c, rx, ry, rz, om_s, om_b, rho0, r);
}

template <typename T>
__global__ void k_fill_from_coarse(const T* __restrict__ coarse, T* __restrict__ fine, Coupling c) {
  GIdx s;
  if (!grown_index(c.fb, s)) return;
  cell_fill_from_coarse<T>(coarse, fine, c, s.x, s.y, s.z);
}

// ------------------------------------------------------------------ faithful (FP64)

__global__ void k_f_fill_single(const double* __restrict__ src, double* __restrict__ dst, Box3 b) {
  GIdx s;
  if (!grown_index(b, s)) return;
  f_cell_fill_single(src, dst, b, s.x, s.y, s.z);
}

__global__ void k_f_fill_two(const double* __restrict__ fnow, double* __restrict__ dst,
                             const double* __restrict__ cnow, Coupling c, int fdx, int fdy,
                             int fdz) {
  GIdx s;
  if (!grown_index(c.fb, s)) return;
  f_cell_fill_two(fnow, dst, cnow, c, fdx, fdy, fdz, s.x, s.y, s.z);
}

__global__ void k_f_zero_ring0(double* __restrict__ f, Box3 b) {
  GIdx s;
  if (!grown_index(b, s)) return;
  f_cell_zero_ring0(f, b, s.x, s.y, s.z);
}

template <bool PAIRED>
__global__ void k_f_collide(double* __restrict__ f, Box3 b, IBox cov, double om_s, double om_b,
                            DfRates r) {
  int x, y, z;
  row_xyz(x, y, z);
  if (x >= b.n[0] || y >= b.n[1]) return;
  f_cell_collide<PAIRED>(f, b, cov, x, y, z, om_s, om_b, r);
}

__global__ void k_f_stream(const double* __restrict__ src, double* __restrict__ dst, Box3 b) {
  GIdx s;
  if (!grown_index(b, s)) return;
  f_cell_stream(src, dst, b, s.x, s.y, s.z);
}

__global__ void k_f_fill_boundary(double* __restrict__ f, Box3 b) {
  GIdx s;
  if (!grown_index(b, s)) return;
  f_cell_fill_boundary(f, b, s.x, s.y, s.z);
}

__global__ void k_f_zero_invalid(double* __restrict__ f, Box3 b) {
  GIdx s;
  if (!grown_index(b, s)) return;
  f_cell_zero_invalid(f, b, s.x, s.y, s.z);
}

__global__ void k_f_sum_from_fine(const double* __restrict__ fnow, double* __restrict__ cnext,
                                  Coupling c) {
  // coarse cells of coarsen(fine valid) grown by one
  const int ex = c.fb.n[0] / 2 + 2, ey = c.fb.n[1] / 2 + 2, ez = c.fb.n[2] / 2 + 2;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)ex * ey * ez) return;
  const int rx = (int)(t % ex), ry = (int)((t / ex) % ey), rz = (int)(t / ((long long)ex * ey));
  f_cell_sum_from_fine(fnow, cnext, c, rx, ry, rz);
}

inline unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }
// cells of coarsen(patch) grown by one (interior and ring)
inline long long grown_coarse_cells(const Box3& fb) {
  return (long long)(fb.n[0] / 2 + 2) * (fb.n[1] / 2 + 2) * (fb.n[2] / 2 + 2);
}

}  // namespace

template <typename T>
cudaError_t launch_explode(const T* coarse, T* fine, const Coupling& c, double om_s, double om_b,
                           double rho0, cudaStream_t st, bool paired) {
  const unsigned grid = blocks_for(ghost_cells_of(c.fb), 128);
  if constexpr (sizeof(T) == 8) {
    if (paired) {
      k_explode<double, true><<<grid, 128, 0, st>>>(coarse, fine, c, om_s, om_b, 0.0,
                                                    df_rates(om_s, om_b));
      return cudaGetLastError();
    }
  }
  k_explode<T, false><<<grid, 128, 0, st>>>(coarse, fine, c, (T)om_s, (T)om_b, (T)rho0, DfRates{});
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_step_patch(const T* fin, T* fout, const Box3& b, IBox covered, double om_s,
                              double om_b, double rho0, cudaStream_t st, bool paired) {
  const bool cov = covered.hi[0] >= covered.lo[0] && covered.hi[1] >= covered.lo[1] &&
                   covered.hi[2] >= covered.lo[2];
  const RowLaunch rl = grown_launch(b, 128);
  if constexpr (sizeof(T) == 8) {
    if (paired) {
      const DfRates r = df_rates(om_s, om_b);
      if (cov)
        k_step_patch<double, true, true><<<rl.grid, rl.block, 0, st>>>(fin, fout, b, covered, om_s, om_b,
                                                               0.0, r);
      else
        k_step_patch<double, false, true><<<rl.grid, rl.block, 0, st>>>(fin, fout, b, covered, om_s, om_b,
                                                                0.0, r);
      return cudaGetLastError();
    }
  }
  if (cov)
    k_step_patch<T, true, false><<<rl.grid, rl.block, 0, st>>>(fin, fout, b, covered, (T)om_s, (T)om_b,
                                                       (T)rho0, DfRates{});
  else
    k_step_patch<T, false, false><<<rl.grid, rl.block, 0, st>>>(fin, fout, b, covered, (T)om_s, (T)om_b,
                                                        (T)rho0, DfRates{});
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_coalesce(const T* fine, T* coarse, const Coupling& c, double rho0,
                            cudaStream_t st) {
  k_coalesce<T><<<blocks_for(ring_cells_of(c) * NV, 128), 128, 0, st>>>(fine, coarse, c, (T)rho0);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_restrict(const T* fine, T* coarse, const Coupling& c, cudaStream_t st) {
  const long long n = (long long)(c.fb.n[0] / 2) * (c.fb.n[1] / 2) * (c.fb.n[2] / 2);
  k_restrict<T><<<blocks_for(n, 128), 128, 0, st>>>(fine, coarse, c);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_explode_resc(const T* cprev, const T* cnow, T* fine, const Coupling& c,
                                double om_s, double om_b, double rho0, double wp, double wn,
                                cudaStream_t st, bool paired) {
  const unsigned grid = blocks_for(ghost_cells_of(c.fb), 128);
  if constexpr (sizeof(T) == 8) {
    if (paired) {
      k_explode_resc<double, true><<<grid, 128, 0, st>>>(cprev, cnow, fine, c, om_s, om_b, 0.0, wp,
                                                         wn, df_rates(om_s, om_b));
      return cudaGetLastError();
    }
  }
  k_explode_resc<T, false><<<grid, 128, 0, st>>>(cprev, cnow, fine, c, (T)om_s, (T)om_b, (T)rho0,
                                                 (T)wp, (T)wn, DfRates{});
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_restrict_resc(const T* fine, T* coarse, const Coupling& c, double om_s,
                                 double om_b, double rho0, cudaStream_t st, bool paired) {
  const long long n = (long long)(c.fb.n[0] / 2) * (c.fb.n[1] / 2) * (c.fb.n[2] / 2);
  if constexpr (sizeof(T) == 8) {
    if (paired) {
      k_restrict_resc<double, true><<<blocks_for(n, 128), 128, 0, st>>>(fine, coarse, c, om_s, om_b,
                                                                       0.0, df_rates(om_s, om_b));
      return cudaGetLastError();
    }
  }
  k_restrict_resc<T, false><<<blocks_for(n, 128), 128, 0, st>>>(fine, coarse, c, (T)om_s, (T)om_b,
                                                               (T)rho0, DfRates{});
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_fill_from_coarse(const T* coarse, T* fine, const Coupling& c, cudaStream_t st) {
  const RowLaunch rl = grown_launch(c.fb, 128);
  k_fill_from_coarse<T><<<rl.grid, rl.block, 0, st>>>(coarse, fine, c);
  return cudaGetLastError();
}

#define LBX_INST(T)                                                                            \
  template cudaError_t launch_explode<T>(const T*, T*, const Coupling&, double, double, double, \
                                         cudaStream_t, bool);                                  \
  template cudaError_t launch_step_patch<T>(const T*, T*, const Box3&, IBox, double, double,   \
                                            double, cudaStream_t, bool);                       \
  template cudaError_t launch_coalesce<T>(const T*, T*, const Coupling&, double, cudaStream_t); \
  template cudaError_t launch_restrict<T>(const T*, T*, const Coupling&, cudaStream_t);        \
  template cudaError_t launch_fill_from_coarse<T>(const T*, T*, const Coupling&, cudaStream_t); \
  template cudaError_t launch_explode_resc<T>(const T*, const T*, T*, const Coupling&, double,   \
                                              double, double, double, double, cudaStream_t,     \
                                              bool);                                            \
  template cudaError_t launch_restrict_resc<T>(const T*, T*, const Coupling&, double, double,   \
                                               double, cudaStream_t, bool);
LBX_INST(double)
LBX_INST(float)
#undef LBX_INST

cudaError_t launch_f_fill_single(const double* src, double* dst, const Box3& b, cudaStream_t st) {
  const RowLaunch rl = grown_launch(b, 128);
  k_f_fill_single<<<rl.grid, rl.block, 0, st>>>(src, dst, b);
  return cudaGetLastError();
}
cudaError_t launch_f_fill_two(const double* fine_now, double* dst, const double* coarse_now,
                              const Coupling& c, const int* fdom, cudaStream_t st) {
  const RowLaunch rl = grown_launch(c.fb, 128);
  k_f_fill_two<<<rl.grid, rl.block, 0, st>>>(fine_now, dst, coarse_now, c, fdom[0],
                                                         fdom[1], fdom[2]);
  return cudaGetLastError();
}
cudaError_t launch_f_zero_ring0(double* f, const Box3& b, cudaStream_t st) {
  const RowLaunch rl = grown_launch(b, 128);
  k_f_zero_ring0<<<rl.grid, rl.block, 0, st>>>(f, b);
  return cudaGetLastError();
}
cudaError_t launch_f_collide(double* f, const Box3& b, IBox covered, double om_s, double om_b,
                             cudaStream_t st, bool paired) {
  const RowLaunch rl = row_launch(b.n[0], b.n[1], b.n[2], 128);
  if (paired)
    k_f_collide<true><<<rl.grid, rl.block, 0, st>>>(f, b, covered, om_s, om_b, df_rates(om_s, om_b));
  else
    k_f_collide<false><<<rl.grid, rl.block, 0, st>>>(f, b, covered, om_s, om_b, DfRates{});
  return cudaGetLastError();
}
cudaError_t launch_f_stream(const double* src, double* dst, const Box3& b, cudaStream_t st) {
  const RowLaunch rl = grown_launch(b, 128);
  k_f_stream<<<rl.grid, rl.block, 0, st>>>(src, dst, b);
  return cudaGetLastError();
}
cudaError_t launch_f_fill_boundary(double* f, const Box3& b, cudaStream_t st) {
  const RowLaunch rl = grown_launch(b, 128);
  k_f_fill_boundary<<<rl.grid, rl.block, 0, st>>>(f, b);
  return cudaGetLastError();
}
cudaError_t launch_f_zero_invalid(double* f, const Box3& b, cudaStream_t st) {
  const RowLaunch rl = grown_launch(b, 128);
  k_f_zero_invalid<<<rl.grid, rl.block, 0, st>>>(f, b);
  return cudaGetLastError();
}
cudaError_t launch_f_sum_from_fine(const double* fine_now, double* coarse_next, const Coupling& c,
                                   cudaStream_t st) {
  k_f_sum_from_fine<<<blocks_for(grown_coarse_cells(c.fb), 128), 128, 0, st>>>(fine_now, coarse_next, c);
  return cudaGetLastError();
}

}  // namespace lbx
