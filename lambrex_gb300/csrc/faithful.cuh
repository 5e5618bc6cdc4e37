// faithful.cuh -- per-cell bodies of the reference-faithful Rohde cycle
// (src/AmrSim.cpp:430-631), FP64: the passes of the cycle over a level's
// grown box (fill patch, masked collide, stream into a fresh buffer, zero the
// invalid ghost components, periodic ghost refresh) and the fine-to-coarse
// sum.  The kernels in kernels_amr.cu call one of these per thread; a host
// build runs them cell by cell in the tests.
#pragma once
#include "cells.cuh"

namespace lbx {

// FillPatchSingleLevel (src/AmrSim.cpp:359-372): storage cell (sx,sy,sz) of
// the grown box <- its periodic image in the valid region
__host__ __device__ __forceinline__ void f_cell_fill_single(const double* __restrict__ src,
                                                           double* __restrict__ dst, const Box3& b,
                                                           int sx, int sy, int sz) {
  const int g = b.g;
  const long long d = sidx(b, sx, sy, sz);
  const long long c = b.at(wrapi(sx - g, b.n[0]), wrapi(sy - g, b.n[1]), wrapi(sz - g, b.n[2]));
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(dst, q * b.sq + d, b, ld_pop(src, q * b.sq + c, b));
}

// FillPatchTwoLevels + PCInterp (src/AmrSim.cpp:373-388), single time level:
// fine now (or its periodic image over the fine domain fdx x fdy x fdz) where
// it exists, else the parent coarse cell of coarse now
__host__ __device__ __forceinline__ void f_cell_fill_two(const double* __restrict__ fnow,
                                                        double* __restrict__ dst,
                                                        const double* __restrict__ cnow,
                                                        const Coupling& c, int fdx, int fdy,
                                                        int fdz, int sx, int sy, int sz) {
  const int g = c.fb.g;
  const int X = c.flo[0] + sx - g, Y = c.flo[1] + sy - g, Z = c.flo[2] + sz - g;  // global
  const long long d = sidx(c.fb, sx, sy, sz);
  const int wx = wrapi(X, fdx) - c.flo[0], wy = wrapi(Y, fdy) - c.flo[1], wz = wrapi(Z, fdz) - c.flo[2];
  if (in_valid(c.fb, wx, wy, wz)) {
    const long long f = c.fb.at(wx, wy, wz);
#pragma unroll
    for (int q = 0; q < NV; ++q)
      st_pop(dst, q * c.fb.sq + d, c.fb, ld_pop(fnow, q * c.fb.sq + f, c.fb));
    return;
  }
  const int px = wrapi(floordiv2(X), c.cdom[0]) - c.clo[0];
  const int py = wrapi(floordiv2(Y), c.cdom[1]) - c.clo[1];
  const int pz = wrapi(floordiv2(Z), c.cdom[2]) - c.clo[2];
  if (!in_valid(c.cb, px, py, pz)) return;
  const long long cc = c.cb.at(px, py, pz);
#pragma unroll
  for (int q = 0; q < NV; ++q)
    st_pop(dst, q * c.fb.sq + d, c.fb, ld_pop(cnow, q * c.cb.sq + cc, c.cb));
}

// the outermost ghost layer, component 0 only (src/AmrSim.cpp:479-481)
__host__ __device__ __forceinline__ void f_cell_zero_ring0(double* __restrict__ f, const Box3& b,
                                                          int sx, int sy, int sz) {
  const int SX = b.n[0] + 2 * b.g, SY = b.n[1] + 2 * b.g, SZ = b.n[2] + 2 * b.g;
  if (sx == 0 || sy == 0 || sz == 0 || sx == SX - 1 || sy == SY - 1 || sz == SZ - 1)
    st_pop(f, sidx(b, sx, sy, sz), b, 0.0);
}

// Collide of valid cell (x,y,z) in place, zero where the mask marks it
// covered (CoarseCollide / FineCollide, src/AmrSim.cpp:487-590)
template <bool PAIRED>
__host__ __device__ __forceinline__ void f_cell_collide(double* __restrict__ f, const Box3& b,
                                                       const IBox& cov, int x, int y, int z,
                                                       double om_s, double om_b,
                                                       const DfRates& r) {
  const long long c = b.at(x, y, z);
  double v[NV];
  if (cov.contains(x, y, z)) {
#pragma unroll
    for (int q = 0; q < NV; ++q) st_pop(f, q * b.sq + c, b, 0.0);
    return;
  }
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = ld_pop_rw(f, q * b.sq + c, b);
  collide_cell<double, PAIRED>(v, om_s, om_b, 0.0, r);
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(f, q * b.sq + c, b, v[q]);
}

// Stream (src/AmrSim.cpp:109-122, include/component.h:22-29): pull over the
// valid cells and one ghost ring into a fresh buffer
__host__ __device__ __forceinline__ void f_cell_stream(const double* __restrict__ src,
                                                      double* __restrict__ dst, const Box3& b,
                                                      int sx, int sy, int sz) {
  const int g = b.g;
  const int vx = sx - g, vy = sy - g, vz = sz - g;
  if (vx < -1 || vx > b.n[0] || vy < -1 || vy > b.n[1] || vz < -1 || vz > b.n[2]) return;
  const long long d = sidx(b, sx, sy, sz);
#pragma unroll
  for (int q = 0; q < NV; ++q)
    st_pop(dst, q * b.sq + d, b, ld_pop(src, q * b.sq + sidx(b, sx - CX(q), sy - CY(q), sz - CZ(q)), b));
}

// FillBoundary(periodicity) of level 0 (src/AmrSim.cpp:19-23, 132): ghost
// cell <- its periodic image
__host__ __device__ __forceinline__ void f_cell_fill_boundary(double* __restrict__ f, const Box3& b,
                                                             int sx, int sy, int sz) {
  const int g = b.g;
  const int vx = sx - g, vy = sy - g, vz = sz - g;
  if (in_valid(b, vx, vy, vz)) return;
  const long long d = sidx(b, sx, sy, sz);
  const long long c = b.at(wrapi(vx, b.n[0]), wrapi(vy, b.n[1]), wrapi(vz, b.n[2]));
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(f, q * b.sq + d, b, ld_pop_rw(f, q * b.sq + c, b));
}

// ZeroInvalidComponents (src/AmrSim.cpp:604-617): a ghost cell keeps
// component q only if pos - 2 c_q is valid
__host__ __device__ __forceinline__ void f_cell_zero_invalid(double* __restrict__ f, const Box3& b,
                                                            int sx, int sy, int sz) {
  const int g = b.g;
  const int vx = sx - g, vy = sy - g, vz = sz - g;
  if (in_valid(b, vx, vy, vz)) return;
  const long long d = sidx(b, sx, sy, sz);
#pragma unroll
  for (int q = 0; q < NV; ++q)
    if (!in_valid(b, vx - 2 * CX(q), vy - 2 * CY(q), vz - 2 * CZ(q))) st_pop(f, q * b.sq + d, b, 0.0);
}

// element i of a population store += v (atomic on the device: several
// periodic images may add into one cell)
__host__ __device__ __forceinline__ void f_add_pop(double* p, long long i, const Box3& b, double v) {
  if (!idx_ok(i, NV * b.sq)) return;
#ifdef __CUDA_ARCH__
  atomicAdd(p + i, v);
#else
  p[i] += v;
#endif
}

// SumFromFine (src/AmrSim.cpp:592-602, sum_fine_to_coarse): the mean of the
// 2^3 fine cells under coarse cell (rx,ry,rz) of coarsen(fine valid) grown by
// one, added to every periodic image of that cell on the coarse level
__host__ __device__ __forceinline__ void f_cell_sum_from_fine(const double* __restrict__ fnow,
                                                             double* __restrict__ cnext,
                                                             const Coupling& c, int rx, int ry,
                                                             int rz) {
  const int cgx = c.flo[0] / 2 + rx - 1, cgy = c.flo[1] / 2 + ry - 1, cgz = c.flo[2] / 2 + rz - 1;
  const int fx0 = 2 * cgx - c.flo[0], fy0 = 2 * cgy - c.flo[1], fz0 = 2 * cgz - c.flo[2];
  for (int q = 0; q < NV; ++q) {
    double s = 0.0;
    for (int kr = 0; kr < 2; ++kr)
      for (int jr = 0; jr < 2; ++jr)
        for (int ir = 0; ir < 2; ++ir)
          s += ld_pop(fnow, q * c.fb.sq + c.fb.at(fx0 + ir, fy0 + jr, fz0 + kr), c.fb);
    const double avg = 0.125 * s;
    for (int sz = -1; sz <= 1; ++sz)
      for (int sy = -1; sy <= 1; ++sy)
        for (int sx = -1; sx <= 1; ++sx) {
          const int a = cgx + sx * c.cdom[0] - c.clo[0];
          const int bb = cgy + sy * c.cdom[1] - c.clo[1];
          const int e = cgz + sz * c.cdom[2] - c.clo[2];
          if (!in_valid(c.cb, a, bb, e)) continue;
          f_add_pop(cnext, q * c.cb.sq + c.cb.at(a, bb, e), c.cb, avg);
        }
  }
}

}  // namespace lbx
