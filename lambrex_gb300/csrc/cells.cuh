// cells.cuh -- per-cell bodies shared by the single-simulation kernels and
// the batch engine: one fused collide + push-stream update of a periodic
// box or of an AMR patch, and the three coarse/fine coupling operations of
// the conservative scheme (explode, coalesce, restrict).
#pragma once
#include "checked.cuh"
#include "df32.cuh"
#include "kernels.cuh"

namespace lbx {

// value of an empty population (f = 0) in the storage variable
template <typename T>
__host__ __device__ __forceinline__ T zero_pop(int q, T rho0) {
  return rho0 == T(0) ? T(0) : T(-W(q)) * rho0;
}
// collision of one cell: native in T, or for an FP64 store in paired FP32
// arithmetic with its twin operations packed (df32.cuh; rho0 is 0 there)
template <typename T, bool PAIRED>
__host__ __device__ __forceinline__ void collide_cell(T* f, T om_s, T om_b, T rho0, const DfRates& r) {
  if constexpr (PAIRED)
    collide_f64_via_df_w(f, r);
  else
    collide<T>(f, om_s, om_b, rho0);
}
__host__ __device__ __forceinline__ int floordiv2(int x) { return x >= 0 ? x / 2 : -((-x + 1) / 2); }
__host__ __device__ __forceinline__ int wrapi(int x, int n) {
  int r = x % n;
  return r < 0 ? r + n : r;
}
__host__ __device__ __forceinline__ long long sidx(const Box3& b, int sx, int sy, int sz) {
  return (long long)sz * b.sxy + (long long)sy * b.sx + sx;
}
// Index arithmetic of a store in type I: long long for the single-simulation
// kernels (stores up to 15 x 2^31 elements), int for the batch engine, whose
// boxes stay below 2^23 cells so that every element index fits in 32 bits
// and the per-thread offsets take half the registers.
template <typename I>
__host__ __device__ __forceinline__ I sidx_i(const Box3& b, int sx, int sy, int sz) {
  return (I)sz * (I)b.sxy + (I)sy * (I)b.sx + (I)sx;
}
__host__ __device__ __forceinline__ bool in_valid(const Box3& b, int vx, int vy, int vz) {
  return vx >= 0 && vx < b.n[0] && vy >= 0 && vy < b.n[1] && vz >= 0 && vz < b.n[2];
}

// push post-collision populations of valid cell (x,y,z) to x + c_q with
// periodic wrap over the valid region
template <typename T, typename I = long long>
__host__ __device__ __forceinline__ void push_periodic(T* __restrict__ fout, const Box3& b, int x, int y,
                                              int z, const T* f) {
  const int xm = x == 0 ? b.n[0] - 1 : x - 1, xp = x == b.n[0] - 1 ? 0 : x + 1;
  const int ym = y == 0 ? b.n[1] - 1 : y - 1, yp = y == b.n[1] - 1 ? 0 : y + 1;
  const int zm = z == 0 ? b.n[2] - 1 : z - 1, zp = z == b.n[2] - 1 ? 0 : z + 1;
  const I sx = (I)b.sx, sxy = (I)b.sxy, sq = (I)b.sq;
  const I ox[3] = {(I)(xm + b.g), (I)(x + b.g), (I)(xp + b.g)};
  const I oy[3] = {(I)(ym + b.g) * sx, (I)(y + b.g) * sx, (I)(yp + b.g) * sx};
  const I oz[3] = {(I)(zm + b.g) * sxy, (I)(z + b.g) * sxy, (I)(zp + b.g) * sxy};
#pragma unroll
  for (int q = 0; q < NV; ++q)
    st_pop(fout, (I)q * sq + oz[CZ(q) + 1] + oy[CY(q) + 1] + ox[CX(q) + 1], b, f[q]);
}

// Covered cells (under a finer patch) take no part in the dynamics: their
// values are replaced by the restriction before any readout.  They load
// nothing.  Those on the covered box's boundary push empty populations, so
// that the uncovered ring cells next to them receive zeros, to which the
// coalescence adds the fine level's contributions; those strictly inside
// write nothing, since every D3Q15 neighbour of theirs is covered.
__host__ __device__ __forceinline__ bool covered_inside(const IBox& c, int x, int y, int z) {
  return x > c.lo[0] && x < c.hi[0] && y > c.lo[1] && y < c.hi[1] && z > c.lo[2] && z < c.hi[2];
}

// Periodic box, valid cell (x,y,z): collide (or emit zeros if covered) and
// push f(x, q) to x + c_q with wrap (src/AmrSim.cpp:25-135 as a push).
template <typename T, bool COVER, bool PAIRED = false, typename I = long long>
__host__ __device__ __forceinline__ void cell_step_periodic(const T* __restrict__ fin, T* __restrict__ fout,
                                                   const Box3& b, const IBox& cov, int x, int y,
                                                   int z, T om_s, T om_b, T rho0,
                                                   const DfRates& r = DfRates{}) {
  T f[NV];
  if (COVER && cov.contains(x, y, z)) {
    if (covered_inside(cov, x, y, z)) return;
#pragma unroll
    for (int q = 0; q < NV; ++q) f[q] = zero_pop<T>(q, rho0);
  } else {
    const I c = sidx_i<I>(b, x + b.g, y + b.g, z + b.g), sq = (I)b.sq;
#pragma unroll
    for (int q = 0; q < NV; ++q) f[q] = ld_pop(fin, (I)q * sq + c, b);
    collide_cell<T, PAIRED>(f, om_s, om_b, rho0, r);
  }
  push_periodic<T, I>(fout, b, x, y, z, f);
}

// Pull form.  The store holds Q_n = C(R_{n-1}), the post-collision
// populations of the previous step, so that the streamed state is
// R_n(x, q) = Q_n(x - c_q, q).  One step gathers R_n (loads shifted by at
// most one element, merged in L1/L2), collides it and writes
// Q_{n+1} = C(R_n) aligned: Q_{n+1} = C(S(Q_n)) is the reference's
// R_{n+1} = S(C(R_n)) one stream behind.  Readouts gather R_n from Q_n;
// entering the form from R is the inverse shift Q(x, q) = R(x + c_q, q).
// SIGN = +1 gathers from x - c_q (S), SIGN = -1 from x + c_q (inverse of S).
template <typename T, int SIGN = 1, typename I = long long>
__host__ __device__ __forceinline__ void gather_periodic(const T* __restrict__ fin, const Box3& b, int x,
                                                int y, int z, T* f) {
  const int xm = x == 0 ? b.n[0] - 1 : x - 1, xp = x == b.n[0] - 1 ? 0 : x + 1;
  const int ym = y == 0 ? b.n[1] - 1 : y - 1, yp = y == b.n[1] - 1 ? 0 : y + 1;
  const int zm = z == 0 ? b.n[2] - 1 : z - 1, zp = z == b.n[2] - 1 ? 0 : z + 1;
  const I sx = (I)b.sx, sxy = (I)b.sxy, sq = (I)b.sq;
  // source of population q is x - SIGN c_q: index [c + 1] selects it
  const I ox[3] = {(I)((SIGN > 0 ? xp : xm) + b.g), (I)(x + b.g), (I)((SIGN > 0 ? xm : xp) + b.g)};
  const I oy[3] = {(I)((SIGN > 0 ? yp : ym) + b.g) * sx, (I)(y + b.g) * sx,
                   (I)((SIGN > 0 ? ym : yp) + b.g) * sx};
  const I oz[3] = {(I)((SIGN > 0 ? zp : zm) + b.g) * sxy, (I)(z + b.g) * sxy,
                   (I)((SIGN > 0 ? zm : zp) + b.g) * sxy};
#pragma unroll
  for (int q = 0; q < NV; ++q)
    f[q] = ld_pop(fin, (I)q * sq + oz[CZ(q) + 1] + oy[CY(q) + 1] + ox[CX(q) + 1], b);
}

template <typename T, bool PAIRED, typename I = long long>
__host__ __device__ __forceinline__ void cell_step_pull(const T* __restrict__ fin, T* __restrict__ fout,
                                               const Box3& b, int x, int y, int z, T om_s, T om_b,
                                               T rho0, const DfRates& r) {
  T f[NV];
  gather_periodic<T, 1, I>(fin, b, x, y, z, f);
  collide_cell<T, PAIRED>(f, om_s, om_b, rho0, r);
  const I c = sidx_i<I>(b, x + b.g, y + b.g, z + b.g), sq = (I)b.sq;
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(fout, (I)q * sq + c, b, f[q]);
}

// rho and u of one cell's populations p (src/AmrSim.cpp:957-971) into the
// FP64 fields at cell v of n: moments 0..3 from even/odd pairs, in the
// storage precision (the shifted FP32 values are fluctuations, so FP32 sums
// keep ~1e-10 of rho)
template <typename T>
__host__ __device__ __forceinline__ void store_hydro(const T* p, double rho0, double* __restrict__ rho,
                                                    double* __restrict__ u, long long v,
                                                    long long n) {
  const T s1 = p[1] + p[2], s3 = p[3] + p[4], s5 = p[5] + p[6];
  const T d7 = p[7] - p[14], d8 = p[8] - p[13], d9 = p[9] - p[12], dA = p[10] - p[11];
  const T D = (p[7] + p[14]) + (p[8] + p[13]) + ((p[9] + p[12]) + (p[10] + p[11]));
  const T drho = p[0] + (s1 + s3 + s5) + D;
  const T jx = (p[1] - p[2]) + (d7 + d8) + (d9 + dA);
  const T jy = (p[3] - p[4]) + (d7 + d8) - (d9 + dA);
  const T jz = (p[5] - p[6]) + (d7 - d8) + (d9 - dA);
  const double m = (double)drho + rho0;  // sum_q w_q rho0 = rho0, sum_q c_q w_q = 0
  st_cell(rho, v, n, m);
  if constexpr (sizeof(T) == 4) {
    // the FP32 store's momenta carry FP32 rounding already: an FP32
    // reciprocal adds ~2e-7 relative and keeps the slow FP64 pipe out
    const float inv = 1.0f / (float)m;
    st_cell(u, v, 3 * n, (double)(jx * inv));
    st_cell(u, n + v, 3 * n, (double)(jy * inv));
    st_cell(u, 2 * n + v, 3 * n, (double)(jz * inv));
  } else {
    const double inv = 1.0 / m;
    st_cell(u, v, 3 * n, (double)jx * inv);
    st_cell(u, n + v, 3 * n, (double)jy * inv);
    st_cell(u, 2 * n + v, 3 * n, (double)jz * inv);
  }
}

// CalcHydroVars (src/AmrSim.cpp:938-979) of valid cell (x,y,z): rho and u
// into per-cell FP64 fields in FAB order; GATHER: the store is in the pull
// form and the streamed state is gathered first
template <typename T, bool GATHER>
__host__ __device__ __forceinline__ void cell_hydro(const T* __restrict__ f, const Box3& b,
                                                   double rho0, double* __restrict__ rho,
                                                   double* __restrict__ u, int x, int y, int z) {
  const long long n = (long long)b.n[0] * b.n[1] * b.n[2];
  const long long v = ((long long)z * b.n[1] + y) * b.n[0] + x;
  const long long c = b.at(x, y, z);
  T p[NV];
  if (GATHER) {  // pull-form store: the streamed state is gathered
    gather_periodic<T>(f, b, x, y, z, p);
  } else {
#pragma unroll
    for (int q = 0; q < NV; ++q) p[q] = ld_pop(f, q * b.sq + c, b);
  }
  store_hydro<T>(p, rho0, rho, u, v, n);
}

// The pull-form step with CalcHydroVars as its epilogue: the gathered state
// R_n is the one CalcHydroVars reads, so its rho and u are written (the same
// values as cell_hydro<T, true>) before the collision, and the step writes
// Q_{n+1} as cell_step_pull does.
template <typename T, bool PAIRED, typename I = long long>
__host__ __device__ __forceinline__ void cell_step_pull_hydro(const T* __restrict__ fin,
                                                     T* __restrict__ fout, const Box3& b, int x,
                                                     int y, int z, T om_s, T om_b, T rho0,
                                                     const DfRates& r, double rho0_d,
                                                     double* __restrict__ rho,
                                                     double* __restrict__ u) {
  T f[NV];
  gather_periodic<T, 1, I>(fin, b, x, y, z, f);
  const long long n = (long long)b.n[0] * b.n[1] * b.n[2];
  store_hydro<T>(f, rho0_d, rho, u, ((long long)z * b.n[1] + y) * b.n[0] + x, n);
  collide_cell<T, PAIRED>(f, om_s, om_b, rho0, r);
  const I c = sidx_i<I>(b, x + b.g, y + b.g, z + b.g), sq = (I)b.sq;
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(fout, (I)q * sq + c, b, f[q]);
}

// New fine level, storage cell (sx,sy,sz) of the grown box (ghosts
// included): the populations of its parent coarse cell, through the periodic
// wrap when the parent level is level 0 (MakeNewLevelFromCoarse with PCInterp,
// src/AmrSim.cpp:689-713); cells whose parent is not on the coarse level are
// left as they are.
template <typename T>
__host__ __device__ __forceinline__ void cell_fill_from_coarse(const T* __restrict__ coarse,
                                                             T* __restrict__ fine,
                                                             const Coupling& c, int sx, int sy,
                                                             int sz) {
  const int g = c.fb.g;
  int P[3] = {floordiv2(c.flo[0] + sx - g), floordiv2(c.flo[1] + sy - g),
              floordiv2(c.flo[2] + sz - g)};
  if (c.cper)
    for (int d = 0; d < 3; ++d) P[d] = wrapi(P[d], c.cdom[d]);
  const int px = P[0] - c.clo[0], py = P[1] - c.clo[1], pz = P[2] - c.clo[2];
  if (!in_valid(c.cb, px, py, pz)) return;
  const long long cc = c.cb.at(px, py, pz), fc = sidx(c.fb, sx, sy, sz);
#pragma unroll
  for (int q = 0; q < NV; ++q)
    st_pop(fine, q * c.fb.sq + fc, c.fb, ld_pop(coarse, q * c.cb.sq + cc, c.cb));
}

// AMR patch, storage cell (sx,sy,sz) of the grown box: valid cells collide
// (covered ones emit zeros), ghost cells stream raw, pushes leaving the
// storage are dropped and entries nothing streams into are set empty.
template <typename T, bool COVER, bool PAIRED = false, typename I = long long>
__host__ __device__ __forceinline__ void cell_step_patch(const T* __restrict__ fin, T* __restrict__ fout,
                                                const Box3& b, const IBox& cov, int sx, int sy,
                                                int sz, T om_s, T om_b, T rho0,
                                                const DfRates& r = DfRates{}) {
  const int g = b.g;
  const int vx = sx - g, vy = sy - g, vz = sz - g;
  const I c = sidx_i<I>(b, sx, sy, sz), sq = (I)b.sq, rx = (I)b.sx, rxy = (I)b.sxy;
  T f[NV];
  const bool valid = in_valid(b, vx, vy, vz);
  if (COVER && valid && cov.contains(vx, vy, vz)) {  // see covered_inside
    if (covered_inside(cov, vx, vy, vz)) return;
#pragma unroll
    for (int q = 0; q < NV; ++q) f[q] = zero_pop<T>(q, rho0);
  } else {
#pragma unroll
    for (int q = 0; q < NV; ++q) f[q] = ld_pop(fin, (I)q * sq + c, b);
    if (valid) collide_cell<T, PAIRED>(f, om_s, om_b, rho0, r);
  }
  const int SX = b.n[0] + 2 * g, SY = b.n[1] + 2 * g, SZ = b.n[2] + 2 * g;
  if (sx > 0 && sx < SX - 1 && sy > 0 && sy < SY - 1 && sz > 0 && sz < SZ - 1) {
    // every target lies in the storage and every source too: constant offsets
#pragma unroll
    for (int q = 0; q < NV; ++q)
      st_pop(fout, (I)q * sq + c + (I)CZ(q) * rxy + (I)CY(q) * rx + (I)CX(q), b, f[q]);
    return;
  }
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int tx = sx + CX(q), ty = sy + CY(q), tz = sz + CZ(q);
    if (tx >= 0 && tx < SX && ty >= 0 && ty < SY && tz >= 0 && tz < SZ)
      st_pop(fout, (I)q * sq + sidx_i<I>(b, tx, ty, tz), b, f[q]);
    const int ux = sx - CX(q), uy = sy - CY(q), uz = sz - CZ(q);
    if (!(ux >= 0 && ux < SX && uy >= 0 && uy < SY && uz >= 0 && uz < SZ))
      st_pop(fout, (I)q * sq + c, b, zero_pop<T>(q, rho0));
  }
}

// ---- pull form of the conservative coupling (batch engine) ------------------
// The stores hold Q = C(R) on stepped cells and the raw state on ghost cells;
// a step gathers R(x, q) = Q(x - c_q, q), collides valid cells and stores
// aligned.  Covered cells are not stepped: the boundary ones store empty
// populations, into which the coalescence adds the fine level's outflow
// before the next step gathers them; the inner ones store nothing.
//
// Periodic box (level 0), valid cell (x,y,z).
template <typename T, typename I = long long>
__host__ __device__ __forceinline__ void cell_step_periodic_pull(const T* __restrict__ fin,
                                                                T* __restrict__ fout,
                                                                const Box3& b, const IBox& cov,
                                                                int x, int y, int z, T om_s, T om_b,
                                                                T rho0) {
  if (cov.contains(x, y, z)) {
    if (covered_inside(cov, x, y, z)) return;
    const I c = sidx_i<I>(b, x + b.g, y + b.g, z + b.g), sq = (I)b.sq;
#pragma unroll
    for (int q = 0; q < NV; ++q) st_pop(fout, (I)q * sq + c, b, zero_pop<T>(q, rho0));
    return;
  }
  cell_step_pull<T, false, I>(fin, fout, b, x, y, z, om_s, om_b, rho0, DfRates{});
}

// AMR patch, storage cell (sx,sy,sz) of the grown box: sources outside the
// storage are empty.
template <typename T, typename I = long long>
__host__ __device__ __forceinline__ void cell_step_patch_pull(const T* __restrict__ fin,
                                                             T* __restrict__ fout, const Box3& b,
                                                             const IBox& cov, int sx, int sy,
                                                             int sz, T om_s, T om_b, T rho0) {
  const int g = b.g;
  const int vx = sx - g, vy = sy - g, vz = sz - g;
  const I c = sidx_i<I>(b, sx, sy, sz), sq = (I)b.sq, rx = (I)b.sx, rxy = (I)b.sxy;
  const bool valid = in_valid(b, vx, vy, vz);
  if (valid && cov.contains(vx, vy, vz)) {
    if (covered_inside(cov, vx, vy, vz)) return;
#pragma unroll
    for (int q = 0; q < NV; ++q) st_pop(fout, (I)q * sq + c, b, zero_pop<T>(q, rho0));
    return;
  }
  T f[NV];
  const int SX = b.n[0] + 2 * g, SY = b.n[1] + 2 * g, SZ = b.n[2] + 2 * g;
  if (sx > 0 && sx < SX - 1 && sy > 0 && sy < SY - 1 && sz > 0 && sz < SZ - 1) {
#pragma unroll
    for (int q = 0; q < NV; ++q)
      f[q] = ld_pop(fin, (I)q * sq + c - ((I)CZ(q) * rxy + (I)CY(q) * rx + (I)CX(q)), b);
  } else {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const int ux = sx - CX(q), uy = sy - CY(q), uz = sz - CZ(q);
      f[q] = (ux >= 0 && ux < SX && uy >= 0 && uy < SY && uz >= 0 && uz < SZ)
                 ? ld_pop(fin, (I)q * sq + sidx_i<I>(b, ux, uy, uz), b)
                 : zero_pop<T>(q, rho0);
    }
  }
  if (valid) collide_cell<T, false>(f, om_s, om_b, rho0, DfRates{});
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(fout, (I)q * sq + c, b, f[q]);
}

// Into the pull form in place, valid cell (x,y,z) of a periodic box or a
// patch: Q = C(R) on stepped cells, empty populations on covered cells with
// an uncovered neighbour; ghost cells keep their (raw) state.
template <typename T, typename I = long long>
__host__ __device__ __forceinline__ void cell_to_qform(T* __restrict__ f, const Box3& b,
                                                      const IBox& cov, int x, int y, int z, T om_s,
                                                      T om_b, T rho0) {
  const I c = sidx_i<I>(b, x + b.g, y + b.g, z + b.g), sq = (I)b.sq;
  T p[NV];
  if (cov.contains(x, y, z)) {
    if (covered_inside(cov, x, y, z)) return;
#pragma unroll
    for (int q = 0; q < NV; ++q) p[q] = zero_pop<T>(q, rho0);
  } else {
#pragma unroll
    for (int q = 0; q < NV; ++q) p[q] = ld_pop(f, (I)q * sq + c, b);
    collide_cell<T, false>(p, om_s, om_b, rho0, DfRates{});
  }
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(f, (I)q * sq + c, b, p[q]);
}

// Back to the streamed state R = S(Q) at valid cell (x,y,z), gathered from
// the store before the last step (qprev) into `r`: with the periodic wrap on
// a box without ghost cells, from the ghost shell on a patch.
template <typename T, typename I = long long>
__host__ __device__ __forceinline__ void cell_to_rform(const T* __restrict__ qprev, T* __restrict__ r,
                                                      const Box3& b, int x, int y, int z) {
  T p[NV];
  const I c = sidx_i<I>(b, x + b.g, y + b.g, z + b.g), sq = (I)b.sq;
  if (b.g == 0) {
    gather_periodic<T, 1, I>(qprev, b, x, y, z, p);
  } else {
    const I rx = (I)b.sx, rxy = (I)b.sxy;
#pragma unroll
    for (int q = 0; q < NV; ++q)
      p[q] = ld_pop(qprev, (I)q * sq + c - ((I)CZ(q) * rxy + (I)CY(q) * rx + (I)CX(q)), b);
  }
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(r, (I)q * sq + c, b, p[q]);
}

// Explosion onto the fine ghost cell at storage (sx,sy,sz): the parent's
// post-collision populations that will enter the patch within two fine
// sub-steps (x + 2 c_q inside), empty otherwise.  QFORM: the coarse store
// holds post-collision populations already (pull form).
template <typename T, bool PAIRED = false, typename I = long long, bool QFORM = false>
__host__ __device__ __forceinline__ void cell_explode(const T* __restrict__ coarse, T* __restrict__ fine,
                                             const Coupling& c, int sx, int sy, int sz, T om_s,
                                             T om_b, T rho0, const DfRates& r = DfRates{}) {
  const int g = c.fb.g;
  const int vx = sx - g, vy = sy - g, vz = sz - g;
  if (in_valid(c.fb, vx, vy, vz)) return;
  int P[3] = {floordiv2(c.flo[0] + vx), floordiv2(c.flo[1] + vy), floordiv2(c.flo[2] + vz)};
  if (c.cper)
    for (int d = 0; d < 3; ++d) P[d] = wrapi(P[d], c.cdom[d]);
  const I cc = sidx_i<I>(c.cb, P[0] - c.clo[0] + c.cb.g, P[1] - c.clo[1] + c.cb.g,
                         P[2] - c.clo[2] + c.cb.g);
  const I csq = (I)c.cb.sq, fsq = (I)c.fb.sq;
  T f[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) f[q] = ld_pop(coarse, (I)q * csq + cc, c.cb);
  if (!QFORM) collide_cell<T, PAIRED>(f, om_s, om_b, rho0, r);
  const I fc = sidx_i<I>(c.fb, sx, sy, sz);
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const bool in = in_valid(c.fb, vx + 2 * CX(q), vy + 2 * CY(q), vz + 2 * CZ(q));
    st_pop(fine, (I)q * fsq + fc, c.fb, in ? f[q] : zero_pop<T>(q, rho0));
  }
}

// ---- rescaled coupling ------------------------------------------------------
// Covered coarse cells stay active; the fine ghost shell is refilled before
// every fine sub-step and the covered cells are restricted after the two.
// Rescaling the non-equilibrium moments by s is the collision at rate 1 - s,
// so both transfers are collisions at rates the host derives per coupling.
//
// Fine ghost cell at storage (sx,sy,sz) <- its parent's populations collided
// at the explosion rates (the fine post-collision state, non-equilibrium
// part rescaled to the fine level), interpolated in time: wp times the
// parent at the start of the coarse step (cprev) plus wn times the parent at
// its end (cnow; not read when wn == 0).
template <typename T, bool PAIRED = false, typename I = long long>
__host__ __device__ __forceinline__ void cell_explode_resc(const T* __restrict__ cprev,
                                                  const T* __restrict__ cnow, T* __restrict__ fine,
                                                  const Coupling& c, int sx, int sy, int sz,
                                                  T om_s, T om_b, T rho0, T wp, T wn,
                                                  const DfRates& r = DfRates{}) {
  const int g = c.fb.g;
  const int vx = sx - g, vy = sy - g, vz = sz - g;
  if (in_valid(c.fb, vx, vy, vz)) return;
  int P[3] = {floordiv2(c.flo[0] + vx), floordiv2(c.flo[1] + vy), floordiv2(c.flo[2] + vz)};
  if (c.cper)
    for (int d = 0; d < 3; ++d) P[d] = wrapi(P[d], c.cdom[d]);
  const I cc = sidx_i<I>(c.cb, P[0] - c.clo[0] + c.cb.g, P[1] - c.clo[1] + c.cb.g,
                         P[2] - c.clo[2] + c.cb.g);
  const I csq = (I)c.cb.sq, fsq = (I)c.fb.sq;
  T a[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) a[q] = ld_pop(cprev, (I)q * csq + cc, c.cb);
  collide_cell<T, PAIRED>(a, om_s, om_b, rho0, r);
  if (wn != T(0)) {
    T b[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) b[q] = ld_pop(cnow, (I)q * csq + cc, c.cb);
    collide_cell<T, PAIRED>(b, om_s, om_b, rho0, r);
#pragma unroll
    for (int q = 0; q < NV; ++q) a[q] = wp * a[q] + wn * b[q];
  }
  const I fc = sidx_i<I>(c.fb, sx, sy, sz);
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(fine, (I)q * fsq + fc, c.fb, a[q]);
}

// covered coarse cell (rx,ry,rz) of coarsen(patch) <- the mean of its
// children collided at the restriction rates (the inverse rescaling)
template <typename T, bool PAIRED = false, typename I = long long>
__host__ __device__ __forceinline__ void cell_restrict_resc(const T* __restrict__ fine,
                                                   T* __restrict__ coarse, const Coupling& c,
                                                   int rx, int ry, int rz, T om_s, T om_b,
                                                   T rho0, const DfRates& r = DfRates{}) {
  int P[3] = {c.flo[0] / 2 + rx, c.flo[1] / 2 + ry, c.flo[2] / 2 + rz};
  if (c.cper)
    for (int d = 0; d < 3; ++d) P[d] = wrapi(P[d], c.cdom[d]);
  const I cc = sidx_i<I>(c.cb, P[0] - c.clo[0] + c.cb.g, P[1] - c.clo[1] + c.cb.g,
                         P[2] - c.clo[2] + c.cb.g);
  const I csq = (I)c.cb.sq, fsq = (I)c.fb.sq;
  const int g = c.fb.g;
  T f[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    T v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m)
      v[m] = ld_pop(fine,
                    (I)q * fsq + sidx_i<I>(c.fb, 2 * rx + (m & 1) + g, 2 * ry + ((m >> 1) & 1) + g,
                                           2 * rz + (m >> 2) + g),
                    c.fb);
    f[q] = T(0.125) * (((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7])));
  }
  collide_cell<T, PAIRED>(f, om_s, om_b, rho0, r);
#pragma unroll
  for (int q = 0; q < NV; ++q) st_pop(coarse, (I)q * csq + cc, c.cb, f[q]);
}

// Cells of the shell of thickness w of a box with extents (ex, ey, ez),
// enumerated without visiting the interior: the two z slabs, then the two y
// slabs between them, then the two x slabs between those.
__host__ __device__ __forceinline__ long long shell_cells(int ex, int ey, int ez, int w) {
  return (long long)ex * ey * ez - (long long)(ex - 2 * w) * (ey - 2 * w) * (ez - 2 * w);
}
__host__ __device__ __forceinline__ bool shell_coords(int t, int ex, int ey, int ez, int w, int* p) {
  const int nzf = ex * ey * w;
  if (t < 2 * nzf) {
    const int f = t / nzf;
    int r = t - f * nzf;
    p[2] = r / (ex * ey) + (f ? ez - w : 0);
    r -= (r / (ex * ey)) * (ex * ey);
    p[1] = r / ex;
    p[0] = r - p[1] * ex;
    return true;
  }
  t -= 2 * nzf;
  const int izl = ez - 2 * w;
  const int nyf = ex * w * izl;
  if (t < 2 * nyf) {
    const int f = t / nyf;
    int r = t - f * nyf;
    p[2] = w + r / (ex * w);
    r -= (r / (ex * w)) * (ex * w);
    p[1] = r / ex + (f ? ey - w : 0);
    p[0] = r - (r / ex) * ex;
    return true;
  }
  t -= 2 * nyf;
  const int iyl = ey - 2 * w;
  const int nxf = w * iyl * izl;
  if (t < 2 * nxf) {
    const int f = t / nxf;
    int r = t - f * nxf;
    p[2] = w + r / (iyl * w);
    r -= (r / (iyl * w)) * (iyl * w);
    p[1] = w + r / w;
    p[0] = r - (r / w) * w + (f ? ex - w : 0);
    return true;
  }
  return false;
}

// ring cells of a coupling: the shell of thickness 1 of coarsen(patch)
// grown by one (extents nf/2 + 2 per axis)
__host__ __device__ __forceinline__ long long ring_cells_of(const Coupling& c) {
  return shell_cells(c.fb.n[0] / 2 + 2, c.fb.n[1] / 2 + 2, c.fb.n[2] / 2 + 2, 1);
}
__host__ __device__ __forceinline__ bool ring_coords(const Coupling& c, int t, int* r) {
  return shell_coords(t, c.fb.n[0] / 2 + 2, c.fb.n[1] / 2 + 2, c.fb.n[2] / 2 + 2, 1, r);
}
// fine ghost cells: the shell of thickness g of the grown storage box
__host__ __device__ __forceinline__ long long ghost_cells_of(const Box3& b) {
  return shell_cells(b.n[0] + 2 * b.g, b.n[1] + 2 * b.g, b.n[2] + 2 * b.g, b.g);
}
__host__ __device__ __forceinline__ bool ghost_coords(const Box3& b, int t, int* s) {
  return shell_coords(t, b.n[0] + 2 * b.g, b.n[1] + 2 * b.g, b.n[2] + 2 * b.g, b.g, s);
}

// Coalescence of population q into the coarse ring cell (rx,ry,rz) (ring
// coordinates): every population q that left the patch in the last two fine
// sub-steps is added with volume weight 1/8.  One thread per (ring cell,
// population): fifteen independent threads with eight loads each keep more
// loads in flight than one thread walking the populations.  QFORM (pull
// form): the ring cell will gather population q from its neighbour at
// -c_q, so the sum is added to that neighbour's entry of the coarse store
// (the values are those the push form adds to, bit for bit).
template <typename T, typename I = long long, bool QFORM = false>
__host__ __device__ __forceinline__ void cell_coalesce_q(const T* __restrict__ fine, T* __restrict__ coarse,
                                                const Coupling& c, int rx, int ry, int rz, int q,
                                                T rho0) {
  const int cgx = c.flo[0] / 2 + rx - 1, cgy = c.flo[1] / 2 + ry - 1, cgz = c.flo[2] / 2 + rz - 1;
  const int cx = CX(q), cy = CY(q), cz = CZ(q);
  int P[3] = {cgx, cgy, cgz};
  if (QFORM) {
    P[0] -= cx;
    P[1] -= cy;
    P[2] -= cz;
  }
  if (c.cper)
    for (int d = 0; d < 3; ++d) P[d] = wrapi(P[d], c.cdom[d]);
  const I cc = sidx_i<I>(c.cb, P[0] - c.clo[0] + c.cb.g, P[1] - c.clo[1] + c.cb.g,
                         P[2] - c.clo[2] + c.cb.g);
  const int fx0 = 2 * cgx - c.flo[0], fy0 = 2 * cgy - c.flo[1], fz0 = 2 * cgz - c.flo[2];
  const I fq = (I)q * (I)c.fb.sq;
  T v[8];
  int k = 0;
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const int x = fx0 + (m & 1), y = fy0 + ((m >> 1) & 1), z = fz0 + (m >> 2);
    // a population at a ghost cell came from the patch iff it was inside
    // one or two sub-steps ago
    const bool from_patch = in_valid(c.fb, x - cx, y - cy, z - cz) ||
                            in_valid(c.fb, x - 2 * cx, y - 2 * cy, z - 2 * cz);
    v[m] = from_patch ? ld_pop(fine, fq + sidx_i<I>(c.fb, x + c.fb.g, y + c.fb.g, z + c.fb.g), c.fb)
                      : T(0);
    k += from_patch ? 1 : 0;
  }
  if (k == 0) return;
  const T sum = ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]));
  const I i = (I)q * (I)c.cb.sq + cc;
  // f_c += (1/8) sum f  ==  g_c += (k/8) w rho0 + (1/8) sum g
  st_pop(coarse, i, c.cb,
         (ld_pop_rw(coarse, i, c.cb) + T(0.125) * T(k) * T(W(q)) * rho0) + T(0.125) * sum);
}

// covered coarse cell (rx,ry,rz) of coarsen(patch) <- mean of its children
template <typename T, typename I = long long>
__host__ __device__ __forceinline__ void cell_restrict(const T* __restrict__ fine, T* __restrict__ coarse,
                                              const Coupling& c, int rx, int ry, int rz) {
  int P[3] = {c.flo[0] / 2 + rx, c.flo[1] / 2 + ry, c.flo[2] / 2 + rz};
  if (c.cper)
    for (int d = 0; d < 3; ++d) P[d] = wrapi(P[d], c.cdom[d]);
  const I cc = sidx_i<I>(c.cb, P[0] - c.clo[0] + c.cb.g, P[1] - c.clo[1] + c.cb.g,
                         P[2] - c.clo[2] + c.cb.g);
  const I csq = (I)c.cb.sq, fsq = (I)c.fb.sq;
  const int g = c.fb.g;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    T v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m)
      v[m] = ld_pop(fine,
                    (I)q * fsq + sidx_i<I>(c.fb, 2 * rx + (m & 1) + g, 2 * ry + ((m >> 1) & 1) + g,
                                           2 * rz + (m >> 2) + g),
                    c.fb);
    st_pop(coarse, (I)q * csq + cc, c.cb,
           T(0.125) * (((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]))));
  }
}

}  // namespace lbx
