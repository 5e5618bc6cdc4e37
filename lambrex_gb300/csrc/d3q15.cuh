// d3q15.cuh -- D3Q15 velocity set and the per-cell collision used by every
// kernel of liblbx_cuda.so.
//
// The collision is the reference's moment-space two-relaxation-rate operator
// (src/AmrSim.cpp:25-107): project f on 15 modes, keep rho and j, relax the
// trace of the stress with omega_b toward rho u^2 and its traceless part with
// omega_s toward rho (u_a u_b - u^2 DELTA_ab) with DELTA = diag(1/15)
// (src/AmrSim.cpp:1033-1035), zero the five ghost modes and project back.
// Here the 15x15 products are not formed: populations are split into
// even/odd pairs (f_q, f_-q), the ten needed moments come from pair sums and
// differences, and the back-projection uses the closed form of columns 0..9
// of the inverse mode matrix (src/AmrSim.cpp:1056-1073).  About 115 floating
// point operations per cell instead of about 930; results agree with the
// reference order to a few ulps per step.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace lbx {

constexpr int NV = 15;

// velocity components, ordering of include/d3q15_bgk.h:14-22
__host__ __device__ constexpr int CX(int q) {
  return q == 1 ? 1 : q == 2 ? -1 : (q >= 7 && q <= 10) ? 1 : (q >= 11) ? -1 : 0;
}
__host__ __device__ constexpr int CY(int q) {
  return q == 3 ? 1 : q == 4 ? -1 : (q == 7 || q == 8 || q == 11 || q == 12) ? 1
                                   : (q == 9 || q == 10 || q == 13 || q == 14) ? -1 : 0;
}
__host__ __device__ constexpr int CZ(int q) {
  return q == 5 ? 1 : q == 6 ? -1 : (q == 7 || q == 9 || q == 11 || q == 13) ? 1
                                   : (q == 8 || q == 10 || q == 12 || q == 14) ? -1 : 0;
}
// lattice weights W (include/d3q15_bgk.h:24-28)
__host__ __device__ constexpr double W(int q) {
  return q == 0 ? 2.0 / 9.0 : q <= 6 ? 1.0 / 9.0 : 1.0 / 72.0;
}

__host__ __device__ __forceinline__ double rcp(double x) {
#ifdef __CUDA_ARCH__
  return __drcp_rn(x);
#else
  return 1.0 / x;
#endif
}
__host__ __device__ __forceinline__ float rcp(float x) {
#ifdef __CUDA_ARCH__
  return __frcp_rn(x);
#else
  return 1.0f / x;
#endif
}

// v / 3 in FP32 without the bias of the rounded constant: q = v c3, then
// the exact residual v - 3 q (one FMA) corrects it by one more FMA
__host__ __device__ __forceinline__ float third_f(float v) {
  const float c3 = (float)(1.0 / 3.0);
  const float q = v * c3;
#ifdef __CUDA_ARCH__
  return __fmaf_rn(__fmaf_rn(-3.0f, q, v), c3, q);
#else
  return std::fma(std::fma(-3.0f, q, v), c3, q);
#endif
}

// In-place collision of one cell.  f holds populations (rho0 == 0) or
// shifted populations g_q = f_q - w_q rho0 (rho0 > 0); the rest state w rho0
// is exactly mode 0, so the shift only turns the mode-0 value into
// delta-rho and adds rho0 back where the density divides.
template <typename T>
__host__ __device__ __forceinline__ void collide(T* f, T om_s, T om_b, T rho0) {
  const T s1 = f[1] + f[2], d1 = f[1] - f[2];
  const T s3 = f[3] + f[4], d3 = f[3] - f[4];
  const T s5 = f[5] + f[6], d5 = f[5] - f[6];
  const T s7 = f[7] + f[14], d7 = f[7] - f[14];    // (+,+,+) / (-,-,-)
  const T s8 = f[8] + f[13], d8 = f[8] - f[13];    // (+,+,-) / (-,-,+)
  const T s9 = f[9] + f[12], d9 = f[9] - f[12];    // (+,-,+) / (-,+,-)
  const T sA = f[10] + f[11], dA = f[10] - f[11];  // (+,-,-) / (-,+,+)
  const T Q1 = s7 + s8, Q2 = s9 + sA, Q3 = s7 - s8, Q4 = s9 - sA;
  const T D = Q1 + Q2;             // sum over diagonal pairs
  const T A = s1 + s3 + s5;        // sum over axis pairs
  const T drho = f[0] + A + D;     // mode 0 (delta rho when shifted)
  const T rho = drho + rho0;
  const T P1 = d7 + d8, P2 = d9 + dA, P3 = d7 - d8, P4 = d9 - dA;
  const T jx = d1 + P1 + P2;       // modes 1..3
  const T jy = d3 + P1 - P2;
  const T jz = d5 + P3 + P4;
  const T sxy = Q1 - Q2, sxz = Q3 + Q4, syz = Q3 - Q4;  // modes 5, 6, 8
  const T A3 = A * T(1.0 / 3.0);
  const T dxx = s1 - A3, dyy = s3 - A3, dzz = s5 - A3;  // traceless part of 4, 7, 9
  const T TrS = fma(T(3), D, A) - drho;                 // trace of 4 + 7 + 9
  const T inv = rcp(rho);
  const T ux = jx * inv, uy = jy * inv, uz = jz * inv;
  const T rusq = fma(jx, ux, fma(jy, uy, jz * uz));     // rho u^2
  const T c15 = rusq * T(1.0 / 15.0);                   // rho u^2 DELTA_aa
  const T TrS3 = fma(om_b, rusq - TrS, TrS) * T(1.0 / 3.0);
  const T mxx = fma(om_s, fma(jx, ux, -c15) - dxx, dxx) + TrS3;
  const T myy = fma(om_s, fma(jy, uy, -c15) - dyy, dyy) + TrS3;
  const T mzz = fma(om_s, fma(jz, uz, -c15) - dzz, dzz) + TrS3;
  const T mxy = fma(om_s, fma(jx, uy, -sxy), sxy);
  const T mxz = fma(om_s, fma(jx, uz, -sxz), sxz);
  const T myz = fma(om_s, fma(jy, uz, -syz), syz);
  const T Tp = mxx + myy + mzz;  // not TrS': DELTA = 1/15 leaves a trace
  // back-projection: columns 0..9 of the inverse mode matrix
  f[0] = fma(T(-1.0 / 3.0), Tp, T(2.0 / 9.0) * drho);
  const T ba = fma(T(-1.0 / 6.0), Tp, T(1.0 / 9.0) * drho);
  const T ex = fma(T(0.5), mxx, ba), ey = fma(T(0.5), myy, ba), ez = fma(T(0.5), mzz, ba);
  const T bd = fma(T(1.0 / 24.0), Tp, T(1.0 / 72.0) * drho);
  const T R1 = mxy + mxz, R2 = mxy - mxz;
  const T e7 = fma(T(0.125), R1 + myz, bd);
  const T e8 = fma(T(0.125), R2 - myz, bd);
  const T e9 = fma(T(-0.125), R2 + myz, bd);
  const T eA = fma(T(-0.125), R1 - myz, bd);
  const T S1 = jx + jy, S2 = jx - jy;
  const T o7 = S1 + jz, o8 = S1 - jz, o9 = S2 + jz, oA = S2 - jz;
  if constexpr (sizeof(T) == 4) {
    // The momentum of the outputs is j/3 from each axis pair and j/24 from
    // each diagonal pair.  1/3 (and 1/24) rounded to FP32 is 3e-8 too large,
    // so products with it would add 3e-8 of every cell's momentum at every
    // step (1e-5 of the velocity after 500 steps).  The thirds are taken
    // with their exact FMA residual instead, q = v/3 + (v - 3 q)/3, which
    // is within an ulp of v/3 and unbiased.
    const T jx3 = third_f(jx), jy3 = third_f(jy), jz3 = third_f(jz);
    f[1] = ex + jx3;
    f[2] = ex - jx3;
    f[3] = ey + jy3;
    f[4] = ey - jy3;
    f[5] = ez + jz3;
    f[6] = ez - jz3;
    const T q7 = third_f(o7), q8 = third_f(o8), q9 = third_f(o9), qA = third_f(oA);
    f[7] = fma(T(0.125), q7, e7);
    f[14] = fma(T(-0.125), q7, e7);
    f[8] = fma(T(0.125), q8, e8);
    f[13] = fma(T(-0.125), q8, e8);
    f[9] = fma(T(0.125), q9, e9);
    f[12] = fma(T(-0.125), q9, e9);
    f[10] = fma(T(0.125), qA, eA);
    f[11] = fma(T(-0.125), qA, eA);
  } else {
    f[1] = fma(T(1.0 / 3.0), jx, ex);
    f[2] = fma(T(-1.0 / 3.0), jx, ex);
    f[3] = fma(T(1.0 / 3.0), jy, ey);
    f[4] = fma(T(-1.0 / 3.0), jy, ey);
    f[5] = fma(T(1.0 / 3.0), jz, ez);
    f[6] = fma(T(-1.0 / 3.0), jz, ez);
    f[7] = fma(T(1.0 / 24.0), o7, e7);
    f[14] = fma(T(-1.0 / 24.0), o7, e7);
    f[8] = fma(T(1.0 / 24.0), o8, e8);
    f[13] = fma(T(-1.0 / 24.0), o8, e8);
    f[9] = fma(T(1.0 / 24.0), o9, e9);
    f[12] = fma(T(-1.0 / 24.0), o9, e9);
    f[10] = fma(T(1.0 / 24.0), oA, eA);
    f[11] = fma(T(-1.0 / 24.0), oA, eA);
  }
}

// Second-order equilibrium (src/AmrSim.cpp:873-927) in FP64.  The
// reference divides by c_s^2 = 1/3 and 2 c_s^4 = 2/9; here those are the
// exact multipliers 3, 4.5, 1.5 and 3 (agreement to an ulp, no divisions on
// the slow FP64 pipe).
__host__ __device__ __forceinline__ void equilibrium(double rho, double ux, double uy, double uz,
                                            double* out) {
  const double rw0 = rho * (2.0 / 9.0), rw1 = rho * (1.0 / 9.0), rw2 = rho * (1.0 / 72.0);
  const double u2x = ux * ux, u2y = uy * uy, u2z = uz * uz;
  const double ax = ux * 3.0, ay = uy * 3.0, az = uz * 3.0;      // u / c_s^2
  const double bx = u2x * 4.5, by = u2y * 4.5, bz = u2z * 4.5;   // u^2 / (2 c_s^4)
  const double uv = ax * ay, vw = ay * az, uw = ax * az;
  const double usq = u2x + u2y + u2z;
  const double m1 = usq * 1.5;  // u^2 / (2 c_s^2)
  const double m2 = usq * 3.0;  // u^2 (1 - c_s^2) / (2 c_s^4)
  out[0] = rw0 * (1.0 - m1);
  out[1] = rw1 * (1.0 - m1 + ax + bx);
  out[2] = rw1 * (1.0 - m1 - ax + bx);
  out[3] = rw1 * (1.0 - m1 + ay + by);
  out[4] = rw1 * (1.0 - m1 - ay + by);
  out[5] = rw1 * (1.0 - m1 + az + bz);
  out[6] = rw1 * (1.0 - m1 - az + bz);
  out[7] = rw2 * (1.0 + ax + ay + az + uv + vw + uw + m2);
  out[8] = rw2 * (1.0 + ax + ay - az + uv - vw - uw + m2);
  out[9] = rw2 * (1.0 + ax - ay + az - uv - vw + uw + m2);
  out[10] = rw2 * (1.0 + ax - ay - az - uv + vw - uw + m2);
  out[11] = rw2 * (1.0 - ax + ay + az - uv + vw - uw + m2);
  out[12] = rw2 * (1.0 - ax + ay - az - uv - vw + uw + m2);
  out[13] = rw2 * (1.0 - ax - ay + az + uv - vw - uw + m2);
  out[14] = rw2 * (1.0 - ax - ay - az + uv + vw + uw + m2);
}

// The same equilibrium for the FP32 shifted store, g_q = f_q^eq - w_q rho0
// = w_q [(rho - rho0) + rho t_q] with t_q the velocity polynomial above.
// Only rho - rho0 is formed in FP64 (it cancels); the rest is FP32, within
// an ulp or two of the FP64 value rounded to FP32, and keeps the slow FP64
// pipe to one subtraction and five conversions per cell.
__host__ __device__ __forceinline__ void equilibrium_shifted(double rho, double ux, double uy,
                                                             double uz, double rho0, float* out) {
  const float dr = (float)(rho - rho0), r = (float)rho;
  const float x = (float)ux, y = (float)uy, z = (float)uz;
  const float ax = x * 3.0f, ay = y * 3.0f, az = z * 3.0f;
  const float bx = x * x * 4.5f, by = y * y * 4.5f, bz = z * z * 4.5f;
  const float uv = ax * ay, vw = ay * az, uw = ax * az;
  const float usq = x * x + y * y + z * z;
  const float m1 = usq * 1.5f, m2 = usq * 3.0f;
  const float w0 = 2.0f / 9.0f, w1 = 1.0f / 9.0f, w2 = 1.0f / 72.0f;
  out[0] = w0 * (dr + r * (-m1));
  out[1] = w1 * (dr + r * (-m1 + ax + bx));
  out[2] = w1 * (dr + r * (-m1 - ax + bx));
  out[3] = w1 * (dr + r * (-m1 + ay + by));
  out[4] = w1 * (dr + r * (-m1 - ay + by));
  out[5] = w1 * (dr + r * (-m1 + az + bz));
  out[6] = w1 * (dr + r * (-m1 - az + bz));
  out[7] = w2 * (dr + r * (ax + ay + az + uv + vw + uw + m2));
  out[8] = w2 * (dr + r * (ax + ay - az + uv - vw - uw + m2));
  out[9] = w2 * (dr + r * (ax - ay + az - uv - vw + uw + m2));
  out[10] = w2 * (dr + r * (ax - ay - az - uv + vw - uw + m2));
  out[11] = w2 * (dr + r * (-ax + ay + az - uv + vw - uw + m2));
  out[12] = w2 * (dr + r * (-ax + ay - az - uv - vw + uw + m2));
  out[13] = w2 * (dr + r * (-ax - ay + az + uv - vw - uw + m2));
  out[14] = w2 * (dr + r * (-ax - ay - az + uv + vw + uw + m2));
}

// Storage description of one box: valid extents n, ghost width g, strides.
struct Box3 {
  int n[3];        // valid extents
  int g;           // ghost layers in storage
  long long sx;    // row length  = n[0] + 2g
  long long sxy;   // plane size  = (n[1] + 2g) * sx
  long long sq;    // component stride = (n[2] + 2g) * sxy
  __host__ __device__ long long at(int x, int y, int z) const {  // valid-relative coords
    return (long long)(z + g) * sxy + (long long)(y + g) * sx + (x + g);
  }
};

inline Box3 make_box(int nx, int ny, int nz, int g) {
  Box3 b;
  b.n[0] = nx;
  b.n[1] = ny;
  b.n[2] = nz;
  b.g = g;
  b.sx = nx + 2 * g;
  b.sxy = (long long)(ny + 2 * g) * b.sx;
  b.sq = (long long)(nz + 2 * g) * b.sxy;
  return b;
}

}  // namespace lbx
