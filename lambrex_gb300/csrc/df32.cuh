// df32.cuh -- FP64-store collision carried in pairs of FP32 values.
//
// GB300 issues about 1.9 FP64 instructions per clock per SM against 128 FP32
// ones, so the native FP64 step is bound by the FP64 pipe at about a sixth of
// the HBM roofline.  This variant keeps the FP64 store and the reference's
// algorithm but does the arithmetic of the collision on the FP32 pipe: each
// population is split (with integer operations, no FP64 instruction) into an
// unevaluated sum hi + lo of two floats (48-bit significand), the collision of
// d3q15.cuh is evaluated with error-free transformations (Knuth's two-sum,
// Dekker's two-product via FMA), and the result goes back to FP64 with one
// correctly rounded FP64 addition per population.
//
// Range: the split covers |f| in [2^-74, 2^128); a cell with any population
// outside it is collided with the native FP64 code instead.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#include "d3q15.cuh"

namespace lbx {

struct dfl {
  float hi, lo;
};

__host__ __device__ __forceinline__ float f_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  std::memcpy(&f, &b, 4);
  return f;
#endif
}
__host__ __device__ __forceinline__ uint32_t bits_f(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t b;
  std::memcpy(&b, &f, 4);
  return b;
#endif
}
__host__ __device__ __forceinline__ void d_words(double x, uint32_t* hi, uint32_t* lo) {
#ifdef __CUDA_ARCH__
  *hi = (uint32_t)__double2hiint(x);
  *lo = (uint32_t)__double2loint(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  *hi = (uint32_t)(b >> 32);
  *lo = (uint32_t)b;
#endif
}
__host__ __device__ __forceinline__ double d_from_words(uint32_t hi, uint32_t lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  const uint64_t b = ((uint64_t)hi << 32) | lo;
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}
__host__ __device__ __forceinline__ float fma_f(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}
__host__ __device__ __forceinline__ float add_f(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);  // never contracted into an FMA
#else
  return a + b;
#endif
}
__host__ __device__ __forceinline__ float sub_f(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
__host__ __device__ __forceinline__ float mul_f(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
__host__ __device__ __forceinline__ float u2f(uint32_t r) {
#ifdef __CUDA_ARCH__
  return __uint2float_rn(r);
#else
  return (float)r;
#endif
}

// High word of a double rebiased from exponent 1023 to 127: the exponent
// field e (bits 20..30) becomes e - 896, the sign bit stays (no borrow for
// e >= 896).  Both the range test and the split start from it.
__host__ __device__ __forceinline__ uint32_t rebias_hi(uint32_t h) { return h - 0x38000000u; }

// exponent field of a double within the split range [2^-74, 2^128), i.e.
// 949 <= e <= 1150, from the rebiased high word t: (t << 1) drops the sign,
// (t << 1) - (53 << 21) is ((e - 949) << 21) + (mantissa bits below 2^21)
// modulo 2^32, which is below 202 << 21 exactly when 0 <= e - 949 <= 201
// (one shift-add and one unsigned compare)
__host__ __device__ __forceinline__ bool split_ok_t(uint32_t t) {
  return (t << 1) - (53u << 21) < (202u << 21);
}
__host__ __device__ __forceinline__ bool split_ok(double x) {
  uint32_t h, l;
  d_words(x, &h, &l);
  return split_ok_t(rebias_hi(h));
}

// x = hi + lo: hi = x truncated to 24 bits, lo = the remaining 29 bits
// rounded to 24 (|error| <= 2^-48 |x|).  Valid when split_ok(x).
//   hi bits: the rebiased word shifted left by 3 with the top 3 bits of the
//     low word shifted in (the exponent e - 896 < 256 leaves bits 28..30 of t
//     clear, so bit 31 of the shift is clear), then the sign;
//   lo: the low 29 bits converted to float and scaled by +-2^(e - 1075),
//     whose bits are hi's sign and exponent field lowered by 52 (e - 896 is
//     at least 53, so the field stays positive and the sign is kept).
// Integer operations, one 32-bit integer conversion and one multiplication.
__host__ __device__ __forceinline__ dfl split_words(uint32_t h, uint32_t l) {
  const uint32_t t = rebias_hi(h);
  const uint32_t hb = ((t << 3) | (l >> 29)) | (h & 0x80000000u);
  const float scale = f_bits((hb & 0xff800000u) - (52u << 23));
  return dfl{f_bits(hb), mul_f(u2f(l & 0x1fffffffu), scale)};
}
__host__ __device__ __forceinline__ dfl split(double x) {
  uint32_t h, l;
  d_words(x, &h, &l);
  return split_words(h, l);
}

// float -> double by bits (exact; zero and subnormal floats give +-0)
__host__ __device__ __forceinline__ double widen(float v) {
  const uint32_t b = bits_f(v);
  if ((b & 0x7f800000u) == 0) return d_from_words(b & 0x80000000u, 0u);
  return d_from_words((b & 0x80000000u) | (((b & 0x7fffffffu) >> 3) + 0x38000000u), b << 29);
}
__host__ __device__ __forceinline__ double join(dfl a) { return widen(a.hi) + widen(a.lo); }

// ---- error-free transformations and pair arithmetic -----------------------
__host__ __device__ __forceinline__ dfl quick_two_sum(float a, float b) {
  const float s = add_f(a, b);
  return dfl{s, sub_f(b, sub_f(s, a))};
}
__host__ __device__ __forceinline__ dfl two_sum(float a, float b) {
  const float s = add_f(a, b);
  const float bb = sub_f(s, a);
  return dfl{s, add_f(sub_f(a, sub_f(s, bb)), sub_f(b, bb))};
}
// Pair sum with one two-sum of the leading parts (11 FP32 operations).  Its
// error is bounded by about 2^-46 (|a| + |b|); over 100 to 500 lattice steps
// the collision stays within 4e-14 to 1.2e-13 of the FP64 reference order
// (CPU check against the oracle), the same as with the fully renormalised
// sum.
__host__ __device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  const dfl s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, add_f(s.lo, add_f(a.lo, b.lo)));
}
__host__ __device__ __forceinline__ dfl operator-(dfl a) { return dfl{-a.hi, -a.lo}; }
__host__ __device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
// The same sum without the final renormalisation (8 operations): the
// trailing part may grow to a few ulps of the leading one.  Used where the
// operands are populations or their final combinations (first pair sums,
// back-projection), where the CPU check over 500 steps shows no change in
// the error; the moments and their relaxation keep the renormalised sum.
__host__ __device__ __forceinline__ dfl add_lz(dfl a, dfl b) {
  const dfl s = two_sum(a.hi, b.hi);
  return dfl{s.hi, add_f(s.lo, add_f(a.lo, b.lo))};
}
__host__ __device__ __forceinline__ dfl sub_lz(dfl a, dfl b) { return add_lz(a, -b); }
__host__ __device__ __forceinline__ dfl renorm(dfl a) { return quick_two_sum(a.hi, a.lo); }
// Products are left unnormalised: |e| is at most a few ulps of p, so the
// pair (p, e) carries the product to 2^-47 as it is, and the sums it feeds
// renormalise (CPU check over 500 steps: the same error as with a final
// quick-two-sum, three operations fewer per product).
__host__ __device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = mul_f(a.hi, b.hi);
  float e = fma_f(a.hi, b.hi, -p);
  e = fma_f(a.hi, b.lo, e);
  e = fma_f(a.lo, b.hi, e);
  return dfl{p, e};
}
// product with an exactly representable float
__host__ __device__ __forceinline__ dfl mulf(dfl a, float f) {
  const float p = mul_f(a.hi, f);
  const float e = fma_f(a.lo, f, fma_f(a.hi, f, -p));
  return dfl{p, e};
}
// product with a power of two (exact)
__host__ __device__ __forceinline__ dfl mul2(dfl a, float p2) { return dfl{mul_f(a.hi, p2), mul_f(a.lo, p2)}; }
// a pair constant for a rational c (rounded to 48 bits)
__host__ __device__ __forceinline__ dfl dconst(double c) {
  const float h = (float)c;
  return dfl{h, (float)(c - (double)h)};
}
// approximate FP32 reciprocal (the hardware's; any error below 2^-16 will do)
__host__ __device__ __forceinline__ float rcp_approx(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / x;
#endif
}
// 1 / a from r ~ 1/a.hi: the residual e = 1 - a r comes from two FMAs
// whose roundings are of the size of e itself (2^-24 |e|), and
// 1/a = r / (1 - e) = r (1 + e + e^2 + ...); keeping e + e^2 leaves
// O(e^3) + 2^-24 |e|, below 2^-46 for |e| < 2^-16.
__host__ __device__ __forceinline__ dfl recip(dfl a) {
  const float r = rcp_approx(a.hi);
  const float t = fma_f(-a.hi, r, 1.0f);
  const float e = fma_f(-a.lo, r, t);
  return dfl{r, mul_f(r, fma_f(e, e, e))};
}

// The collision of d3q15.cuh (collide<T>) with T = pair of floats; same
// algebra and the same restructuring of the 15x15 products.
__host__ __device__ __forceinline__ void collide_df(dfl* f, dfl om_s, dfl om_b) {
  const dfl s1 = add_lz(f[1], f[2]), d1 = sub_lz(f[1], f[2]);
  const dfl s3 = add_lz(f[3], f[4]), d3 = sub_lz(f[3], f[4]);
  const dfl s5 = add_lz(f[5], f[6]), d5 = sub_lz(f[5], f[6]);
  const dfl s7 = add_lz(f[7], f[14]), d7 = sub_lz(f[7], f[14]);
  const dfl s8 = add_lz(f[8], f[13]), d8 = sub_lz(f[8], f[13]);
  const dfl s9 = add_lz(f[9], f[12]), d9 = sub_lz(f[9], f[12]);
  const dfl sA = add_lz(f[10], f[11]), dA = sub_lz(f[10], f[11]);
  const dfl Q1 = s7 + s8, Q2 = s9 + sA, Q3 = s7 - s8, Q4 = s9 - sA;
  const dfl D = Q1 + Q2;
  const dfl A = s1 + s3 + s5;
  const dfl rho = f[0] + A + D;
  const dfl P1 = d7 + d8, P2 = d9 + dA, P3 = d7 - d8, P4 = d9 - dA;
  const dfl jx = d1 + P1 + P2;
  const dfl jy = d3 + P1 - P2;
  const dfl jz = d5 + P3 + P4;
  const dfl sxy = Q1 - Q2, sxz = Q3 + Q4, syz = Q3 - Q4;
  const dfl third = dconst(1.0 / 3.0);
  const dfl A3 = A * third;
  const dfl dxx = s1 - A3, dyy = s3 - A3, dzz = s5 - A3;
  const dfl TrS = mulf(D, 3.0f) + A - rho;
  const dfl inv = recip(rho);
  const dfl ux = jx * inv, uy = jy * inv, uz = jz * inv;
  const dfl rusq = jx * ux + jy * uy + jz * uz;
  const dfl c15 = rusq * dconst(1.0 / 15.0);
  const dfl TrS3 = (TrS + om_b * (rusq - TrS)) * third;
  const dfl mxx = dxx + om_s * (jx * ux - c15 - dxx) + TrS3;
  const dfl myy = dyy + om_s * (jy * uy - c15 - dyy) + TrS3;
  const dfl mzz = dzz + om_s * (jz * uz - c15 - dzz) + TrS3;
  const dfl mxy = sxy + om_s * (jx * uy - sxy);
  const dfl mxz = sxz + om_s * (jx * uz - sxz);
  const dfl myz = syz + om_s * (jy * uz - syz);
  // back-projection; T' is renormalised before its product with 1/3 so that
  // 3 T3 - T' (which enters the mass balance) carries no bias
  const dfl Tp = renorm(add_lz(add_lz(mxx, myy), mzz));
  const dfl T3 = Tp * third;
  // rho / 9 with the residual folded back: the outputs sum to
  // 9 r9 - 3 T3 + T', so any bias of r9 is a mass drift per step (the plain
  // pair product by 1/9 loses about 2e-16 of rho per step on average).
  // rho.hi - 9 r9.hi is exact (Sterbenz); the rest are small terms.
  dfl r9 = rho * dconst(1.0 / 9.0);
  {
    const float p9 = mul_f(9.0f, r9.hi);
    const float e9 = fma_f(9.0f, r9.hi, -p9);
    const float res = add_f(sub_f(rho.hi, p9), sub_f(sub_f(rho.lo, e9), mul_f(9.0f, r9.lo)));
    r9.lo = fma_f(res, (float)(1.0 / 9.0), r9.lo);
  }
  f[0] = sub_lz(mul2(r9, 2.0f), T3);           // 2/9 rho - T'/3
  const dfl ba = sub_lz(r9, mul2(T3, 0.5f));    // rho/9 - T'/6
  const dfl ex = add_lz(ba, mul2(mxx, 0.5f)), ey = add_lz(ba, mul2(myy, 0.5f)),
            ez = add_lz(ba, mul2(mzz, 0.5f));
  const dfl jx3 = jx * third, jy3 = jy * third, jz3 = jz * third;
  f[1] = add_lz(ex, jx3);
  f[2] = sub_lz(ex, jx3);
  f[3] = add_lz(ey, jy3);
  f[4] = sub_lz(ey, jy3);
  f[5] = add_lz(ez, jz3);
  f[6] = sub_lz(ez, jz3);
  const dfl bd = mul2(add_lz(r9, T3), 0.125f);  // rho/72 + T'/24
  const dfl R1 = add_lz(mxy, mxz), R2 = sub_lz(mxy, mxz);
  const dfl e7 = add_lz(bd, mul2(add_lz(R1, myz), 0.125f));
  const dfl e8 = add_lz(bd, mul2(sub_lz(R2, myz), 0.125f));
  const dfl e9 = sub_lz(bd, mul2(add_lz(R2, myz), 0.125f));
  const dfl eA = sub_lz(bd, mul2(sub_lz(R1, myz), 0.125f));
  const dfl S1 = add_lz(jx, jy), S2 = sub_lz(jx, jy);
  const dfl o7 = mul2(add_lz(S1, jz) * third, 0.125f);  // (.)/24
  const dfl o8 = mul2(sub_lz(S1, jz) * third, 0.125f);
  const dfl o9 = mul2(add_lz(S2, jz) * third, 0.125f);
  const dfl oA = mul2(sub_lz(S2, jz) * third, 0.125f);
  f[7] = add_lz(e7, o7);
  f[14] = sub_lz(e7, o7);
  f[8] = add_lz(e8, o8);
  f[13] = sub_lz(e8, o8);
  f[9] = add_lz(e9, o9);
  f[12] = sub_lz(e9, o9);
  f[10] = add_lz(eA, oA);
  f[11] = sub_lz(eA, oA);
}

// Relaxation rates of a launch as FP64 (for the fallback) and as pairs.
struct DfRates {
  double om_s, om_b;
  dfl ps, pb;
};
inline DfRates df_rates(double om_s, double om_b) {
  return DfRates{om_s, om_b, dconst(om_s), dconst(om_b)};
}

// FP64 populations in, FP64 populations out, arithmetic in float pairs;
// cells outside the split range use the native FP64 collision.
__host__ __device__ __forceinline__ void collide_f64_via_df(double* f, const DfRates& r) {
  bool ok = true;
#pragma unroll
  for (int q = 0; q < NV; ++q) ok = ok && split_ok(f[q]);
  if (!ok) {
    collide<double>(f, r.om_s, r.om_b, 0.0);
    return;
  }
  dfl g[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) g[q] = split(f[q]);
  collide_df(g, r.ps, r.pb);
#pragma unroll
  for (int q = 0; q < NV; ++q) f[q] = join(g[q]);
}

// ---- pair arithmetic on the packed FP32x2 instructions --------------------
//
// Blackwell issues two FP32 additions, multiplications or FMAs of a float2 in
// one instruction (__fadd2_rn, __fmul2_rn, __ffma2_rn, sm_100 and later).
// dfl2 holds two pair values, lane x and lane y; every operation below is the
// scalar one of the section above applied per lane in the same order (a - b
// is a + (-b), exactly the IEEE subtraction).  A host build does each lane
// with the scalar operation, so the packed collision can be checked against
// the scalar one off the GPU.
struct dfl2 {
  float2 hi, lo;
};
__host__ __device__ __forceinline__ float2 p_add(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
  return __fadd2_rn(a, b);
#else
  return make_float2(add_f(a.x, b.x), add_f(a.y, b.y));
#endif
}
__host__ __device__ __forceinline__ float2 p_neg(float2 a) { return make_float2(-a.x, -a.y); }
__host__ __device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return p_add(a, p_neg(b)); }
__host__ __device__ __forceinline__ float2 p_mul(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
  return __fmul2_rn(a, b);
#else
  return make_float2(mul_f(a.x, b.x), mul_f(a.y, b.y));
#endif
}
__host__ __device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) {
#ifdef __CUDA_ARCH__
  return __ffma2_rn(a, b, c);
#else
  return make_float2(fma_f(a.x, b.x, c.x), fma_f(a.y, b.y, c.y));
#endif
}
__host__ __device__ __forceinline__ float2 p_splat(float v) { return make_float2(v, v); }

__host__ __device__ __forceinline__ dfl2 quick_two_sum2(float2 a, float2 b) {
  const float2 s = p_add(a, b);
  return dfl2{s, p_sub(b, p_sub(s, a))};
}
__host__ __device__ __forceinline__ dfl2 two_sum2(float2 a, float2 b) {
  const float2 s = p_add(a, b);
  const float2 bb = p_sub(s, a);
  return dfl2{s, p_add(p_sub(a, p_sub(s, bb)), p_sub(b, bb))};
}
__host__ __device__ __forceinline__ dfl2 operator+(dfl2 a, dfl2 b) {
  const dfl2 s = two_sum2(a.hi, b.hi);
  return quick_two_sum2(s.hi, p_add(s.lo, p_add(a.lo, b.lo)));
}
__host__ __device__ __forceinline__ dfl2 operator-(dfl2 a) { return dfl2{p_neg(a.hi), p_neg(a.lo)}; }
__host__ __device__ __forceinline__ dfl2 operator-(dfl2 a, dfl2 b) { return a + (-b); }
__host__ __device__ __forceinline__ dfl2 add_lz(dfl2 a, dfl2 b) {
  const dfl2 s = two_sum2(a.hi, b.hi);
  return dfl2{s.hi, p_add(s.lo, p_add(a.lo, b.lo))};
}
__host__ __device__ __forceinline__ dfl2 sub_lz(dfl2 a, dfl2 b) { return add_lz(a, -b); }
__host__ __device__ __forceinline__ dfl2 operator*(dfl2 a, dfl2 b) {
  const float2 p = p_mul(a.hi, b.hi);
  float2 e = p_fma(a.hi, b.hi, p_neg(p));
  e = p_fma(a.hi, b.lo, e);
  e = p_fma(a.lo, b.hi, e);
  return dfl2{p, e};
}
__host__ __device__ __forceinline__ dfl2 mul2(dfl2 a, float p2) {
  const float2 P = p_splat(p2);
  return dfl2{p_mul(a.hi, P), p_mul(a.lo, P)};
}
__host__ __device__ __forceinline__ dfl2 splat(dfl a) { return dfl2{p_splat(a.hi), p_splat(a.lo)}; }

// ---- one cell, twin operations packed -------------------------------------
__host__ __device__ __forceinline__ dfl2 pack(dfl a, dfl b) {
  return dfl2{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)};
}
__host__ __device__ __forceinline__ dfl lane_x(dfl2 a) { return dfl{a.hi.x, a.lo.x}; }
__host__ __device__ __forceinline__ dfl lane_y(dfl2 a) { return dfl{a.hi.y, a.lo.y}; }

// collide_df with the operations of one cell that come in twins (the same
// pair operation on two different operand pairs: the x/y components, the
// first pair sums, the output pairs f_q, f_q') issued as one packed
// operation; every value keeps the operation order of collide_df, so the
// results are bit-identical to it.
__host__ __device__ __forceinline__ void collide_df_w(dfl* f, dfl om_s, dfl om_b) {
  const dfl2 X13 = pack(f[1], f[3]), Y24 = pack(f[2], f[4]);
  const dfl2 S13 = add_lz(X13, Y24), D13 = sub_lz(X13, Y24);            // (s1, s3), (d1, d3)
  const dfl2 X79 = pack(f[7], f[9]), Y1412 = pack(f[14], f[12]);
  const dfl2 S79 = add_lz(X79, Y1412), D79 = sub_lz(X79, Y1412);        // (s7, s9), (d7, d9)
  const dfl2 X810 = pack(f[8], f[10]), Y1311 = pack(f[13], f[11]);
  const dfl2 S8A = add_lz(X810, Y1311), D8A = sub_lz(X810, Y1311);      // (s8, sA), (d8, dA)
  const dfl s5 = add_lz(f[5], f[6]), d5 = sub_lz(f[5], f[6]);
  const dfl2 Q12 = S79 + S8A, Q34 = S79 - S8A;                          // (Q1, Q2), (Q3, Q4)
  const dfl D = lane_x(Q12) + lane_y(Q12);
  const dfl A = lane_x(S13) + lane_y(S13) + s5;
  const dfl rho = f[0] + A + D;
  const dfl2 P12 = D79 + D8A, P34 = D79 - D8A;                          // (P1, P2), (P3, P4)
  const dfl P1 = lane_x(P12), P2 = lane_y(P12);
  const dfl2 Jxy = D13 + splat(P1) + pack(P2, -P2);                     // (jx, jy)
  const dfl jx = lane_x(Jxy), jy = lane_y(Jxy);
  const dfl jz = d5 + lane_x(P34) + lane_y(P34);
  const dfl Q1 = lane_x(Q12), Q2 = lane_y(Q12), Q3 = lane_x(Q34), Q4 = lane_y(Q34);
  const dfl2 Sxyxz = pack(Q1 - Q2, Q3 + Q4);                            // (sxy, sxz)
  const dfl syz = Q3 - Q4;
  const dfl third = dconst(1.0 / 3.0);
  const dfl A3 = A * third;
  const dfl2 Dxy = S13 - splat(A3);                                     // (dxx, dyy)
  const dfl dzz = s5 - A3;
  const dfl TrS = mulf(D, 3.0f) + A - rho;
  const dfl inv = recip(rho);
  const dfl2 Uxy = Jxy * splat(inv);                                    // (ux, uy)
  const dfl uy = lane_y(Uxy), uz = jz * inv;
  const dfl2 JU = Jxy * Uxy;                                            // (jx ux, jy uy)
  const dfl rusq = lane_x(JU) + lane_y(JU) + jz * uz;
  const dfl c15 = rusq * dconst(1.0 / 15.0);
  const dfl TrS3 = (TrS + om_b * (rusq - TrS)) * third;
  const dfl2 Mxy = Dxy + splat(om_s) * (JU - splat(c15) - Dxy) + splat(TrS3);  // (mxx, myy)
  const dfl mzz = dzz + om_s * (jz * uz - c15 - dzz) + TrS3;
  const dfl2 Oxy = Sxyxz + splat(om_s) * (splat(jx) * pack(uy, uz) - Sxyxz);    // (mxy, mxz)
  const dfl myz = syz + om_s * (jy * uz - syz);
  const dfl mxx = lane_x(Mxy), myy = lane_y(Mxy);
  const dfl Tp = renorm(add_lz(add_lz(mxx, myy), mzz));
  const dfl T3 = Tp * third;
  dfl r9 = rho * dconst(1.0 / 9.0);
  {
    const float p9 = mul_f(9.0f, r9.hi);
    const float e9 = fma_f(9.0f, r9.hi, -p9);
    const float res = add_f(sub_f(rho.hi, p9), sub_f(sub_f(rho.lo, e9), mul_f(9.0f, r9.lo)));
    r9.lo = fma_f(res, (float)(1.0 / 9.0), r9.lo);
  }
  f[0] = sub_lz(mul2(r9, 2.0f), T3);
  const dfl ba = sub_lz(r9, mul2(T3, 0.5f));
  const dfl2 Exy = add_lz(splat(ba), mul2(Mxy, 0.5f));                  // (ex, ey)
  const dfl ez = add_lz(ba, mul2(mzz, 0.5f));
  const dfl2 J3 = Jxy * splat(third);                                   // (jx/3, jy/3)
  const dfl jz3 = jz * third;
  const dfl2 F13 = add_lz(Exy, J3), F24 = sub_lz(Exy, J3);
  f[1] = lane_x(F13);
  f[3] = lane_y(F13);
  f[2] = lane_x(F24);
  f[4] = lane_y(F24);
  f[5] = add_lz(ez, jz3);
  f[6] = sub_lz(ez, jz3);
  const dfl bd = mul2(add_lz(r9, T3), 0.125f);
  const dfl mxy = lane_x(Oxy), mxz = lane_y(Oxy);
  const dfl R1 = add_lz(mxy, mxz), R2 = sub_lz(mxy, mxz);
  const dfl2 Zpm = pack(myz, -myz);
  const dfl2 E78 = add_lz(splat(bd), mul2(add_lz(pack(R1, R2), Zpm), 0.125f));  // (e7, e8)
  const dfl2 E9A = sub_lz(splat(bd), mul2(add_lz(pack(R2, R1), Zpm), 0.125f));  // (e9, eA)
  const dfl S1 = add_lz(jx, jy), S2 = sub_lz(jx, jy);
  const dfl2 Jpm = pack(jz, -jz);
  const dfl2 O78 = mul2(add_lz(splat(S1), Jpm) * splat(third), 0.125f);  // (o7, o8)
  const dfl2 O9A = mul2(add_lz(splat(S2), Jpm) * splat(third), 0.125f);  // (o9, oA)
  const dfl2 F78 = add_lz(E78, O78), F1413 = sub_lz(E78, O78);
  const dfl2 F910 = add_lz(E9A, O9A), F1211 = sub_lz(E9A, O9A);
  f[7] = lane_x(F78);
  f[8] = lane_y(F78);
  f[14] = lane_x(F1413);
  f[13] = lane_y(F1413);
  f[9] = lane_x(F910);
  f[10] = lane_y(F910);
  f[12] = lane_x(F1211);
  f[11] = lane_y(F1211);
}

// widen() of a normal float (exponent field not 0): the same bits without
// the test for zero and subnormal values
__host__ __device__ __forceinline__ double widen_normal(float v) {
  const uint32_t b = bits_f(v);
  return d_from_words((b & 0x80000000u) | (((b & 0x7fffffffu) >> 3) + 0x38000000u), b << 29);
}

// collide_f64_via_df with collide_df_w: the same bits.  The join tests once
// per cell that all thirty parts are normal floats (one compare each) and
// then widens them without the per-value test; otherwise it joins as join().
__host__ __device__ __forceinline__ void collide_f64_via_df_w(double* f, const DfRates& r) {
  uint32_t h[NV], l[NV];
  bool ok = true;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    d_words(f[q], &h[q], &l[q]);
    ok = ok & split_ok_t(rebias_hi(h[q]));
  }
  if (!ok) {
    collide<double>(f, r.om_s, r.om_b, 0.0);
    return;
  }
  dfl g[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) g[q] = split_words(h[q], l[q]);
  collide_df_w(g, r.ps, r.pb);
  bool normal = true;
#pragma unroll
  for (int q = 0; q < NV; ++q)
    normal = normal & (fabsf(g[q].hi) >= 0x1p-126f) & (fabsf(g[q].lo) >= 0x1p-126f);
  if (normal) {
#pragma unroll
    for (int q = 0; q < NV; ++q) f[q] = widen_normal(g[q].hi) + widen_normal(g[q].lo);
  } else {
#pragma unroll
    for (int q = 0; q < NV; ++q) f[q] = join(g[q]);
  }
}

}  // namespace lbx
