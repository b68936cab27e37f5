// Double-single ("float-float") arithmetic: a value is the unevaluated sum
// hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2, about 48 significant
// bits.  GB300 runs FP32 at 64x its FP64 rate, so the FP32C path's transforms
// and w-screens use these instead of FP64.
//
// Published algorithms, written out here from the mathematics:
//   two_sum       Knuth, TAOCP vol. 2, 4.2.2 (error-free sum, 6 operations)
//   quick_two_sum Dekker 1971, "A floating-point technique for extending the
//                 available precision" (|a| >= |b|, 3 operations)
//   two_prod      the error-free product through one FMA
//   ds_sqrt       one Newton step on an FP32 root (Karp and Markstein, 1997)
//   ds_div        one correction step on an FP32 quotient
// Every FP32 operation is an explicit round-to-nearest intrinsic so the
// compiler cannot contract or reorder the error terms away.
#pragma once
#include <cuda_runtime.h>

namespace arlgpu {

struct dsf {
  float hi, lo;
};

__device__ __forceinline__ dsf two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
  return {s, e};
}

__device__ __forceinline__ dsf quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dsf two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ dsf ds_add(dsf a, dsf b) {
  const dsf s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ dsf ds_neg(dsf a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ dsf ds_sub(dsf a, dsf b) { return ds_add(a, ds_neg(b)); }

__device__ __forceinline__ dsf ds_mul(dsf a, dsf b) {
  const dsf p = two_prod(a.hi, b.hi);
  const float e = __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.lo, p.lo));
  return quick_two_sum(p.hi, e);
}

__device__ __forceinline__ dsf ds_mul_f(dsf a, float b) {
  const dsf p = two_prod(a.hi, b);
  return quick_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}

// sqrt(a), a > 0: s0 = sqrtf(a.hi), s = s0 + (a - s0^2) / (2 s0).
__device__ __forceinline__ dsf ds_sqrt(dsf a) {
  if (!(a.hi > 0.f)) return {0.f, 0.f};
  const float s0 = sqrtf(a.hi);
  const dsf sq = two_prod(s0, s0);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, sq.hi), sq.lo), a.lo);
  return quick_two_sum(s0, __fdiv_rn(r, __fmul_rn(2.f, s0)));
}

// a / b: q0 = a.hi / b.hi, q = q0 + (a - q0 b) / b.hi.
__device__ __forceinline__ dsf ds_div(dsf a, dsf b) {
  const float q0 = __fdiv_rn(a.hi, b.hi);
  const dsf qb = ds_mul_f(b, q0);
  const dsf r = ds_sub(a, qb);
  return quick_two_sum(q0, __fdiv_rn(r.hi, b.hi));
}

// Exact split of an integer |n| < 2^48.
__device__ __forceinline__ dsf ds_from_i64(long long n) {
  const float hi = (float)n;  // round to nearest
  return {hi, (float)(n - (long long)hi)};
}

__device__ __forceinline__ dsf ds_from_double(double x) {
  const float hi = __double2float_rn(x);
  return {hi, __double2float_rn(x - (double)hi)};
}

__device__ __forceinline__ double ds_to_double(dsf a) { return (double)a.hi + (double)a.lo; }

// w-screen phase of create_w_term_like at one pixel, in double-single:
// nterm = 1 - sqrt(1 - r^2), r^2 = c2 ((y - n/2)^2 + (x - n/2)^2) with
// c2 = fov^2 / n^2 (split from FP64).  The subtraction loses relative accuracy
// only where nterm is small, and there the phase w nterm is small too: its
// absolute error stays ~1e-14 w.
// state 0: r^2 == 0 (screen 1), 1: inside, 2: r^2 >= 1 (screen 0).
struct DsPix {
  dsf nterm;
  int state;
};
__device__ __forceinline__ DsPix ds_wpix(int y, int x, int n, dsf c2) {
  const long long dy = y - n / 2, dx = x - n / 2;
  const long long R = dy * dy + dx * dx;
  DsPix p;
  p.nterm = {0.f, 0.f};
  if (R == 0) {
    p.state = 0;
    return p;
  }
  const dsf r2 = ds_mul(c2, ds_from_i64(R));
  if (r2.hi > 1.f || (r2.hi == 1.f && r2.lo >= 0.f)) {
    p.state = 2;
    return p;
  }
  p.nterm = ds_sub({1.f, 0.f}, ds_sqrt(ds_sub({1.f, 0.f}, r2)));
  p.state = 1;
  return p;
}

// exp(-2 pi i w nterm) with the phase in turns reduced in double-single
// before an FP32 sincospi: the phase error is FP32 rounding of the reduced
// argument (< 1e-7 rad) for any w.
__device__ __forceinline__ float2 ds_wbeam(const DsPix &p, dsf w) {
  if (p.state == 0) return make_float2(1.f, 0.f);
  if (p.state == 2) return make_float2(0.f, 0.f);
  const dsf t = ds_mul(w, p.nterm);
  const float f = __fadd_rn(__fsub_rn(t.hi, rintf(t.hi)), t.lo);
  float s, c;
  sincospif(-2.f * f, &s, &c);
  return make_float2(c, s);
}

}  // namespace arlgpu
