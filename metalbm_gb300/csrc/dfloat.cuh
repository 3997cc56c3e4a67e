// Double-float arithmetic: a value held as the unevaluated sum hi + lo of two
// floats (|lo| <= ulp(hi)/2, about 48 significant bits), built on the
// error-free transformations of T. J. Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18 (1971), and
// D. E. Knuth, TAOCP vol. 2, 4.2.2 (TwoSum). On GB300 FP32 runs at ~73x the
// FP64 rate, so a double-float operation (3 to 11 FP32 instructions) costs a
// fraction of an FP64 one in pipe time.
//
// Every operation uses the _rn intrinsics: they are never contracted into
// FMAs by the compiler, which would break the exactness of the
// transformations.
#pragma once

#include "common.cuh"

namespace mlbm {

struct dfl {
  float hi, lo;
};

// a + b = s + e exactly (TwoSum, 6 operations, no ordering condition)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// a + b = s + e exactly when |a| >= |b| or a = 0 (FastTwoSum, 3 operations)
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ dfl dfl_from(double x) {
  const float h = narrow_rn(x);
  return {h, narrow_rn(x - widen_exact(h))};
}

__device__ __forceinline__ double dfl_to_double(dfl a) {
  return widen_exact(a.hi) + widen_exact(a.lo);
}

__device__ __forceinline__ dfl dfl_add(dfl a, dfl b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  fast_two_sum(s, e, s, e);
  return {s, e};
}

__device__ __forceinline__ dfl dfl_neg(dfl a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ dfl dfl_sub(dfl a, dfl b) { return dfl_add(a, dfl_neg(b)); }

// a + b with b a float
__device__ __forceinline__ dfl dfl_add_f(dfl a, float b) {
  float s, e;
  two_sum(a.hi, b, s, e);
  e = __fadd_rn(e, a.lo);
  fast_two_sum(s, e, s, e);
  return {s, e};
}

__device__ __forceinline__ dfl dfl_mul(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);  // exact residual of the product
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  float s;
  fast_two_sum(p, e, s, e);
  return {s, e};
}

__device__ __forceinline__ dfl dfl_mul_f(dfl a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  float s;
  fast_two_sum(p, e, s, e);
  return {s, e};
}

// a * b + c
__device__ __forceinline__ dfl dfl_fma(dfl a, dfl b, dfl c) { return dfl_add(dfl_mul(a, b), c); }

// ---- two double-float values in packed FP32x2 lanes ---------------------------
// (hi.x + lo.x, hi.y + lo.y): every float operation of the functions above
// becomes one packed instruction for both values (GB300's FADD2 / FMUL2 /
// FFMA2, round to nearest like the scalar _rn intrinsics), so each lane
// computes exactly what the scalar function computes.
struct dfl2 {
  float2 hi, lo;
};

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 bcast2(float s) { return make_float2(s, s); }

__device__ __forceinline__ dfl2 dfl2_pack(dfl a, dfl b) {
  return {make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)};
}
__device__ __forceinline__ dfl dfl2_x(dfl2 a) { return {a.hi.x, a.lo.x}; }
__device__ __forceinline__ dfl dfl2_y(dfl2 a) { return {a.hi.y, a.lo.y}; }

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = add2(a, b);
  const float2 bb = sub2(s, a);
  e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

__device__ __forceinline__ void fast_two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = add2(a, b);
  e = sub2(b, sub2(s, a));
}

__device__ __forceinline__ dfl2 dfl2_add(dfl2 a, dfl2 b) {
  float2 s, e;
  two_sum2(a.hi, b.hi, s, e);
  e = add2(e, add2(a.lo, b.lo));
  fast_two_sum2(s, e, s, e);
  return {s, e};
}

__device__ __forceinline__ dfl2 dfl2_neg(dfl2 a) { return {neg2(a.hi), neg2(a.lo)}; }

__device__ __forceinline__ dfl2 dfl2_sub(dfl2 a, dfl2 b) { return dfl2_add(a, dfl2_neg(b)); }

// a + b with b a pair of floats
__device__ __forceinline__ dfl2 dfl2_add_f(dfl2 a, float2 b) {
  float2 s, e;
  two_sum2(a.hi, b, s, e);
  e = add2(e, a.lo);
  fast_two_sum2(s, e, s, e);
  return {s, e};
}

__device__ __forceinline__ dfl2 dfl2_mul(dfl2 a, dfl2 b) {
  const float2 p = mul2(a.hi, b.hi);
  float2 e = fma2(a.hi, b.hi, neg2(p));
  e = fma2(a.hi, b.lo, fma2(a.lo, b.hi, e));
  float2 s;
  fast_two_sum2(p, e, s, e);
  return {s, e};
}

__device__ __forceinline__ dfl2 dfl2_mul_f(dfl2 a, float2 b) {
  const float2 p = mul2(a.hi, b);
  float2 e = fma2(a.hi, b, neg2(p));
  e = fma2(a.lo, b, e);
  float2 s;
  fast_two_sum2(p, e, s, e);
  return {s, e};
}

}  // namespace mlbm
