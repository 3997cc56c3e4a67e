// FP64 natural logarithm and log1p for the entropy function.
//
// ln(x), table-driven after P. T. P. Tang, "Table-driven implementation of
// the logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4),
// 1990: write x = 2^e m with m in [1, 2); j = the top 7 fraction bits of m;
// inv_j = RN(1 / c_j) for the centre c_j = 1 + (j + 1/2)/128 of m's interval;
// r = m inv_j - 1 with a single rounding (one FMA), |r| < 0.0045;
// ln x = e ln2 + ln(1/inv_j) + log1p(r), with ln(1/inv_j) and ln2 held as
// double-double constants and log1p(r) a degree-7 Taylor polynomial
// (truncation < 2e-20). The absolute error is a few ulp of ln 2 for any
// positive normal or subnormal x (the relative error grows only where
// ln x -> 0, which the entropy sums, weighted by f ~ 1e-2, do not see).
//
// The table (128 x {inv, hi, lo}) is built on the host in extended precision
// by make_log_table() and staged into shared memory by each block.
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace mlbm {

constexpr int LOG_TABLE = 128;

struct LogEntry {
  double inv;  // RN(1 / c_j)
  double hi;   // -ln(inv) = ln(1/inv), leading part
  double lo;   // trailing part
};

// ln 2 split so that e * kLn2Hi is exact for |e| < 2^11 (kLn2Hi has 42
// significant bits): kLn2Hi + kLn2Lo = ln 2 to ~1e-29.
constexpr double kLn2Hi = 0x1.62e42fefa3800p-1;
constexpr double kLn2Lo = 0x1.ef35793c76730p-45;
constexpr double kLn2 = 0x1.62e42fefa39efp-1;  // RN(ln 2)

// Degree-7 Taylor polynomial of log1p(r) = r - r^2/2 + r^3/3 - ... - r^8/8,
// truncated after r^7 (|r| < 0.0045 gives |r|^8/8 < 2e-20).
__device__ __forceinline__ double log1p_series7(double r) {
  double p = 1.0 / 7.0;
  p = fma(p, r, -1.0 / 6.0);
  p = fma(p, r, 1.0 / 5.0);
  p = fma(p, r, -1.0 / 4.0);
  p = fma(p, r, 1.0 / 3.0);
  p = fma(p, r, -0.5);
  return fma(p * r, r, r);
}

// log1p(t) for |t| <= 2^-6 by its Taylor series to t^9 (truncation
// |t|^10/10 < 1e-19 relative to t).
__device__ __forceinline__ double log1p_small(double t) {
  double p = 1.0 / 9.0;
  p = fma(p, t, -1.0 / 8.0);
  p = fma(p, t, 1.0 / 7.0);
  p = fma(p, t, -1.0 / 6.0);
  p = fma(p, t, 1.0 / 5.0);
  p = fma(p, t, -1.0 / 4.0);
  p = fma(p, t, 1.0 / 3.0);
  p = fma(p, t, -0.5);
  return fma(p * t, t, t);
}

// log1p(t) for |t| <= 2^-10 by its Taylor series to t^5 (truncation
// |t|^6/6 < 3e-19).
__device__ __forceinline__ double log1p_tiny(double t) {
  double p = 1.0 / 5.0;
  p = fma(p, t, -1.0 / 4.0);
  p = fma(p, t, 1.0 / 3.0);
  p = fma(p, t, -0.5);
  return fma(p * t, t, t);
}

// ln(x) for x > 0 (finite). `tab` is the shared-memory table.
__device__ __forceinline__ double fast_log(double x, const LogEntry* tab) {
  int64_t bits = __double_as_longlong(x);
  int e = (int)((bits >> 52) & 0x7ff);
  if (e == 0) {  // subnormal: scale by 2^54
    bits = __double_as_longlong(x * 18014398509481984.0);
    e = (int)((bits >> 52) & 0x7ff) - 54;
  }
  e -= 1023;
  const int j = (int)((bits >> 45) & (LOG_TABLE - 1));
  const double m = __longlong_as_double((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  const LogEntry t = tab[j];
  const double r = fma(m, t.inv, -1.0);
  const double ed = (double)e;
  const double hi = fma(ed, kLn2Hi, t.hi);  // exact product, one rounding in the sum
  const double lo = fma(ed, kLn2Lo, t.lo) + log1p_series7(r);
  return hi + lo;
}

// The exponent e as a double without a conversion instruction (integer to
// FP64 conversion runs on GB300's narrow FP64 path): the bit pattern of
// 1.5 * 2^52 + e, minus 1.5 * 2^52, exact for |e| < 2^51.
__device__ __forceinline__ double exponent_as_double(int e) {
  return __longlong_as_double(0x4338000000000000LL + (long long)e) - 6755399441055744.0;
}

// ln(x) to about 1e-15 absolute for positive normal or subnormal x: the same
// reduction as fast_log without the double-double tails, and a degree-5
// series (truncation |r|^6/6 < 6e-16 for |r| <= 2^-8). For sums weighted by
// small factors (B1 = sum f_neq ln(f/w) of the entropy function), where the
// error is multiplied by sum |f_neq| <= rho max|f_neq/f|.
__device__ __forceinline__ double fast_log_short(double x, const LogEntry* tab) {
  int64_t bits = __double_as_longlong(x);
  int e = (int)((bits >> 52) & 0x7ff);
  if (e == 0) {
    bits = __double_as_longlong(x * 18014398509481984.0);
    e = (int)((bits >> 52) & 0x7ff) - 54;
  }
  e -= 1023;
  const int j = (int)((bits >> 45) & (LOG_TABLE - 1));
  const double m = __longlong_as_double((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  const LogEntry t = tab[j];
  const double r = fma(m, t.inv, -1.0);
  double p = 1.0 / 5.0;
  p = fma(p, r, -1.0 / 4.0);
  p = fma(p, r, 1.0 / 3.0);
  p = fma(p, r, -0.5);
  const double lp = fma(p * r, r, r);
  return fma(exponent_as_double(e), kLn2, t.hi) + lp;
}

// Finer table for ln(x) inside the moment-series tier of the entropy function:
// 1024 intervals, entry {RN(1/c_j), RN(ln(1/inv_j))}, c_j = 1 + (j + 1/2)/1024.
constexpr int LOG_TABLE_FINE = 1024;
struct LogEntryFine {
  double inv;
  double hi;
};

// ln(x) with |r| <= 2^-11 after the reduction and
// log1p(r) = r + r^2 (r/3 - 1/2) + O(r^4), the r^2 tail in FP32:
// |tail| <= 1.2e-7 with a relative error of a few float roundings, so the
// result is within 5e-14 of ln(x) (truncation r^4/4 <= 1.4e-14 included).
// Used for B1 = sum f_neq ln(f/w) when max|f_neq/f| <= 0.0125, where the
// error is multiplied by sum |f_neq| <= 0.0125 rho.
__device__ __forceinline__ double fast_log_fine(double x, const LogEntryFine* tab) {
  int64_t bits = __double_as_longlong(x);
  int e = (int)((bits >> 52) & 0x7ff);
  if (e == 0) {
    bits = __double_as_longlong(x * 18014398509481984.0);
    e = (int)((bits >> 52) & 0x7ff) - 54;
  }
  e -= 1023;
  const int j = (int)((bits >> 42) & (LOG_TABLE_FINE - 1));
  const double m = __longlong_as_double((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  const LogEntryFine t = tab[j];
  const double r = fma(m, t.inv, -1.0);
  const float rf = narrow_rn(r);
  const float tail = (rf * rf) * fmaf(rf, 1.0f / 3.0f, -0.5f);
  return fma(exponent_as_double(e), kLn2, t.hi) + (r + widen_exact(tail));
}

// The fine table is followed in device memory by the lattice's constants
// C_q(d) = d ln 2 - ln(m_q), d = -1, 0, 1, at [3 q + d + 1], where w_q = m_q 2^e_q
// with m_q in [1, 2): ln(f_q / w_q) = C_q(d) + ln(mantissa of f_q) for
// d = exponent(f_q) - e_q.
constexpr int LNW_CONSTS = 81;

__device__ __forceinline__ void stage_log_table_fine(LogEntryFine* sh, double* sh_lnw,
                                                     const LogEntryFine* __restrict__ g) {
  for (int i = threadIdx.x; i < LOG_TABLE_FINE; i += blockDim.x) sh[i] = g[i];
  const double* c = reinterpret_cast<const double*>(g + LOG_TABLE_FINE);
  for (int i = threadIdx.x; i < LNW_CONSTS; i += blockDim.x) sh_lnw[i] = c[i];
}

// Float companion of the fine table for the double-float evaluation of B1
// (FP32 storage, whose populations are floats): inv = RN_float(1/c_j) and
// ln(1/inv) as a float pair hi + lo (about 48 significant bits). For a float
// mantissa m in the j-th interval, m inv - 1 = (RN(m inv) - 1) + the FMA
// residual exactly, |m inv - 1| < 4.9e-4.
struct LogEntryFineF {
  float inv, hi, lo, pad;
};

// Device layout of the fine tables (built on the host): the FP64 table and
// the lattice's constants C_q(d) (FP64), then the float table and -ln(m_q) of
// each population's weight significand as float pairs.
struct FineTables {
  LogEntryFine t[LOG_TABLE_FINE];
  double lnw[LNW_CONSTS];
  double pad;
  LogEntryFineF tf[LOG_TABLE_FINE];
  float lnwf[27][2];
};

__device__ __forceinline__ void stage_log_table_fine_f(LogEntryFineF* sh, float2* sh_c,
                                                       const FineTables* __restrict__ g) {
  const float4* src = reinterpret_cast<const float4*>(g->tf);
  float4* dst = reinterpret_cast<float4*>(sh);
  for (int i = threadIdx.x; i < LOG_TABLE_FINE; i += blockDim.x) dst[i] = src[i];
  for (int i = threadIdx.x; i < 27; i += blockDim.x) sh_c[i] = make_float2(g->lnwf[i][0], g->lnwf[i][1]);
}

// Binary exponent e of a positive constant w = m 2^e, m in [1, 2).
__host__ __device__ constexpr int exponent_of(double w) {
  int e = 0;
  while (w >= 2.0) { w *= 0.5; ++e; }
  while (w < 1.0) { w *= 2.0; --e; }
  return e;
}

// Block-cooperative staging of the table into shared memory.
__device__ __forceinline__ void stage_log_table(LogEntry* sh, const LogEntry* __restrict__ g) {
  for (int i = threadIdx.x; i < LOG_TABLE; i += blockDim.x) sh[i] = g[i];
}

}  // namespace mlbm
