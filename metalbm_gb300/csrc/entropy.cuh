// The entropy-balance function of the residual-mode alpha solve, shared by
// the FP64-storage and FP32/FP16-storage entropic kernels.
#pragma once

#include "common.cuh"
#include "fastlog.cuh"
#include "lattice.cuh"

namespace mlbm {

// Entropy-balance function in log1p form. With r_q = f_neq_q / f_q and
// t_q = -x r_q (so g_q = f_q (1 + t_q)), ln(g_q/w_q) = L_q + log1p(t_q) where
// L_q = ln(f_q/w_q), and F(x) = sum f ln(f/w) - sum g ln(g/w) of
// EntropicStep.h:31-45 becomes
//   F(x)  = x B1 - sum_q f_q (1 + t_q) log1p(t_q),   B1 = sum_q f_neq_q L_q,
//   F'(x) = C0 + sum_q f_q r_q log1p(t_q),           C0 = sum_q f_neq_q + B1
// (the derivative of EntropicStep.h:47-62). The L_q are computed once per node;
// an evaluation then needs log1p of |t| <= 2^-6 only (a short series), with a
// full logarithm only for larger deviations. The two sums are O(|f_neq|)
// instead of the O(1) terms of the direct form, so F is also better
// conditioned.
template <int LAT>
struct HLog1p {
  const double* f;
  const double* r;
  double B1, C0;
  double rmax;  // max_q |r_q|
  const LogEntry* tab;
  __device__ __forceinline__ void operator()(double x, double& Fv, double& Dv) const {
    using L = Lattice<LAT>;
    double s = 0.0, d = 0.0;
    if (x * rmax <= 0.0009765625) {
      // every |t| <= 2^-10: degree-5 series, truncation < |t|^6/6 < 3e-19
#pragma unroll
      for (int q = 0; q < L::Q; ++q) {
        const double t = -x * r[q];
        const double lp = log1p_tiny(t);
        s = fma(fma(f[q], t, f[q]), lp, s);
        d = fma(f[q] * r[q], lp, d);
      }
    } else {
#pragma unroll
      for (int q = 0; q < L::Q; ++q) {
        const double t = -x * r[q];
        const double opt = 1.0 + t;
        double lp;
        if (fabs(t) <= 0.015625) lp = log1p_small(t);
        else if (opt > 0.0) lp = fast_log(opt, tab);
        else lp = -745.0;  // g = 0 at alpha_max: g ln g -> 0
        if (opt > 0.0) s = fma(f[q] * opt, lp, s);
        d = fma(f[q] * r[q], lp, d);
      }
    }
    Fv = fma(x, B1, -s);
    Dv = C0 + d;
  }
};

// Moment-series form of the same function for small deviations. With
// (1 + t) log1p(t) = t + sum_{k>=2} (-1)^k t^k / (k (k - 1)), t_q = -x r_q,
// and the moments M_k = sum_q f_q r_q^k (M_1 = sum_q f_neq_q = 0 for the
// TruncationMa3 equilibrium of all three lattices, whose weights make
// sum_q w_q P_q(u) vanish identically):
//   F(x)  = x B1 - sum_{k>=2} x^k M_k / (k (k - 1)),
//   F'(x) = B1   - sum_{k>=2} x^(k-1) M_k / (k - 1).
// Kept to k = 8, which is accurate to |F error| <= rho (2.5 r)^9 / 72 < 5e-16
// for x <= alpha_max <= 2.5 and r = max_q |r_q| <= kSeriesRmax. M_2..M_4 are
// FP64 sums; M_5..M_8 are FP32 sums, whose terms are bounded by
// 4.9 r^3 M_2 and lose at most 1.6e-6 of that (< 3e-15 absolute at the limit).
// An evaluation is then a handful of FP64 operations instead of Q logarithms
// or series.
constexpr float kSeriesRmax = 0.0125f;

struct HSeries {
  double c1;          // B1
  double a2, a3, a4;  // M2/2, M3/6, M4/12
  double b2, b3, b4;  // M2,   M3/2, M4/3
  float h5, h6, h7, h8;  // M5/20, M6/30, M7/42, M8/56
  float g5, g6, g7, g8;  // M5/4,  M6/5,  M7/6,  M8/7
  __device__ __forceinline__ void operator()(double x, double& Fv, double& Dv) const {
    const float xf = narrow_rn(x);
    const float x2f = xf * xf;
    const float x4f = x2f * x2f;
    const float h = fmaf(fmaf(fmaf(h8, xf, h7), xf, h6), xf, h5) * (x4f * xf);
    const float g = fmaf(fmaf(fmaf(g8, xf, g7), xf, g6), xf, g5) * x4f;
    const double p = fma(fma(a4, x, a3), x, a2);
    const double q = fma(fma(b4, x, b3), x, b2);
    Fv = fma(x, c1, -fma(x * x, p, widen_exact(h)));
    Dv = fma(-x, q, c1 - widen_exact(g));
  }
};

// L_q, B1, C0 and r_q of a node (27 logarithms, 27 divisions).
template <int LAT>
__device__ __forceinline__ HLog1p<LAT> make_hlog1p(const double f[], const double fn[], double r[],
                                                   const LogEntry* tab) {
  using L = Lattice<LAT>;
  double B1 = 0.0, sfn = 0.0, rmax = 0.0;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    B1 = fma(fn[q], fast_log(f[q] * (1.0 / L::w(q)), tab), B1);
    sfn += fn[q];
    r[q] = fn[q] / f[q];
    rmax = fmax(rmax, fabs(r[q]));
  }
  return HLog1p<LAT>{f, r, B1, sfn + B1, rmax, tab};
}

// The same with r_q given (the caller already formed them).
template <int LAT>
__device__ __forceinline__ HLog1p<LAT> make_hlog1p_r(const double f[], const double fn[],
                                                     const double r[], double rmax,
                                                     const LogEntry* tab) {
  using L = Lattice<LAT>;
  double B1 = 0.0, sfn = 0.0;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    B1 = fma(fn[q], fast_log(f[q] * (1.0 / L::w(q)), tab), B1);
    sfn += fn[q];
  }
  return HLog1p<LAT>{f, r, B1, sfn + B1, rmax, tab};
}

}  // namespace mlbm
