// Residual-mode entropic alpha solve, shared by the FP64 and the mixed
// precision kernels.
//
// Accept alpha when |F(alpha)| <= tol, F the entropy-balance function of
// EntropicStep.h:31-45. Phases: the guess (or the alternative guess when the
// first leaves its bracket), Newton from there (the update of
// EntropicStep.h:111-140), and when Newton leaves (1, alpha_max) or runs out
// of iterations, the safeguarded bisection-Newton of EntropicStep.h:142-220 on
// [1, alpha_max]; alpha = 2 when that fails too. Newton takes at most maxit
// steps and the bracketed solver bmaxit (maxit = 0 sends every node whose
// guess fails straight to the bracketed solver).
//
// The whole solve is one loop with a single evaluation site: F and F' cost Q
// FP64 logarithms, and one inlined copy of them keeps the kernel's code (its
// instruction-cache footprint and its compile time) small.
#pragma once

#include "common.cuh"

namespace mlbm {

// kFloatStep: Newton and bisection-Newton steps fe/de in FP32 (a step with a
// relative error of 1e-7 is still a convergent step; acceptance is decided by
// the FP64 residual alone).
template <int kFloatStep>
__device__ __forceinline__ double newton_step(double fe, double de) {
  if constexpr (kFloatStep) return widen_exact(__fdiv_rn(narrow_rn(fe), narrow_rn(de)));
  else return fe / de;
}

template <class Eval, bool kFloatStep = false>
__device__ __forceinline__ double residual_alpha_solve(const Eval& eval, double guess,
                                                       double alt, double alphaMax, double tol,
                                                       int maxit, int bmaxit, unsigned c[]) {
  enum { P_GUESS, P_NEWTON, P_LOW, P_HIGH, P_BISECT, P_DONE };
  int phase;
  double x;
  if (guess > 1.0 && guess < alphaMax) { x = guess; phase = P_GUESS; }
  else if (alt > 1.0 && alt < alphaMax) { x = alt; phase = P_NEWTON; }
  else { x = 1.0; phase = P_LOW; ++c[CNT_BISECT]; }
  unsigned iters = 0;
  int newton_left = maxit, bisect_left = bmaxit;
  bool first_bisect = true;
  double fLow = 0.0, xLow = 1.0, xHigh = alphaMax, dx = 0.0, dxOld = 0.0;
  double result = 2.0;
  bool ok = false;
  // one evaluation per pass: guess + maxit Newton + 2 bracket ends +
  // midpoint + bmaxit bisection steps at most
  for (int pass = 0; pass < maxit + bmaxit + 4 && phase != P_DONE; ++pass) {
    double fe, de;
    eval(x, fe, de);
    if (phase == P_GUESS || phase == P_NEWTON) {
      if (fabs(fe) <= tol) {
        if (phase == P_GUESS) ++c[CNT_HITS];
        result = x; ok = true; phase = P_DONE;
        continue;
      }
      phase = P_NEWTON;
      if (newton_left-- > 0) {
        ++iters;
        const double xn = x - newton_step<kFloatStep>(fe, de);
        if (xn > 1.0 && xn < alphaMax) { x = xn; continue; }
      }
      ++c[CNT_BISECT];
      x = 1.0;
      phase = P_LOW;
    } else if (phase == P_LOW) {
      fLow = fe;
      x = alphaMax;
      phase = P_HIGH;
    } else if (phase == P_HIGH) {
      // bracket check before either end is accepted (EntropicStep.h:151-164)
      if ((fLow > 0.0 && fe > 0.0) || (fLow < 0.0 && fe < 0.0)) { phase = P_DONE; continue; }
      if (fabs(fLow) <= tol) { result = 1.0; ok = true; phase = P_DONE; continue; }
      if (fabs(fe) <= tol) { result = alphaMax; ok = true; phase = P_DONE; continue; }
      if (fLow < 0.0) { xLow = 1.0; xHigh = alphaMax; } else { xLow = alphaMax; xHigh = 1.0; }
      x = 0.5 * (1.0 + alphaMax);
      dxOld = fabs(alphaMax - 1.0);
      dx = dxOld;
      phase = P_BISECT;
    } else {  // P_BISECT: fe, de at x
      if (!first_bisect) {
        if (fe < 0.0) xLow = x; else xHigh = x;
      }
      first_bisect = false;
      if (fabs(fe) <= tol) { result = x; ok = true; phase = P_DONE; continue; }
      if (bisect_left-- <= 0) { phase = P_DONE; continue; }
      ++iters;
      if ((((x - xHigh) * de - fe) * ((x - xLow) * de - fe) > 0.0) ||
          (fabs(2.0 * fe) > fabs(dxOld * de))) {
        dxOld = dx;
        dx = 0.5 * (xHigh - xLow);
        x = xLow + dx;
        if (xLow == x) { result = x; ok = true; phase = P_DONE; }
      } else {
        dxOld = dx;
        dx = newton_step<kFloatStep>(fe, de);
        const double xt = x;
        x -= dx;
        if (xt == x) { result = x; ok = true; phase = P_DONE; }
      }
    }
  }
  c[CNT_ITER] += iters;
  if (ok) return result;
  ++c[CNT_FALLBACK];
  return 2.0;
}

}  // namespace mlbm
