// FP64 fused collide-and-stream pull kernels, bit-compatible with the reference.
//
// This translation unit is compiled with -fmad=false: every multiply and add
// below is a separately rounded IEEE operation in the reference's order
// (left-to-right evaluation of the cited C++ expressions), so BGK results are
// bit-identical to the reference CPU build. Rearrangements used here are
// exact: products by +-1 are sign changes, additions of the zero products of
// c_d = 0 are dropped (x + 0 = x), and the odd/even powers of c.u are shared
// between the populations q and -q (c.u changes sign exactly).
//
// One thread per node; populations are SoA, population q of node i at
// q*V + i, i = (x*Ly + y)*Lz + z (the reference's node order, z contiguous),
// so a warp's loads of one population are 32 consecutive doubles shifted by
// at most one element. The periodic wrap is the index arithmetic of
// PullOffsets (replaces Communication.h:134-180 and Boundary.h:50-100).

#include "common.cuh"
#include "kernels.h"
#include "entropy.cuh"
#include "solver.cuh"

namespace mlbm {

// ---- c . v with the reference's dot order (MathVector.h:45-53) ----------
template <int LAT>
__device__ __forceinline__ double cdot(int q, const double v[3]) {
  using L = Lattice<LAT>;
  double r = 0.0;
  bool any = false;
#pragma unroll
  for (int d = 0; d < L::D; ++d) {
    const int c = L::c(q, d);
    if (c != 0) {
      // c v with c = +-1 is a sign change, with c = +-2 an exact doubling
      const double t = c == 1 ? v[d] : (c == -1 ? -v[d] : (double)c * v[d]);
      r = any ? r + t : t;
      any = true;
    }
  }
  return r;
}

// Node-invariant part of Equilibrium<TruncationMa3> (Equilibrium.h:17-33).
struct EqNode {
  double rho, u2, t2, t6;
};
template <int LAT>
__device__ __forceinline__ EqNode eq_node(double rho, double u2) {
  using K = EqConst<LAT>;
  EqNode e;
  e.rho = rho;
  e.u2 = u2;
  e.t2 = 0.5 * u2 * K::ics;
  e.t6 = 0.125 * u2 * u2 * K::p2;
  return e;
}

// Equilibrium of the pair (q, -q) from cu = c_q . u, with k = inv_cs2:
//   fEq = 1 + k cu - k/2 u2 + k^2/2 cu^2 - k^2/2 cu u2 + k^3/6 cu^3
//         + k^2/8 u2^2 - k^3/4 cu^2 u2 + k^4/24 cu^4,
// each term as the reference forms it (k = 3: 4.5, 27/6, 6.75, 81/24).
template <int LAT>
__device__ __forceinline__ void eq_pair(const EqNode& e, double cu, double rw_plus,
                                        double rw_minus, double& feq_plus, double& feq_minus) {
  using K = EqConst<LAT>;
  const double t1 = cu * K::ics;
  const double a = K::half_p2 * cu;
  const double t3 = a * cu;
  const double t4 = a * e.u2;
  const double c3 = cu * cu * cu;
  const double t5 = c3 * K::p3 / 6.0;
  const double t7 = 0.25 * cu * cu * e.u2 * K::p3;
  const double t8 = c3 * cu * K::p4 / 24.0;
  const double sp = 1.0 + t1 - e.t2 + t3 - t4 + t5 + e.t6 - t7 + t8;
  const double sm = 1.0 - t1 - e.t2 + t3 + t4 - t5 + e.t6 - t7 + t8;
  feq_plus = rw_plus * sp;
  feq_minus = rw_minus * sm;
}

__device__ __forceinline__ double eq_rest(const EqNode& e, double rw) {
  // cu = 0: fEq = ((1 - t2) + t6), all other terms are exact zeros.
  return rw * (1.0 - e.t2 + e.t6);
}

template <int LAT>
__device__ __forceinline__ void equilibria(double rho, const double u[3], double u2,
                                           double feq[Lattice<LAT>::Q]) {
  using L = Lattice<LAT>;
  const EqNode e = eq_node<LAT>(rho, u2);
  feq[0] = eq_rest(e, rho * L::w(0));
#pragma unroll
  for (int q = 1; q < L::Q; ++q) {
    if (is_pair_leader<LAT>(q)) {
      const int qb = opposite<LAT>(q);
      eq_pair<LAT>(e, cdot<LAT>(q, u), rho * L::w(q), rho * L::w(qb), feq[q], feq[qb]);
    }
  }
}

// Source term S_q of the forcing scheme (ForcingScheme.h:41-198).
template <int LAT, int FS>
__device__ __forceinline__ double source(const StepParams& p, int q, double rho, const double u[3],
                                         const double F[3], double cu3, double eq_q,
                                         const double* feq_shift) {
  using L = Lattice<LAT>;
  if (FS == FS_GUO) {
    // ((c - u) + (inv_cs2 c.u) c) . F, then ((1 - 1/(2 tau)) w) inv_cs2 * R;
    // cu3 = inv_cs2 c.u, and (cu3) c is exact for c = +-1, +-2
    double v[3];
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      const int c = L::c(q, d);
      const double cmu = c == 0 ? -u[d] : (double)c - u[d];
      v[d] = c == 0 ? cmu : cmu + (c == 1 ? cu3 : (c == -1 ? -cu3 : (double)c * cu3));
    }
    double R = v[0] * F[0];
#pragma unroll
    for (int d = 1; d < L::D; ++d) R = R + v[d] * F[d];
    return p.guo_k[q] * R;
  } else if (FS == FS_EDM) {
    return feq_shift[q] - eq_q;
  }
  return 0.0;
}

template <int LAT>
__device__ __forceinline__ void pull(const double* __restrict__ prev, long long V,
                                     const PullOffsetsR<Lattice<LAT>::R>& o,
                                     double f[Lattice<LAT>::Q]) {
  using L = Lattice<LAT>;
#pragma unroll
  for (int q = 0; q < L::Q; ++q)
    f[q] = __ldg(pop(prev, V, q) + o.at(L::c(q, 0), L::c(q, 1), L::c(q, 2)));
}

// rho = f0 + f1 + ... ; u_d = sum_q c_qd f_q ; u /= rho (Moment.h:13-47)
template <int LAT>
__device__ __forceinline__ void moments(const double f[Lattice<LAT>::Q], double& rho,
                                        double u[3]) {
  using L = Lattice<LAT>;
  rho = f[0];
#pragma unroll
  for (int q = 1; q < L::Q; ++q) rho = rho + f[q];
#pragma unroll
  for (int d = 0; d < 3; ++d) u[d] = 0.0;
#pragma unroll
  for (int d = 0; d < L::D; ++d) {
    double s = 0.0;
    bool any = false;
#pragma unroll
    for (int q = 1; q < L::Q; ++q) {
      const int c = L::c(q, d);
      if (c != 0) {
        const double t = c == 1 ? f[q] : (c == -1 ? -f[q] : (double)c * f[q]);
        s = any ? s + t : t;
        any = true;
      }
    }
    u[d] = s / rho;
  }
}

template <int LAT>
__device__ __forceinline__ double norm2(const double v[3]) {
  double r = v[0] * v[0];
#pragma unroll
  for (int d = 1; d < Lattice<LAT>::D; ++d) r = r + v[d] * v[d];
  return r;
}

// EDM: f_eq(rho, u + F/rho) for every q (ForcingScheme.h:183-197).
template <int LAT, int FS>
__device__ __forceinline__ void shifted_equilibria(double rho, const double u[3], const double F[3],
                                                   double out[Lattice<LAT>::Q]) {
  if (FS != FS_EDM) return;
  const double inv = 1.0 / rho;
  double v[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int d = 0; d < Lattice<LAT>::D; ++d) v[d] = u[d] + F[d] * inv;
  equilibria<LAT>(rho, v, norm2<LAT>(v), out);
}

template <int LAT>
__device__ __forceinline__ void store_node_fields(const StepParams& p, long long idx, double rho,
                                                  const double u[3], const double F[3],
                                                  bool shifted, double alpha, double& energy,
                                                  double& mach) {
  using L = Lattice<LAT>;
  double uh[3] = {0.0, 0.0, 0.0};
  const double h = 0.5 / rho;
#pragma unroll
  for (int d = 0; d < L::D; ++d) uh[d] = shifted ? u[d] + F[d] * h : u[d];
  if (p.store) {
    p.rho_out[idx] = rho;
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      p.u_out[(long long)d * p.V + idx] = uh[d];
      p.force_out[(long long)d * p.V + idx] = F[d];
    }
    if (p.alpha_field) p.alpha_field[idx] = alpha;
  }
  if (p.diag) {
    energy = 0.0;
#pragma unroll
    for (int d = 0; d < L::D; ++d) energy = energy + 0.5 * rho * uh[d] * uh[d];
    mach = L::ics * norm2<LAT>(uh);  // |u|^2 / c_s^2; the square root is taken once, in finalize_diag
  }
}

// ---- BGK (Collision.h:103-180 + Algorithm.h:97-126) ----------------------
template <int LAT, int FS>
__global__ void __launch_bounds__(256) bgk_f64_kernel(const double* __restrict__ prev,
                                                      double* __restrict__ next, StepParams p) {
  using L = Lattice<LAT>;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = idx < p.V;
  double mass = 0.0, energy = 0.0, mach = 0.0;
  if (active) {
    uint32_t x, y, z;
    node_coords(p, idx, x, y, z);
    const auto o = pull_offsets_r<L::R>(p, x, y, z);
    double f[L::Q];
    pull<LAT>(prev, p.V, o, f);
    double rho, u[3];
    moments<LAT>(f, rho, u);
    const double u2 = norm2<LAT>(u);
    double F[3];
    node_force<L::D>(p, x, y, z, F);
    double feq[L::Q];
    equilibria<LAT>(rho, u, u2, feq);
    double fsh[FS == FS_EDM ? L::Q : 1];
    shifted_equilibria<LAT, FS>(rho, u, F, fsh);
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      const double cu3 = cdot<LAT>(q, u) * L::ics;
      double r = p.bgk_a * f[q] + p.bgk_b * feq[q];
      if (FS == FS_GUO || FS == FS_EDM) r = r + source<LAT, FS>(p, q, rho, u, F, cu3, feq[q], fsh);
      pop(next, p.V, q)[(uint32_t)idx] = r;
    }
    if (!(rho > 0.0) || !isfinite(rho)) atomicOr(p.err_word, ERR_NONFINITE);
    mass = rho;
    store_node_fields<LAT>(p, idx, rho, u, F, FS != FS_NONE, 2.0, energy, mach);
  }
  if (p.diag) block_reduce_diag(mass, energy, mach, 2.0, 2.0, p.diag_partials);
}

// ---- Entropic SRT (Collision.h:182-376, EntropicStep.h:15-220) ----------
// Reference-mode Newton (EntropicStep.h:111-140). f ln(f/w) is formed once
// per node; F and F' per iterate reuse ln(g/w) (the reference evaluates the
// same logarithms, in the same order, in its two functor calls).
template <int LAT>
__device__ __forceinline__ bool newton_reference(const double f[], const double fneq[],
                                                 const double flf[], double tol, int maxit,
                                                 double& xR, double xMin, double xMax,
                                                 unsigned& iters) {
  using L = Lattice<LAT>;
  double xStep = 0.0;
  for (int it = 1; it <= maxit; ++it) {
    xR = xR - xStep;
    double Fv = 0.0, Dv = 0.0;
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      const double g = f[q] - xR * fneq[q];
      const double lg = log(g / L::w(q));
      Fv = Fv + (flf[q] - g * lg);
      Dv = Dv + fneq[q] * (1 + lg);
    }
    ++iters;
    xStep = Fv / Dv;
    if (fabs(xStep) <= tol) return xR > xMin && xR < xMax;
  }
  return false;
}

// ELBM::calculateAlpha (Collision.h:351-375) in either solver mode. c[] holds
// the solver counters of this thread.
template <int LAT>
__device__ __forceinline__ double entropic_alpha(const StepParams& p, const double f[],
                                                 const double fneq[], double guess, unsigned c[],
                                                 const LogEntry* tab) {
  using L = Lattice<LAT>;
  bool small = true;
#pragma unroll
  for (int q = 0; q < L::Q; ++q)
    if (fabs(fneq[q]) / f[q] > p.deviation_threshold) small = false;
  if (small) { ++c[CNT_SHORTCUT]; return 2.0; }
  double alphaMax = 2.5;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    if (fneq[q] > 0) {
      const double t = fabs(f[q]) / fneq[q];
      if (t < alphaMax) alphaMax = t;
    }
  }
  if (alphaMax < 2.) { ++c[CNT_LIMITED]; return 0.95 * alphaMax; }
  ++c[CNT_SOLVED];
  if (p.guess_mode == GUESS_TWO) guess = 2.0;
  unsigned iters = 0;
  double alpha = guess;
  if (p.alpha_mode == ALPHA_REFERENCE) {
    double flf[L::Q];
#pragma unroll
    for (int q = 0; q < L::Q; ++q) flf[q] = f[q] * log(f[q] / L::w(q));
    const bool ok = newton_reference<LAT>(f, fneq, flf, p.newton_tol, p.newton_maxit, alpha, 1.,
                                          alphaMax, iters);
    c[CNT_ITER] += iters;
    if (ok) return alpha;
    ++c[CNT_FALLBACK];
    return 2.0;
  }
  double r[L::Q];
  const HLog1p<LAT> ev = make_hlog1p<LAT>(f, fneq, r, tab);
  return residual_alpha_solve(ev, guess, guess, alphaMax, p.newton_tol, p.newton_maxit,
                              p.bisect_maxit, c);
}

template <int LAT, int FS>
__global__ void __launch_bounds__(128) elbm_f64_kernel(const double* __restrict__ prev,
                                                       double* __restrict__ next, StepParams p) {
  using L = Lattice<LAT>;
  __shared__ LogEntry s_log[LOG_TABLE];
  stage_log_table(s_log, reinterpret_cast<const LogEntry*>(p.log_table));
  __syncthreads();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = idx < p.V;
  double mass = 0.0, energy = 0.0, mach = 0.0, amin = 1e300, amax = -1e300;
  unsigned cnt[CNT_COUNT] = {};
  if (active) {
    uint32_t x, y, z;
    node_coords(p, idx, x, y, z);
    const auto o = pull_offsets_r<L::R>(p, x, y, z);
    double f[L::Q];
    pull<LAT>(prev, p.V, o, f);
    double rho, u[3];
    moments<LAT>(f, rho, u);
    const double u2 = norm2<LAT>(u);
    double F[3];
    node_force<L::D>(p, x, y, z, F);
    double fneq[L::Q];
    equilibria<LAT>(rho, u, u2, fneq);
#pragma unroll
    for (int q = 0; q < L::Q; ++q) fneq[q] = f[q] - fneq[q];
    const double guess = p.alpha_field[idx];
    const double alpha = entropic_alpha<LAT>(p, f, fneq, guess, cnt, s_log);
    const double tauEff = 1.0 / (alpha * p.beta);
    const double inv = 1.0 / tauEff;
    double fsh[FS == FS_EDM ? L::Q : 1];
    shifted_equilibria<LAT, FS>(rho, u, F, fsh);
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      const double eqq = f[q] - fneq[q];
      double r = f[q] - inv * fneq[q];
      if (FS == FS_GUO || FS == FS_EDM)
        r = r + source<LAT, FS>(p, q, rho, u, F, cdot<LAT>(q, u) * L::ics, eqq, fsh);
      pop(next, p.V, q)[(uint32_t)idx] = r;
    }
    p.alpha_field[idx] = alpha;
    if (!(rho > 0.0) || !isfinite(rho)) atomicOr(p.err_word, ERR_NONFINITE);
    mass = rho;
    amin = alpha;
    amax = alpha;
    store_node_fields<LAT>(p, idx, rho, u, F, FS != FS_NONE, alpha, energy, mach);
  }
  add_counters(p.counters, cnt);
  if (p.diag) block_reduce_diag(mass, energy, mach, amin, amax, p.diag_partials);
}

// f = f_eq(rho, u) (Initialize.h:107-116), FP64 storage.
template <int LAT>
__global__ void init_f64_kernel(const double* __restrict__ rho, const double* __restrict__ u,
                                double* __restrict__ f, long long V) {
  using L = Lattice<LAT>;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= V) return;
  double uu[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int d = 0; d < L::D; ++d) uu[d] = u[(long long)d * V + idx];
  double feq[L::Q];
  equilibria<LAT>(rho[idx], uu, norm2<LAT>(uu), feq);
#pragma unroll
  for (int q = 0; q < L::Q; ++q) f[(long long)q * V + idx] = feq[q];
}

// Sample logger (FP64 storage): (f_neq/rho [Q], alpha) at the given nodes,
// from the pre-collision populations and the alpha the step just wrote.
template <int LAT>
__global__ void samples_f64_kernel(const double* __restrict__ prev, StepParams p,
                                   const long long* __restrict__ nodes, long long n,
                                   double* __restrict__ feat, double* __restrict__ alpha,
                                   int* __restrict__ solved) {
  using L = Lattice<LAT>;
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const long long idx = nodes[s];
  uint32_t x, y, z;
  node_coords(p, idx, x, y, z);
  const auto o = pull_offsets_r<L::R>(p, x, y, z);
  double f[L::Q], rho, u[3], fneq[L::Q];
  pull<LAT>(prev, p.V, o, f);
  moments<LAT>(f, rho, u);
  equilibria<LAT>(rho, u, norm2<LAT>(u), fneq);
  bool small = true;
  double alphaMax = 2.5;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    fneq[q] = f[q] - fneq[q];
    feat[s * L::Q + q] = fneq[q] / rho;
    if (fabs(fneq[q]) / f[q] > p.deviation_threshold) small = false;
    if (fneq[q] > 0) alphaMax = fmin(alphaMax, fabs(f[q]) / fneq[q]);
  }
  alpha[s] = p.alpha_field[idx];
  solved[s] = (!small && alphaMax >= 2.0) ? 1 : 0;
}

// Residual-mode alpha solve of single nodes given as FP64 pulled populations
// and non-equilibrium parts [n][Q] (tests): entropic_alpha of the FP64 kernel
// with the caller's guess. flags: 1 alpha_max < 2 (0.95 alpha_max), 2 the
// bracketed solver ran, 4 alpha = 2 fallback.
template <int LAT>
__global__ void __launch_bounds__(128) alpha_solve_test_kernel(
    const double* __restrict__ f, const double* __restrict__ fneq,
    const double* __restrict__ guess, long long n, StepParams p, double* __restrict__ alpha,
    int* __restrict__ flags) {
  using L = Lattice<LAT>;
  __shared__ LogEntry s_log[LOG_TABLE];
  stage_log_table(s_log, reinterpret_cast<const LogEntry*>(p.log_table));
  __syncthreads();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double fi[L::Q], ni[L::Q];
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    fi[q] = f[i * L::Q + q];
    ni[q] = fneq[i * L::Q + q];
  }
  unsigned c[CNT_COUNT] = {};
  alpha[i] = entropic_alpha<LAT>(p, fi, ni, guess[i], c, s_log);
  flags[i] = (c[CNT_LIMITED] ? 1 : 0) | (c[CNT_BISECT] ? 2 : 0) | (c[CNT_FALLBACK] ? 4 : 0);
}

// ---- host-side launchers --------------------------------------------------
template <int LAT, int FS>
static cudaError_t launch_bgk(const double* prev, double* next, const StepParams& p,
                              cudaStream_t s) {
  const int bs = 256;
  const unsigned grid = (unsigned)((p.V + bs - 1) / bs);
  bgk_f64_kernel<LAT, FS><<<grid, bs, 0, s>>>(prev, next, p);
  return cudaGetLastError();
}

template <int LAT, int FS>
static cudaError_t launch_elbm(const double* prev, double* next, const StepParams& p,
                               cudaStream_t s) {
  const int bs = 128;
  const unsigned grid = (unsigned)((p.V + bs - 1) / bs);
  elbm_f64_kernel<LAT, FS><<<grid, bs, 0, s>>>(prev, next, p);
  return cudaGetLastError();
}

template <int LAT>
static cudaError_t dispatch_fs(int collision, int fs, const double* prev, double* next,
                               const StepParams& p, cudaStream_t s) {
  if (collision == 0) {
    switch (fs) {
      case FS_NONE: return launch_bgk<LAT, FS_NONE>(prev, next, p, s);
      case FS_GUO: return launch_bgk<LAT, FS_GUO>(prev, next, p, s);
      case FS_SHANCHEN: return launch_bgk<LAT, FS_SHANCHEN>(prev, next, p, s);
      case FS_EDM: return launch_bgk<LAT, FS_EDM>(prev, next, p, s);
    }
  } else {
    switch (fs) {
      case FS_NONE: return launch_elbm<LAT, FS_NONE>(prev, next, p, s);
      case FS_GUO: return launch_elbm<LAT, FS_GUO>(prev, next, p, s);
      case FS_SHANCHEN: return launch_elbm<LAT, FS_SHANCHEN>(prev, next, p, s);
      case FS_EDM: return launch_elbm<LAT, FS_EDM>(prev, next, p, s);
    }
  }
  return cudaErrorInvalidValue;
}

// This file is compiled once per lattice (MLBM_LAT = 0..5) so the six sets
// of kernels build in parallel; misc.cu dispatches on the lattice.
#ifndef MLBM_LAT
#error "compile step_f64.cu with -DMLBM_LAT=<0..5>"
#endif
#define MLBM_CAT2(a, b) a##b
#define MLBM_CAT(a, b) MLBM_CAT2(a, b)

cudaError_t MLBM_CAT(step_f64_L, MLBM_LAT)(int collision, int forcing, const double* prev,
                                             double* next, const StepParams& p, cudaStream_t s) {
  return dispatch_fs<MLBM_LAT>(collision, forcing, prev, next, p, s);
}

cudaError_t MLBM_CAT(init_f64_L, MLBM_LAT)(const double* rho, const double* u, double* f,
                                             long long V, cudaStream_t s) {
  const unsigned grid = (unsigned)((V + 255) / 256);
  init_f64_kernel<MLBM_LAT><<<grid, 256, 0, s>>>(rho, u, f, V);
  return cudaGetLastError();
}

cudaError_t MLBM_CAT(alpha_solve_test_L, MLBM_LAT)(const double* f, const double* fneq,
                                                    const double* guess, long long n,
                                                    const StepParams& p, double* alpha,
                                                    int* flags, cudaStream_t s) {
  const unsigned grid = (unsigned)((n + 127) / 128);
  alpha_solve_test_kernel<MLBM_LAT><<<grid, 128, 0, s>>>(f, fneq, guess, n, p, alpha, flags);
  return cudaGetLastError();
}

cudaError_t MLBM_CAT(log_samples_f64_L, MLBM_LAT)(const double* prev, const StepParams& p,
                                                    const long long* nodes, long long n,
                                                    double* features, double* alpha, int* solved,
                                                    cudaStream_t s) {
  const unsigned grid = (unsigned)((n + 127) / 128);
  samples_f64_kernel<MLBM_LAT><<<grid, 128, 0, s>>>(prev, p, nodes, n, features, alpha, solved);
  return cudaGetLastError();
}

}  // namespace mlbm
