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
#include "ref_node.cuh"
#include "solver.cuh"

namespace mlbm {

// ---- BGK (Collision.h:103-180 + Algorithm.h:97-126) ----------------------
template <int LAT, int FS>
__global__ void __launch_bounds__(256) bgk_f64_kernel(const double* __restrict__ prev,
                                                      double* __restrict__ next, StepParams p) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = idx < p.V;
  double mass = 0.0, energy = 0.0, mach = 0.0;
  if (active) {
    uint32_t x, y, z;
    node_coords(p, idx, x, y, z);
    bgk_node_reference<LAT, FS>(prev, next, p, idx, x, y, z, mass, energy, mach);
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

// This file is compiled once per (lattice, forcing scheme) pair (MLBM_LAT =
// 0..5, MLBM_FS = 0..3: None, Guo, Shan-Chen, EDM) so the units build in
// parallel. Each unit holds the step kernels of its forcing scheme; the FS_NONE
// unit also holds the lattice's dispatcher and the kernels that do not depend
// on the forcing scheme. misc.cu dispatches on the lattice.
#if !defined(MLBM_LAT) || !defined(MLBM_FS)
#error "compile step_f64.cu with -DMLBM_LAT=<0..5> -DMLBM_FS=<0..3>"
#endif
#define MLBM_CAT2(a, b) a##b
#define MLBM_CAT(a, b) MLBM_CAT2(a, b)
#define MLBM_FN_FS(fs) MLBM_CAT(MLBM_CAT(MLBM_CAT(step_f64_L, MLBM_LAT), _F), fs)

// one forcing scheme's step launches (collision 0 BGK, otherwise entropic)
cudaError_t MLBM_FN_FS(0)(int collision, const double* prev, double* next, const StepParams& p,
                          cudaStream_t s);
cudaError_t MLBM_FN_FS(1)(int collision, const double* prev, double* next, const StepParams& p,
                          cudaStream_t s);
cudaError_t MLBM_FN_FS(2)(int collision, const double* prev, double* next, const StepParams& p,
                          cudaStream_t s);
cudaError_t MLBM_FN_FS(3)(int collision, const double* prev, double* next, const StepParams& p,
                          cudaStream_t s);

cudaError_t MLBM_FN_FS(MLBM_FS)(int collision, const double* prev, double* next,
                                const StepParams& p, cudaStream_t s) {
  if (collision == 0) return launch_bgk<MLBM_LAT, MLBM_FS>(prev, next, p, s);
  return launch_elbm<MLBM_LAT, MLBM_FS>(prev, next, p, s);
}

#if MLBM_FS == 0
cudaError_t MLBM_CAT(step_f64_L, MLBM_LAT)(int collision, int forcing, const double* prev,
                                             double* next, const StepParams& p, cudaStream_t s) {
  static_assert(FS_NONE == 0 && FS_GUO == 1 && FS_SHANCHEN == 2 && FS_EDM == 3,
                "the units are numbered by the forcing scheme's value");
  switch (forcing) {
    case FS_NONE: return MLBM_FN_FS(0)(collision, prev, next, p, s);
    case FS_GUO: return MLBM_FN_FS(1)(collision, prev, next, p, s);
    case FS_SHANCHEN: return MLBM_FN_FS(2)(collision, prev, next, p, s);
    case FS_EDM: return MLBM_FN_FS(3)(collision, prev, next, p, s);
  }
  return cudaErrorInvalidValue;
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
#endif  // MLBM_FS == 0

}  // namespace mlbm
