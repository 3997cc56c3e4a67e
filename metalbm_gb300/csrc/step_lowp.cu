// FP32 / FP16-shifted storage kernels of the fused collide-and-stream pull step.
//
// Storage (MLBM_STORAGE_F32): f_q as float. (MLBM_STORAGE_F16_SHIFTED): the
// deviation d_q = f_q - w_q scaled by 2^k_q, k_q = round(log2(1024/w_q)), as
// binary16. Either way the collision works in FP32 on the deviations
// d_q = f_q - w_q, whose moments are rho - 1 and rho u (sum_q w_q = 1,
// sum_q w_q c_q = 0), so the small hydrodynamic signal is not rounded against
// the O(w) populations.
//
// Entropic collision: the populations are widened to FP64 and the alpha solve
// (the entropy function F(alpha), its residual test, Newton and the bracketed
// fallback) runs in FP64 as in step_f64.cu; the post-collision update and the
// storage stay in FP32.
//
// Same node order and periodic pull as step_f64.cu.

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"
#include "kernels.h"
#include "mlp_device.cuh"
#include "entropy.cuh"
#include "fastlog.cuh"
#include "solver.cuh"

namespace mlbm {

enum : int { ST_F32 = 1, ST_F16 = 2 };

template <int LAT>
__host__ __device__ constexpr int shift_exponent(int q) {
  // round(log2(1024 / w_q)) for the weight classes of the three lattices
  return Lattice<LAT>::w(q) > 0.4 ? 11                      // 4/9
         : Lattice<LAT>::w(q) > 0.3 ? 12                    // 1/3, 8/27
         : Lattice<LAT>::w(q) > 0.1 ? 13                    // 1/9
         : Lattice<LAT>::w(q) > 0.06 ? 14                   // 2/27, 1/18
         : Lattice<LAT>::w(q) > 0.025 ? 15                  // 1/36
         : Lattice<LAT>::w(q) > 0.01 ? 16                   // 1/54
                                     : 18;                  // 1/216
}

template <int ST>
struct Storage;

template <>
struct Storage<ST_F32> {
  using T = float;
  template <int LAT>
  __device__ __forceinline__ static float load(const float* p, int q) {
    return __ldg(p) - (float)Lattice<LAT>::w(q);
  }
  template <int LAT>
  __device__ __forceinline__ static void store(float* p, int q, float d) {
    *p = (float)Lattice<LAT>::w(q) + d;
  }
  template <int LAT>
  __host__ __device__ static double decode(float v, int q) { return (double)v; }
  template <int LAT>
  __device__ static float encode(double f, int q) { return (float)f; }
};

template <>
struct Storage<ST_F16> {
  using T = __half;
  template <int LAT>
  __device__ __forceinline__ static float load(const __half* p, int q) {
    return __half2float(__ldg(p)) * (1.0f / (float)(1 << shift_exponent<LAT>(q)));
  }
  template <int LAT>
  __device__ __forceinline__ static void store(__half* p, int q, float d) {
    *p = __float2half_rn(d * (float)(1 << shift_exponent<LAT>(q)));
  }
  template <int LAT>
  __device__ static double decode(__half v, int q) {
    return Lattice<LAT>::w(q) + (double)__half2float(v) / (double)(1 << shift_exponent<LAT>(q));
  }
  template <int LAT>
  __device__ static __half encode(double f, int q) {
    return __float2half_rn((float)((f - Lattice<LAT>::w(q)) * (double)(1 << shift_exponent<LAT>(q))));
  }
};

// Exact FP64 value of a stored population.
template <int LAT, int ST>
__device__ __forceinline__ double load_f64(const typename Storage<ST>::T* p, int q) {
  if constexpr (ST == ST_F32) {
    return (double)__ldg(p);
  } else {
    return Lattice<LAT>::w(q) +
           (double)__half2float(__ldg(p)) * (1.0 / (double)(1 << shift_exponent<LAT>(q)));
  }
}

// f_eq in FP64 (TruncationMa3 polynomial, Equilibrium.h:17-33), pairwise.
template <int LAT>
__device__ __forceinline__ void feq_pairs_f64(double rho, const double u[3], double feq[]) {
  using L = Lattice<LAT>;
  const double u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double common = u2 * (1.125 * u2 - 1.5);
  feq[0] = rho * L::w(0) * (1.0 + common);
#pragma unroll
  for (int q = 1; q < L::Q; ++q) {
    if (is_pair_leader<LAT>(q)) {
      const int qb = opposite<LAT>(q);
      double cu = 0.0;
#pragma unroll
      for (int k = 0; k < L::D; ++k) {
        if (L::c(q, k) > 0) cu += u[k];
        if (L::c(q, k) < 0) cu -= u[k];
      }
      const double c2 = cu * cu;
      const double E = fma(c2, fma(3.375, c2, fma(-6.75, u2, 4.5)), common);
      const double O = cu * fma(4.5, c2, fma(-4.5, u2, 3.0));
      feq[q] = rho * L::w(q) * (1.0 + (E + O));
      feq[qb] = rho * L::w(qb) * (1.0 + (E - O));
    }
  }
}

template <int LAT, int ST>
__device__ __forceinline__ void store_f64(typename Storage<ST>::T* p, int q, double f) {
  if constexpr (ST == ST_F32) {
    *p = (float)f;
  } else {
    *p = __float2half_rn((float)((f - Lattice<LAT>::w(q)) * (double)(1 << shift_exponent<LAT>(q))));
  }
}

template <int LAT>
__device__ __forceinline__ float cdotf(int q, const float v[3]) {
  using L = Lattice<LAT>;
  float r = 0.0f;
#pragma unroll
  for (int d = 0; d < L::D; ++d) {
    const int c = L::c(q, d);
    if (c > 0) r += v[d];
    if (c < 0) r -= v[d];
  }
  return r;
}

// TruncationMa3 polynomial P = fEq/(rho w) - 1 (Equilibrium.h:17-33) split
// into the parts even and odd in c.u: P(+-cu) = E(cu) +- O(cu).
struct PolyNode {
  float u2, common;
};
__device__ __forceinline__ PolyNode poly_node(float u2) {
  PolyNode n;
  n.u2 = u2;
  n.common = u2 * (1.125f * u2 - 1.5f);
  return n;
}
__device__ __forceinline__ void poly_pair(const PolyNode& n, float cu, float& E, float& O) {
  const float c2 = cu * cu;
  E = fmaf(c2, fmaf(3.375f, c2, fmaf(-6.75f, n.u2, 4.5f)), n.common);
  O = cu * fmaf(4.5f, c2, fmaf(-4.5f, n.u2, 3.0f));
}

// Equilibrium deviations deq_q = f_eq_q - w_q = w_q (rho' + rho P_q),
// rho' = rho - 1.
template <int LAT>
__device__ __forceinline__ void eq_dev(float rhop, float rho, const float u[3], float u2,
                                       float deq[Lattice<LAT>::Q]) {
  using L = Lattice<LAT>;
  const PolyNode n = poly_node(u2);
  deq[0] = (float)L::w(0) * fmaf(rho, n.common, rhop);
#pragma unroll
  for (int q = 1; q < L::Q; ++q) {
    if (is_pair_leader<LAT>(q)) {
      const int qb = opposite<LAT>(q);
      float E, O;
      poly_pair(n, cdotf<LAT>(q, u), E, O);
      deq[q] = (float)L::w(q) * fmaf(rho, E + O, rhop);
      deq[qb] = (float)L::w(qb) * fmaf(rho, E - O, rhop);
    }
  }
}

template <int LAT, int ST>
__device__ __forceinline__ void pull_dev(const typename Storage<ST>::T* __restrict__ prev,
                                         long long V, const PullOffsets& o,
                                         float d[Lattice<LAT>::Q]) {
  using L = Lattice<LAT>;
#pragma unroll
  for (int q = 0; q < L::Q; ++q)
    d[q] = Storage<ST>::template load<LAT>(
        prev + (long long)q * V + o.at(L::c(q, 0), L::c(q, 1), L::c(q, 2)), q);
}

template <int LAT>
__device__ __forceinline__ void moments_dev(const float d[Lattice<LAT>::Q], float& rhop,
                                            float& rho, float u[3]) {
  using L = Lattice<LAT>;
  rhop = 0.0f;
  float j[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    rhop += d[q];
#pragma unroll
    for (int k = 0; k < L::D; ++k) {
      if (L::c(q, k) > 0) j[k] += d[q];
      if (L::c(q, k) < 0) j[k] -= d[q];
    }
  }
  rho = 1.0f + rhop;
  const float inv = 1.0f / rho;
#pragma unroll
  for (int k = 0; k < 3; ++k) u[k] = j[k] * inv;
}

template <int LAT>
__device__ __forceinline__ void node_force_f(const StepParams& p, uint32_t x, uint32_t y,
                                             uint32_t z, float Ff[3], double F[3]) {
  node_force<Lattice<LAT>::D>(p, x, y, z, F);
#pragma unroll
  for (int k = 0; k < 3; ++k) Ff[k] = (float)F[k];
}

template <int LAT>
__device__ __forceinline__ void lowp_store_fields(const StepParams& p, long long idx, float rho,
                                                  const float u[3], const double F[3], bool shifted,
                                                  double alpha, double& energy, double& mach) {
  using L = Lattice<LAT>;
  double uh[3] = {0.0, 0.0, 0.0};
  const double r = (double)rho;
#pragma unroll
  for (int k = 0; k < L::D; ++k) uh[k] = shifted ? (double)u[k] + F[k] * (0.5 / r) : (double)u[k];
  if (p.store) {
    p.rho_out[idx] = r;
#pragma unroll
    for (int k = 0; k < L::D; ++k) {
      p.u_out[(long long)k * p.V + idx] = uh[k];
      p.force_out[(long long)k * p.V + idx] = F[k];
    }
    if (p.alpha_field_f32) p.alpha_field_f32[idx] = (float)alpha;
  }
  if (p.diag) {
    double e = 0.0, s = 0.0;
#pragma unroll
    for (int k = 0; k < L::D; ++k) {
      e += 0.5 * r * uh[k] * uh[k];
      s += uh[k] * uh[k];
    }
    energy = e;
    mach = sqrt(3.0 * s);
  }
}

// ---- BGK ------------------------------------------------------------------
// Per-node body force in float from the float profile tables.
template <int D>
__device__ __forceinline__ void node_force_float(const StepParams& p, uint32_t x, uint32_t y,
                                                 uint32_t z, float F[3]) {
  F[0] = 0.0f; F[1] = 0.0f; F[2] = 0.0f;
  switch (p.force_type) {
    case FORCE_CONSTANT:
      F[0] = p.amp_f[0]; F[1] = p.amp_f[1]; F[2] = D == 3 ? p.amp_f[2] : 0.0f;
      break;
    case FORCE_SINUSOIDAL:
      F[0] = __ldg(p.force_table_f[0] + x);
      F[1] = __ldg(p.force_table_f[1] + y);
      if (D == 3) F[2] = __ldg(p.force_table_f[2] + z);
      break;
    case FORCE_KOLMOGOROV: {
      const uint32_t c = p.kol_axis == 0 ? x : (p.kol_axis == 1 ? y : z);
      const float v = __ldg(p.force_table_f[0] + c);
      F[0] = p.kol_comp == 0 ? v : 0.0f;
      F[1] = p.kol_comp == 1 ? v : 0.0f;
      F[2] = p.kol_comp == 2 ? v : 0.0f;
      break;
    }
    default:
      break;
  }
}

// BGK in deviation variables (d = f - w):
//   d' = d + 2 beta (d_eq - d) + S,   d_eq_q = w_q (rho' + rho P_q)
// with the pair algebra P(+-cu) = E +- O of the TruncationMa3 polynomial and,
// for Guo (ForcingScheme.h:100-117), S_q = kt w_q [(c_q - u).F + 3 (c_q.u)(c_q.F)]
// = kt w_q (3 cu cF - u.F +- cF) for the pair; EDM: S_q = w_q rho (P_q(v) - P_q(u)),
// v = u + F/rho (ForcingScheme.h:183-197).
template <int LAT, int FS, int ST>
__global__ void __launch_bounds__(256) bgk_lowp_kernel(const typename Storage<ST>::T* __restrict__ prev,
                                                       typename Storage<ST>::T* __restrict__ next,
                                                       StepParams p) {
  using L = Lattice<LAT>;
  using T = typename Storage<ST>::T;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = idx < p.V;
  double mass = 0.0, energy = 0.0, mach = 0.0;
  if (active) {
    uint32_t x, y, z;
    node_coords(p, idx, x, y, z);
    const PullOffsets o = pull_offsets(p, x, y, z);
    float d[L::Q];
    pull_dev<LAT, ST>(prev, p.V, o, d);
    float rhop, rho, u[3];
    moments_dev<LAT>(d, rhop, rho, u);
    float F[3] = {0.0f, 0.0f, 0.0f};
    if (FS != FS_NONE) node_force_float<L::D>(p, x, y, z, F);
    const float u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const PolyNode n = poly_node(u2);
    const float b = p.bgk_b_f;
    float uF = 0.0f, v[3] = {0.0f, 0.0f, 0.0f};
    PolyNode nv = n;
    if (FS == FS_GUO) uF = u[0] * F[0] + u[1] * F[1] + u[2] * F[2];
    if (FS == FS_EDM) {
      const float ir = 1.0f / rho;
#pragma unroll
      for (int k = 0; k < 3; ++k) v[k] = fmaf(F[k], ir, u[k]);
      nv = poly_node(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
    T* out = next + idx;
    {  // rest population
      const float w = (float)L::w(0);
      const float deq = w * fmaf(rho, n.common, rhop);
      float r = fmaf(b, deq - d[0], d[0]);
      if (FS == FS_GUO) r = fmaf(p.guo_kt_f * w, -uF, r);
      if (FS == FS_EDM) r = fmaf(w * rho, nv.common - n.common, r);
      Storage<ST>::template store<LAT>(out, 0, r);
    }
#pragma unroll
    for (int q = 1; q < L::Q; ++q) {
      if (is_pair_leader<LAT>(q)) {
        const int qb = opposite<LAT>(q);
        const float w = (float)L::w(q);
        const float cu = cdotf<LAT>(q, u);
        float E, O;
        poly_pair(n, cu, E, O);
        const float dq = w * fmaf(rho, E + O, rhop), dqb = w * fmaf(rho, E - O, rhop);
        float rq = fmaf(b, dq - d[q], d[q]);
        float rqb = fmaf(b, dqb - d[qb], d[qb]);
        if (FS == FS_GUO) {
          const float cF = cdotf<LAT>(q, F);
          const float Es = fmaf(3.0f * cu, cF, -uF);
          const float kw = p.guo_kt_f * w;
          rq = fmaf(kw, Es + cF, rq);
          rqb = fmaf(kw, Es - cF, rqb);
        }
        if (FS == FS_EDM) {
          float Ev, Ov;
          poly_pair(nv, cdotf<LAT>(q, v), Ev, Ov);
          const float wr = w * rho;
          rq = fmaf(wr, (Ev + Ov) - (E + O), rq);
          rqb = fmaf(wr, (Ev - Ov) - (E - O), rqb);
        }
        Storage<ST>::template store<LAT>(out + (long long)q * p.V, q, rq);
        Storage<ST>::template store<LAT>(out + (long long)qb * p.V, qb, rqb);
      }
    }
    if (!(rho > 0.0f) || !isfinite(rho)) atomicOr(p.err_word, ERR_NONFINITE);
    if (p.store || p.diag) {
      double Fd[3];
      node_force<L::D>(p, x, y, z, Fd);
      if (p.diag) mass = (double)rho;
      lowp_store_fields<LAT>(p, idx, rho, u, Fd, FS != FS_NONE, 2.0, energy, mach);
    }
  }
  if (p.diag) block_reduce_diag(mass, energy, mach, 2.0, 2.0, p.diag_partials);
}

// ---- Entropic SRT with an FP64 alpha solve --------------------------------
// The alpha solve needs f_neq with the exact mass and momentum of the
// stored state, so the entropic kernel widens the stored populations to FP64
// and forms rho, u, f_eq and f_neq there; FP32 deviations would leave a
// residual mass of the order of the storage rounding in f_neq, and F(alpha)
// would then have no root in [1, alpha_max] on well-resolved flows.
template <int LAT, int FS, int ST, bool LEARNED>
__global__ void __launch_bounds__(128) elbm_lowp_kernel(const typename Storage<ST>::T* __restrict__ prev,
                                                        typename Storage<ST>::T* __restrict__ next,
                                                        StepParams p) {
  using L = Lattice<LAT>;
  __shared__ LogEntry s_log[LOG_TABLE];
  stage_log_table(s_log, reinterpret_cast<const LogEntry*>(p.log_table));
  __syncthreads();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = idx < p.V;
  double mass = 0.0, energy = 0.0, mach = 0.0, amin = 1e300, amax = -1e300;
  unsigned cnt[CNT_COUNT] = {0, 0, 0, 0, 0, 0, 0, 0};
  double f[L::Q];
  uint32_t x = 0, y = 0, z = 0;
  float learned = 2.0f;
  {
    float dv[L::Q];  // FP32 deviations f - w (model features)
    if (active) {
      node_coords(p, idx, x, y, z);
      const PullOffsets o = pull_offsets(p, x, y, z);
#pragma unroll
      for (int q = 0; q < L::Q; ++q) {
        const auto* src = prev + (long long)q * p.V + o.at(L::c(q, 0), L::c(q, 1), L::c(q, 2));
        if constexpr (ST == ST_F32) {
          const float v = __ldg(src);
          f[q] = widen_exact(v);  // exact, without a conversion instruction
          dv[q] = v - (float)L::w(q);
        } else {
          const float dev = __half2float(__ldg(src)) * (1.0f / (float)(1 << shift_exponent<LAT>(q)));
          f[q] = L::w(q) + widen_exact(dev);
          dv[q] = dev;
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < L::Q; ++q) { f[q] = L::w(q); dv[q] = 0.0f; }
    }
    // Learned guess: every thread of the block takes part (tile inference),
    // on features f_neq / rho from the FP32 deviations (the BF16 inference
    // does not need FP64 inputs).
    if (LEARNED) {
      float rhop, rf, uf[3], deq[L::Q];
      moments_dev<LAT>(dv, rhop, rf, uf);
      eq_dev<LAT>(rhop, rf, uf, uf[0] * uf[0] + uf[1] * uf[1] + uf[2] * uf[2], deq);
      const float irf = 1.0f / rf;
      float xin[L::Q];
#pragma unroll
      for (int q = 0; q < L::Q; ++q) xin[q] = (dv[q] - deq[q]) * irf;
      learned = mlp_guess_block<L::Q>(reinterpret_cast<const MlpDev*>(p.mlp), xin);
    }
  }
  if (active) {
    double rho = f[0], j[3] = {0.0, 0.0, 0.0}, u[3], F[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 1; q < L::Q; ++q) {
      rho += f[q];
#pragma unroll
      for (int k = 0; k < L::D; ++k) {
        if (L::c(q, k) > 0) j[k] += f[q];
        if (L::c(q, k) < 0) j[k] -= f[q];
      }
    }
    const double ir = 1.0 / rho;
#pragma unroll
    for (int k = 0; k < 3; ++k) u[k] = j[k] * ir;
    if (FS != FS_NONE) node_force<L::D>(p, x, y, z, F);
    // r_q = f_neq_q / f_q; alpha_max = min(2.5, 1 / max_q r_q) over r_q > 0
    // (Collision.h:305-326); the deviation test |f_neq|/f <= threshold
    // (Collision.h:284-303) on |r_q|.
    double r[L::Q], rpos = 0.0, rabs = 0.0;
    feq_pairs_f64<LAT>(rho, u, r);
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      r[q] = (f[q] - r[q]) / f[q];
      rpos = fmax(rpos, r[q]);
      rabs = fmax(rabs, fabs(r[q]));
    }
    const bool small = !(rabs > p.deviation_threshold);
    const double alphaMax = rpos > 0.4 ? 1.0 / rpos : 2.5;
    double alpha;
    if (small) { ++cnt[CNT_SHORTCUT]; alpha = 2.0; }
    else if (alphaMax < 2.0) { ++cnt[CNT_LIMITED]; alpha = 0.95 * alphaMax; }
    else {
      ++cnt[CNT_SOLVED];
      const double prevA = widen_exact(p.alpha_field_f32[idx]);
      const double plain = p.guess_mode == GUESS_TWO ? 2.0 : prevA;
      const double guess = LEARNED ? widen_exact(learned) : plain;
      double B1 = 0.0, sfn = 0.0;
#pragma unroll
      for (int q = 0; q < L::Q; ++q) {
        const double fnq = r[q] * f[q];
        B1 = fma(fnq, fast_log(f[q] * (1.0 / L::w(q)), s_log), B1);
        sfn += fnq;
      }
      const HLog1p<LAT> ev{f, r, B1, sfn + B1, rabs, s_log};
      alpha = residual_alpha_solve(ev, guess, plain, alphaMax, p.newton_tol, p.newton_maxit, cnt);
    }
    const double ab = alpha * p.beta;
    double fsh[FS == FS_EDM ? L::Q : 1];
    if (FS == FS_EDM) {
      double v[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) v[k] = u[k] + F[k] / rho;
      feq_pairs_f64<LAT>(rho, v, fsh);
    }
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      // f - alpha beta f_neq + S  (Collision.h:243-258), f_neq = r f
      const double fnq = r[q] * f[q];
      double rr = fma(-ab, fnq, f[q]);
      if (FS == FS_GUO) {
        double cu = 0.0;
#pragma unroll
        for (int k = 0; k < L::D; ++k) {
          if (L::c(q, k) > 0) cu += u[k];
          if (L::c(q, k) < 0) cu -= u[k];
        }
        double R = 0.0;
#pragma unroll
        for (int k = 0; k < L::D; ++k) R = fma((double)L::c(q, k) - u[k] + L::c(q, k) * 3.0 * cu, F[k], R);
        rr += p.guo_k[q] * R;
      }
      if (FS == FS_EDM) rr += fsh[q] - (f[q] - fnq);
      auto* dst = next + (long long)q * p.V + idx;
      if constexpr (ST == ST_F32) {
        *dst = narrow_rn(rr);
      } else {
        *dst = __float2half_rn(narrow_rn((rr - L::w(q)) * (double)(1 << shift_exponent<LAT>(q))));
      }
    }
    p.alpha_field_f32[idx] = narrow_rn(alpha);
    if (!(rho > 0.0) || !isfinite(rho)) atomicOr(p.err_word, ERR_NONFINITE);
    if (p.store || p.diag) {
      mass = rho;
      amin = alpha;
      amax = alpha;
      const float uf[3] = {(float)u[0], (float)u[1], (float)u[2]};
      lowp_store_fields<LAT>(p, idx, (float)rho, uf, F, FS != FS_NONE, alpha, energy, mach);
    }
  }
  add_counters(p.counters, cnt);
  if (p.diag) block_reduce_diag(mass, energy, mach, amin, amax, p.diag_partials);
}

// ---- init and conversions ---------------------------------------------------
// f_eq(rho, u) is formed in FP64 with the reference polynomial, then encoded.
template <int LAT>
__device__ double feq_f64(double rho, const double u[3], int q) {
  using L = Lattice<LAT>;
  double cu = 0.0, u2 = 0.0;
#pragma unroll
  for (int k = 0; k < L::D; ++k) {
    cu += L::c(q, k) * u[k];
    u2 += u[k] * u[k];
  }
  const double P = 3.0 * cu - 1.5 * u2 + 4.5 * cu * cu - 4.5 * cu * u2 + 4.5 * cu * cu * cu +
                   1.125 * u2 * u2 - 6.75 * cu * cu * u2 + 3.375 * cu * cu * cu * cu;
  return rho * L::w(q) * (1.0 + P);
}

template <int LAT, int ST>
__global__ void init_lowp_kernel(const double* __restrict__ rho, const double* __restrict__ u,
                                 typename Storage<ST>::T* __restrict__ f, long long V) {
  using L = Lattice<LAT>;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= V) return;
  double uu[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < L::D; ++k) uu[k] = u[(long long)k * V + idx];
#pragma unroll
  for (int q = 0; q < L::Q; ++q)
    f[(long long)q * V + idx] = Storage<ST>::template encode<LAT>(feq_f64<LAT>(rho[idx], uu, q), q);
}

template <int LAT, int ST>
__global__ void decode_kernel(const typename Storage<ST>::T* __restrict__ f, int q,
                              double* __restrict__ out, long long V) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= V) return;
  // q is uniform: dispatch the constexpr weight through a switch-free loop
#pragma unroll
  for (int k = 0; k < Lattice<LAT>::Q; ++k)
    if (k == q) out[idx] = Storage<ST>::template decode<LAT>(f[(long long)q * V + idx], k);
}

template <int LAT, int ST>
__global__ void encode_kernel(const double* __restrict__ in, int q, typename Storage<ST>::T* __restrict__ f,
                              long long V) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= V) return;
#pragma unroll
  for (int k = 0; k < Lattice<LAT>::Q; ++k)
    if (k == q) f[(long long)q * V + idx] = Storage<ST>::template encode<LAT>(in[idx], k);
}

// ---- sample logger (f_neq/rho, alpha) --------------------------------------
template <int LAT, int ST>
__global__ void samples_lowp_kernel(const typename Storage<ST>::T* __restrict__ prev, StepParams p,
                                    const long long* __restrict__ nodes, long long n,
                                    double* __restrict__ feat, double* __restrict__ alpha,
                                    int* __restrict__ solved) {
  using L = Lattice<LAT>;
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const long long idx = nodes[s];
  uint32_t x, y, z;
  node_coords(p, idx, x, y, z);
  const PullOffsets o = pull_offsets(p, x, y, z);
  double f[L::Q], fn[L::Q], rho = 0.0, j[3] = {0.0, 0.0, 0.0}, u[3];
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    f[q] = load_f64<LAT, ST>(prev + (long long)q * p.V + o.at(L::c(q, 0), L::c(q, 1), L::c(q, 2)), q);
    rho += f[q];
#pragma unroll
    for (int k = 0; k < L::D; ++k) {
      if (L::c(q, k) > 0) j[k] += f[q];
      if (L::c(q, k) < 0) j[k] -= f[q];
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) u[k] = j[k] / rho;
  feq_pairs_f64<LAT>(rho, u, fn);
  bool small = true;
  double alphaMax = 2.5;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    fn[q] = f[q] - fn[q];
    feat[s * L::Q + q] = fn[q] / rho;
    if (fabs(fn[q]) > p.deviation_threshold * f[q]) small = false;
    if (fn[q] > 0.0) alphaMax = fmin(alphaMax, f[q] / fn[q]);
  }
  alpha[s] = (double)p.alpha_field_f32[idx];
  solved[s] = (!small && alphaMax >= 2.0) ? 1 : 0;
}

// ---- host launchers -----------------------------------------------------------
template <int LAT, int FS, int ST>
static cudaError_t launch_lowp(int collision, const void* prev, void* next, const StepParams& p,
                               cudaStream_t s) {
  using T = typename Storage<ST>::T;
  if (collision == 0) {
    const int bs = 256;
    const unsigned grid = (unsigned)((p.V + bs - 1) / bs);
    bgk_lowp_kernel<LAT, FS, ST><<<grid, bs, 0, s>>>((const T*)prev, (T*)next, p);
  } else {
    const int bs = 128;
    const unsigned grid = (unsigned)((p.V + bs - 1) / bs);
    if (p.guess_mode == GUESS_LEARNED)
      elbm_lowp_kernel<LAT, FS, ST, true><<<grid, bs, 0, s>>>((const T*)prev, (T*)next, p);
    else
      elbm_lowp_kernel<LAT, FS, ST, false><<<grid, bs, 0, s>>>((const T*)prev, (T*)next, p);
  }
  return cudaGetLastError();
}

// This file is compiled once per (lattice, storage) pair (MLBM_LAT = 0..2,
// MLBM_ST = 1 F32 or 2 F16-shifted); misc.cu dispatches.
#if !defined(MLBM_LAT) || !defined(MLBM_ST)
#error "compile step_lowp.cu with -DMLBM_LAT=<0|1|2> -DMLBM_ST=<1|2>"
#endif
#define MLBM_CAT2(a, b, c, d) a##b##c##d
#define MLBM_CAT(a, b, c, d) MLBM_CAT2(a, b, c, d)
#define MLBM_FN(name) MLBM_CAT(name, MLBM_LAT, _S, MLBM_ST)
using StT = typename Storage<MLBM_ST>::T;

cudaError_t MLBM_FN(step_lowp_L)(int collision, int fs, const void* prev, void* next,
                                 const StepParams& p, cudaStream_t s) {
  switch (fs) {
    case FS_NONE: return launch_lowp<MLBM_LAT, FS_NONE, MLBM_ST>(collision, prev, next, p, s);
    case FS_GUO: return launch_lowp<MLBM_LAT, FS_GUO, MLBM_ST>(collision, prev, next, p, s);
    case FS_SHANCHEN: return launch_lowp<MLBM_LAT, FS_SHANCHEN, MLBM_ST>(collision, prev, next, p, s);
    case FS_EDM: return launch_lowp<MLBM_LAT, FS_EDM, MLBM_ST>(collision, prev, next, p, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t MLBM_FN(init_lowp_L)(const double* rho, const double* u, void* f, long long V,
                                 cudaStream_t s) {
  init_lowp_kernel<MLBM_LAT, MLBM_ST><<<(unsigned)((V + 255) / 256), 256, 0, s>>>(rho, u, (StT*)f, V);
  return cudaGetLastError();
}

cudaError_t MLBM_FN(lowp_to_f64_L)(const void* f, int q, double* out, long long V, cudaStream_t s) {
  decode_kernel<MLBM_LAT, MLBM_ST><<<(unsigned)((V + 255) / 256), 256, 0, s>>>((const StT*)f, q, out, V);
  return cudaGetLastError();
}

cudaError_t MLBM_FN(f64_to_lowp_L)(const double* in, int q, void* f, long long V, cudaStream_t s) {
  encode_kernel<MLBM_LAT, MLBM_ST><<<(unsigned)((V + 255) / 256), 256, 0, s>>>(in, q, (StT*)f, V);
  return cudaGetLastError();
}

cudaError_t MLBM_FN(log_samples_lowp_L)(const void* prev, const StepParams& p,
                                        const long long* nodes, long long n, double* features,
                                        double* alpha, int* solved, cudaStream_t s) {
  samples_lowp_kernel<MLBM_LAT, MLBM_ST><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
      (const StT*)prev, p, nodes, n, features, alpha, solved);
  return cudaGetLastError();
}

}  // namespace mlbm
