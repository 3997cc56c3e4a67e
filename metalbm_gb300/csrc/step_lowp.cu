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
#include "dfloat.cuh"

namespace mlbm {

enum : int { ST_F32 = 1, ST_F16 = 2 };

// f_neq of the FP32-storage entropic main pass in double-float arithmetic
// (1) or in FP64 (0).
#ifndef MLBM_NEQ_DFLOAT
#define MLBM_NEQ_DFLOAT 1
#endif

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

// Scaled deviations d'_q = S_q (f_q - w_q), S_q = 1 (F32) or 2^k_q (F16):
// the value a population is stored as, before its rounding to the storage
// type. The BGK kernel works on d' with the scale folded into its
// constants, so the FP16 path spends no multiply on either side of memory.
template <>
struct Storage<ST_F32> {
  using T = float;
  template <int LAT>
  __host__ __device__ static constexpr float scale(int) { return 1.0f; }
  template <int LAT>
  __device__ __forceinline__ static float load_scaled(const float* p, int q) {
    return __ldg(p) - (float)Lattice<LAT>::w(q);
  }
  template <int LAT>
  __device__ __forceinline__ static void store_scaled(float* p, int q, float d) {
    *p = (float)Lattice<LAT>::w(q) + d;
  }
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
  __host__ __device__ static constexpr float scale(int q) {
    return (float)(1 << shift_exponent<LAT>(q));
  }
  template <int LAT>
  __device__ __forceinline__ static float load_scaled(const __half* p, int) {
    return __half2float(__ldg(p));
  }
  template <int LAT>
  __device__ __forceinline__ static void store_scaled(__half* p, int, float d) {
    *p = __float2half_rn(d);
  }
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
        pop(prev, V, q) + o.at(L::c(q, 0), L::c(q, 1), L::c(q, 2)), q);
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

// Stored fields and the diagnostics' node terms from FP64 rho and u (the
// hydrodynamic velocity u + F/(2 rho) for the shifted forcing schemes).
template <int LAT>
__device__ __forceinline__ void store_fields_f64(const StepParams& p, long long idx, double r,
                                                 const double u[3], const double F[3],
                                                 bool shifted, double alpha, double& energy,
                                                 double& mach, bool write_alpha = true) {
  using L = Lattice<LAT>;
  double uh[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < L::D; ++k) uh[k] = shifted ? u[k] + F[k] * (0.5 / r) : u[k];
  if (p.store) {
    p.rho_out[idx] = r;
#pragma unroll
    for (int k = 0; k < L::D; ++k) {
      p.u_out[(long long)k * p.V + idx] = uh[k];
      p.force_out[(long long)k * p.V + idx] = F[k];
    }
    if (p.alpha_field_f32 && write_alpha) p.alpha_field_f32[idx] = narrow_rn(alpha - 2.0);
  }
  if (p.diag) {
    // the node's kinetic energy and |u|^2 / c_s^2 (the square root is taken
    // once, in finalize_diag) in FP32 from the FP64 rho and u: a relative
    // rounding of ~1e-7, below that of the FP32 / FP16 populations themselves,
    // without GB300's narrow FP64 pipe
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < L::D; ++k) {
      const float v = narrow_rn(uh[k]);
      s = fmaf(v, v, s);
    }
    energy = widen_exact(0.5f * narrow_rn(r) * s);
    mach = widen_exact(3.0f * s);
  }
}

template <int LAT>
__device__ __forceinline__ void lowp_store_fields(const StepParams& p, long long idx, float rho,
                                                  const float u[3], const double F[3], bool shifted,
                                                  double alpha, double& energy, double& mach,
                                                  bool write_alpha = true) {
  const double ud[3] = {(double)u[0], (double)u[1], (double)u[2]};
  store_fields_f64<LAT>(p, idx, (double)rho, ud, F, shifted, alpha, energy, mach, write_alpha);
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
    case FORCE_FIELD: {  // Force<Generic>::setForce (Force.h:36-45), float copy
      const uint32_t i = (x * p.ly + y) * p.lz + z;
#pragma unroll
      for (int d = 0; d < D; ++d) F[d] = __ldg(p.force_field_f + (long long)d * p.V + i);
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
// v = u + F/rho (ForcingScheme.h:183-197). Every population is carried in its
// storage scale (d'_q = S_q d_q, Storage::scale), the factors S_q and 1/S_q
// folded into the per-population constants. `d` holds the pulled values on
// entry and the post-collision values on exit.
template <int LAT, int FS, int ST>
__device__ __forceinline__ void bgk_node(const StepParams& p, uint32_t x, uint32_t y, uint32_t z,
                                         float d[Lattice<LAT>::Q], float& rho_out,
                                         float u[3]) {
  using L = Lattice<LAT>;
  using S = Storage<ST>;
  float rhop = 0.0f, j[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    const float is = 1.0f / S::template scale<LAT>(q);
    rhop = fmaf(d[q], is, rhop);
#pragma unroll
    for (int k = 0; k < L::D; ++k) {
      if (L::c(q, k) > 0) j[k] = fmaf(d[q], is, j[k]);
      if (L::c(q, k) < 0) j[k] = fmaf(d[q], -is, j[k]);
    }
  }
  const float rho = 1.0f + rhop;
  const float irho = 1.0f / rho;
#pragma unroll
  for (int k = 0; k < 3; ++k) u[k] = j[k] * irho;
  float F[3] = {0.0f, 0.0f, 0.0f};
  if (FS != FS_NONE) node_force_float<L::D>(p, x, y, z, F);
  const float u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const PolyNode n = poly_node(u2);
  const float b = p.bgk_b_f;
  float uF = 0.0f, v[3] = {0.0f, 0.0f, 0.0f};
  PolyNode nv = n;
  if (FS == FS_GUO) uF = u[0] * F[0] + u[1] * F[1] + u[2] * F[2];
  if (FS == FS_EDM) {
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] = fmaf(F[k], irho, u[k]);
    nv = poly_node(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  }
  {  // rest population
    const float ws = (float)L::w(0) * S::template scale<LAT>(0);
    const float deq = ws * fmaf(rho, n.common, rhop);
    float r = fmaf(b, deq - d[0], d[0]);
    if (FS == FS_GUO) r = fmaf(p.guo_kt_f * ws, -uF, r);
    if (FS == FS_EDM) r = fmaf(ws * rho, nv.common - n.common, r);
    d[0] = r;
  }
#pragma unroll
  for (int q = 1; q < L::Q; ++q) {
    if (is_pair_leader<LAT>(q)) {
      const int qb = opposite<LAT>(q);
      // opposite populations share w_q and therefore S_q
      const float ws = (float)L::w(q) * S::template scale<LAT>(q);
      const float cu = cdotf<LAT>(q, u);
      float E, O;
      poly_pair(n, cu, E, O);
      const float dq = ws * fmaf(rho, E + O, rhop), dqb = ws * fmaf(rho, E - O, rhop);
      float rq = fmaf(b, dq - d[q], d[q]);
      float rqb = fmaf(b, dqb - d[qb], d[qb]);
      if (FS == FS_GUO) {
        const float cF = cdotf<LAT>(q, F);
        const float Es = fmaf(3.0f * cu, cF, -uF);
        const float kw = p.guo_kt_f * ws;
        rq = fmaf(kw, Es + cF, rq);
        rqb = fmaf(kw, Es - cF, rqb);
      }
      if (FS == FS_EDM) {
        float Ev, Ov;
        poly_pair(nv, cdotf<LAT>(q, v), Ev, Ov);
        const float wr = ws * rho;
        rq = fmaf(wr, (Ev + Ov) - (E + O), rq);
        rqb = fmaf(wr, (Ev - Ov) - (E - O), rqb);
      }
      d[q] = rq;
      d[qb] = rqb;
    }
  }
  rho_out = rho;
}

// ---- two nodes in packed FP32x2 lanes -----------------------------------------
// GB300 executes an FP32 add, multiply or FMA on a pair of floats as one
// instruction (FADD2 / FMUL2 / FFMA2): the kernels that hold two nodes a
// thread run bgk_node's arithmetic on both at half the issue slots. Every
// operation is an explicit round-to-nearest one, so the two lanes get the
// results of the scalar operations (bgk_node may contract a multiply and an
// add into one FMA where this function rounds twice: the same formula within
// FP32 rounding). The packed helpers are those of dfloat.cuh.
template <int LAT>
__device__ __forceinline__ float2 cdotf2(int q, const float2 v[3]) {
  using L = Lattice<LAT>;
  float2 r = bcast2(0.0f);
  bool first = true;
#pragma unroll
  for (int d = 0; d < L::D; ++d) {
    const int c = L::c(q, d);
    if (c == 0) continue;
    if (first) r = c > 0 ? v[d] : neg2(v[d]);
    else r = c > 0 ? add2(r, v[d]) : sub2(r, v[d]);
    first = false;
  }
  return r;
}

// the even and odd parts of the TruncationMa3 polynomial for a pair,
// A = 4.5 - 6.75 u^2 and B = 3 - 4.5 u^2 formed once a node
__device__ __forceinline__ void poly_pair2(float2 cu, float2 A, float2 B, float2 common, float2& E,
                                           float2& O) {
  const float2 c2 = mul2(cu, cu);
  E = fma2(c2, fma2(bcast2(3.375f), c2, A), common);
  O = mul2(cu, fma2(bcast2(4.5f), c2, B));
}

template <int D>
__device__ __forceinline__ void node_force_float2(const StepParams& p, uint32_t x, uint32_t y,
                                                  uint32_t z0, uint32_t z1, float2 F[3]) {
  float a[3], b[3];
  node_force_float<D>(p, x, y, z0, a);
  node_force_float<D>(p, x, y, z1, b);
#pragma unroll
  for (int k = 0; k < 3; ++k) F[k] = make_float2(a[k], b[k]);
}

// bgk_node for the nodes (x, y, z0) and (x, y, z1) in the lanes of d.
template <int LAT, int FS, int ST>
__device__ __forceinline__ void bgk_node2(const StepParams& p, uint32_t x, uint32_t y, uint32_t z0,
                                          uint32_t z1, float2 d[Lattice<LAT>::Q], float2& rho_out,
                                          float2 u[3]) {
  using L = Lattice<LAT>;
  using S = Storage<ST>;
  float2 rhop = bcast2(0.0f), j[3] = {bcast2(0.0f), bcast2(0.0f), bcast2(0.0f)};
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    const float is = 1.0f / S::template scale<LAT>(q);
    rhop = fma2(d[q], bcast2(is), rhop);
#pragma unroll
    for (int k = 0; k < L::D; ++k) {
      if (L::c(q, k) > 0) j[k] = fma2(d[q], bcast2(is), j[k]);
      if (L::c(q, k) < 0) j[k] = fma2(d[q], bcast2(-is), j[k]);
    }
  }
  const float2 rho = add2(bcast2(1.0f), rhop);
  // SFU reciprocals (within 1 ulp; u feeds FP16-rounded populations)
  float ix, iy;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ix) : "f"(rho.x));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(iy) : "f"(rho.y));
  const float2 irho = make_float2(ix, iy);
#pragma unroll
  for (int k = 0; k < 3; ++k) u[k] = mul2(j[k], irho);
  float2 F[3] = {bcast2(0.0f), bcast2(0.0f), bcast2(0.0f)};
  if (FS != FS_NONE) node_force_float2<L::D>(p, x, y, z0, z1, F);
  float2 u2 = mul2(u[0], u[0]);
#pragma unroll
  for (int k = 1; k < L::D; ++k) u2 = fma2(u[k], u[k], u2);
  const float2 common = mul2(u2, fma2(bcast2(1.125f), u2, bcast2(-1.5f)));
  const float2 A = fma2(bcast2(-6.75f), u2, bcast2(4.5f));
  const float2 B = fma2(bcast2(-4.5f), u2, bcast2(3.0f));
  // d' = d + b (d_eq - d) as (1 - b) d + b w_q (rho' + rho P_q): b w_q rho'
  // and b w_q rho once a weight
  const float bs = p.bgk_b_f;
  const float2 c1b = bcast2(1.0f - bs);
  float2 uF = bcast2(0.0f), v[3] = {bcast2(0.0f), bcast2(0.0f), bcast2(0.0f)};
  float2 commonv = common, Av = A, Bv = B;
  if (FS == FS_GUO) {
    uF = mul2(u[0], F[0]);
#pragma unroll
    for (int k = 1; k < L::D; ++k) uF = fma2(u[k], F[k], uF);
  }
  if (FS == FS_EDM) {
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] = fma2(F[k], irho, u[k]);
    float2 v2 = mul2(v[0], v[0]);
#pragma unroll
    for (int k = 1; k < L::D; ++k) v2 = fma2(v[k], v[k], v2);
    commonv = mul2(v2, fma2(bcast2(1.125f), v2, bcast2(-1.5f)));
    Av = fma2(bcast2(-6.75f), v2, bcast2(4.5f));
    Bv = fma2(bcast2(-4.5f), v2, bcast2(3.0f));
  }
  {  // rest population
    const float ws = (float)L::w(0) * S::template scale<LAT>(0);
    const float2 bw = bcast2(ws * bs);
    float2 r = fma2(mul2(bw, rho), common, fma2(c1b, d[0], mul2(bw, rhop)));
    if (FS == FS_GUO) r = fma2(bcast2(-(p.guo_kt_f * ws)), uF, r);
    if (FS == FS_EDM) r = fma2(mul2(bcast2(ws), rho), sub2(commonv, common), r);
    d[0] = r;
  }
#pragma unroll
  for (int q = 1; q < L::Q; ++q) {
    if (is_pair_leader<LAT>(q)) {
      const int qb = opposite<LAT>(q);
      const float ws = (float)L::w(q) * S::template scale<LAT>(q);
      const float2 cu = cdotf2<LAT>(q, u);
      float2 E, O;
      poly_pair2(cu, A, B, common, E, O);
      const float2 bw = bcast2(ws * bs);
      const float2 bwr = mul2(bw, rho), bwp = mul2(bw, rhop);
      float2 rq = fma2(bwr, add2(E, O), fma2(c1b, d[q], bwp));
      float2 rqb = fma2(bwr, sub2(E, O), fma2(c1b, d[qb], bwp));
      if (FS == FS_GUO) {
        const float2 cF = cdotf2<LAT>(q, F);
        const float2 Es = fma2(mul2(bcast2(3.0f), cu), cF, neg2(uF));
        const float2 kw = bcast2(p.guo_kt_f * ws);
        rq = fma2(kw, add2(Es, cF), rq);
        rqb = fma2(kw, sub2(Es, cF), rqb);
      }
      if (FS == FS_EDM) {
        float2 Ev, Ov;
        poly_pair2(cdotf2<LAT>(q, v), Av, Bv, commonv, Ev, Ov);
        const float2 wr = mul2(bcast2(ws), rho);
        rq = fma2(wr, sub2(add2(Ev, Ov), add2(E, O)), rq);
        rqb = fma2(wr, sub2(sub2(Ev, Ov), sub2(E, O)), rqb);
      }
      d[q] = rq;
      d[qb] = rqb;
    }
  }
  rho_out = rho;
}

template <int LAT, int FS, int ST>
__device__ __forceinline__ void bgk_node_fields(const StepParams& p, long long idx, uint32_t x,
                                                uint32_t y, uint32_t z, float rho,
                                                const float u[3], double& mass, double& energy,
                                                double& mach) {
  using L = Lattice<LAT>;
  if (!(rho > 0.0f) || !isfinite(rho)) atomicOr(p.err_word, ERR_NONFINITE);
  if (p.store || p.diag) {
    double Fd[3];
    node_force<L::D>(p, x, y, z, Fd);
    if (p.diag) mass = (double)rho;
    lowp_store_fields<LAT>(p, idx, rho, u, Fd, FS != FS_NONE, 2.0, energy, mach);
  }
}

template <int LAT, int FS, int ST>
__global__ void __launch_bounds__(256) bgk_lowp_kernel(const typename Storage<ST>::T* __restrict__ prev,
                                                       typename Storage<ST>::T* __restrict__ next,
                                                       StepParams p) {
  using L = Lattice<LAT>;
  using S = Storage<ST>;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = idx < p.V;
  double mass = 0.0, energy = 0.0, mach = 0.0;
  if (active) {
    uint32_t x, y, z;
    node_coords(p, idx, x, y, z);
    const PullOffsets o = pull_offsets(p, x, y, z);
    float d[L::Q];  // scaled deviations
#pragma unroll
    for (int q = 0; q < L::Q; ++q)
      d[q] = S::template load_scaled<LAT>(pop(prev, p.V, q) + o.at(L::c(q, 0), L::c(q, 1), L::c(q, 2)), q);
    float rho, u[3];
    bgk_node<LAT, FS, ST>(p, x, y, z, d, rho, u);
#pragma unroll
    for (int q = 0; q < L::Q; ++q) S::template store_scaled<LAT>(pop(next, p.V, q) + (uint32_t)idx, q, d[q]);
    bgk_node_fields<LAT, FS, ST>(p, idx, x, y, z, rho, u, mass, energy, mach);
  }
  if (p.diag) block_reduce_diag(mass, energy, mach, 2.0, 2.0, p.diag_partials);
}

// FP16-shifted storage, two z-adjacent nodes a thread (z even, Lz even): the
// populations with c_z = 0 load as one aligned half2 for both nodes, every
// population stores as one half2, the node's coordinates and periodic
// offsets are formed once for the pair, and the two collisions run in packed
// FP32x2 lanes (bgk_node2). Three blocks of 256 threads a SM (80 registers).
// Measured against four nodes a thread (one 8-byte load a population plus
// the line-edge value, 128 registers, two blocks a SM): 0.270 against
// 0.280 ms a step at 256^3 D3Q19.
template <int LAT, int FS>
__global__ void __launch_bounds__(256, 3) bgk_f16_pair_kernel(const __half* __restrict__ prev,
                                                           __half* __restrict__ next,
                                                           StepParams p) {
  using L = Lattice<LAT>;
  const long long idx = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  const bool active = idx < p.V;
  double mass = 0.0, energy = 0.0, mach = 0.0;
  if (active) {
    uint32_t x, y, z;
    node_coords(p, idx, x, y, z);  // z even
    const PullOffsets o = pull_offsets(p, x, y, z);
    // second node's z neighbours: z + 1 reads z + 2 (c_z = -1) and z (c_z = +1)
    const uint32_t z2p = (z + 2 == p.lz) ? 0 : z + 2;
    float2 d[L::Q];
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      const __half* src = pop(prev, p.V, q);
      const int cx = L::c(q, 0), cy = L::c(q, 1), cz = L::c(q, 2);
      const uint32_t xy = o.ox[cx + 1] + o.oy[cy + 1];
      if (cz == 0) {
        d[q] = __half22float2(__ldg(reinterpret_cast<const __half2*>(src + xy + z)));
      } else if (cz > 0) {  // reads z - 1 and z
        d[q] = make_float2(__half2float(__ldg(src + xy + o.oz[2])),
                           __half2float(__ldg(src + xy + z)));
      } else {  // reads z + 1 and z + 2
        d[q] = make_float2(__half2float(__ldg(src + xy + o.oz[0])),
                           __half2float(__ldg(src + xy + z2p)));
      }
    }
    float2 rho2, u2v[3];
    bgk_node2<LAT, FS, ST_F16>(p, x, y, z, z + 1, d, rho2, u2v);
#pragma unroll
    for (int q = 0; q < L::Q; ++q)
      *reinterpret_cast<__half2*>(pop(next, p.V, q) + (uint32_t)idx) = __float22half2_rn(d[q]);
    const float rho0 = rho2.x, rho1 = rho2.y;
    const float u0[3] = {u2v[0].x, u2v[1].x, u2v[2].x}, u1[3] = {u2v[0].y, u2v[1].y, u2v[2].y};
    double m1 = 0.0, e1 = 0.0, a1 = 0.0;
    bgk_node_fields<LAT, FS, ST_F16>(p, idx, x, y, z, rho0, u0, mass, energy, mach);
    bgk_node_fields<LAT, FS, ST_F16>(p, idx + 1, x, y, z + 1, rho1, u1, m1, e1, a1);
    if (p.diag) {  // FP64 only on diagnostics steps
      mass += m1;
      energy += e1;
      mach = fmax(mach, a1);
    }
  }
  if (p.diag) block_reduce_diag(mass, energy, mach, 2.0, 2.0, p.diag_partials);
}

// ---- Entropic SRT with an FP64 alpha solve --------------------------------
// The alpha solve needs f_neq with the exact mass and momentum of the stored
// state, so rho, u, f_eq and f_neq are formed in FP64 from the exact stored
// values (FP32 deviations would leave a residual mass of the order of the
// storage rounding in f_neq, and F(alpha) would then have no root in
// [1, alpha_max] on well-resolved flows). Everything else runs in FP32 or in
// integer operations: GB300 issues FP64 arithmetic and FP32<->FP64
// conversions at a small fraction of the FP32 rate, and the kernel is bound by
// that pipe.
//   * 1/f_q: an FP32 reciprocal refined by one FP64 Newton step (relative
//     error ~2^-46);
//   * alpha_max, the deviation test and the series-tier test: on FP32 r_q;
//   * F(alpha): the moment series (HSeries) when max|r_q| <= kSeriesRmax, the
//     log1p form (HLowpDirect) otherwise;
//   * the update f - alpha beta f_neq (+ forcing) in FP32, rounded once into
//     the storage format.

// The node's pulled populations as stored: F32 keeps f_q, F16 keeps the exact
// deviation f_q - w_q.
template <int LAT, int ST>
struct Pulled {
  float v[Lattice<LAT>::Q];
  __device__ __forceinline__ double f64(int q) const {
    if constexpr (ST == ST_F32) return widen_exact(v[q]);
    else return Lattice<LAT>::w(q) + widen_exact(v[q]);
  }
  __device__ __forceinline__ float f32(int q) const {
    if constexpr (ST == ST_F32) return v[q];
    else return (float)Lattice<LAT>::w(q) + v[q];
  }
  __device__ __forceinline__ float dev(int q) const {
    if constexpr (ST == ST_F32) return v[q] - (float)Lattice<LAT>::w(q);
    else return v[q];
  }
};

// 1/f to ~2^-46 relative: FP32 reciprocal, widened exactly, one Newton step.
__device__ __forceinline__ double recip_refined(double f, float f32) {
  const double y0 = widen_exact(__frcp_rn(f32));
  return fma(y0, fma(-f, y0, 1.0), y0);
}

// The log1p form of the entropy function (HLog1p, with C0 = B1 since
// sum f_neq = 0) over the stored populations and r_q.
template <int LAT, int ST>
struct HLowpDirect {
  const Pulled<LAT, ST>* P;
  const double* r;
  double B1, rmax;
  const LogEntry* tab;
  __device__ __forceinline__ void operator()(double x, double& Fv, double& Dv) const {
    using L = Lattice<LAT>;
    double s = 0.0, d = 0.0;
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      const double f = P->f64(q);
      const double t = -x * r[q];
      const double opt = 1.0 + t;
      double lp;
      if (fabs(t) <= 0.015625) lp = log1p_small(t);
      else if (opt > 0.0) lp = fast_log(opt, tab);
      else lp = -745.0;  // g = 0 at alpha_max: g ln g -> 0
      if (opt > 0.0) s = fma(f * opt, lp, s);
      d = fma(f * r[q], lp, d);
    }
    Fv = fma(x, B1, -s);
    Dv = B1 + d;
  }
};

template <int LAT, int ST, bool SERIES>
struct HLowp {
  HSeries S;
  HLowpDirect<LAT, ST> D;
  __device__ __forceinline__ void operator()(double x, double& Fv, double& Dv) const {
    if constexpr (SERIES) S(x, Fv, Dv);
    else D(x, Fv, Dv);
  }
};

// Moment tiers of the series form (max_q |r_q| = rmax <= kSeriesRmax):
//   A, rmax <= kSeriesTierA: M2 in FP64, M3..M8 as FP32 sums;
//   B, above:                M2..M4 in FP64, M5..M8 as FP32 sums.
// M2 = sum f_neq^2 / f is formed as sum f_neq^2 y0 (1 + e) with y0 the FP32
// reciprocal of the stored f and e = 1 - f y0 (exact in FP32 for F32
// storage): the FP64 part sum f_neq^2 y0 plus an FP32 correction.
// The evaluation error of F is bounded per node (F's error sources):
//   FP32 M3 (tier A):   (2.5^3/6) 2.1e-6 rho rmax^3 (9 roundings a term,
//                       26 in the sum, the seeds from the SFU reciprocal) = 6.0e-6 rho rmax^3,
//                       M4.. smaller;
//   FP32 M5 (tier B):   (2.5^5/20) 2.3e-6 rho rmax^5;
//   B1 (fast_log_fine and the FP32 tail sum): 2.5 x 2.4e-13 rho rmax;
//   FP64 rounding and the k > 8 truncation: < 1e-15.
// The solve accepts alpha when |F| <= tol - bound, so the residual of the
// exact function stays within tol.
constexpr float kSeriesTierA = 0.0025f;

// SFU reciprocal (rcp.approx.ftz.f32, relative error below 2^-22): seeds of
// the FP64 reciprocals and the FP32 r_q, where an approximation is all that
// is needed.
__device__ __forceinline__ float rcp_sfu(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// True when every weight of the lattice has the same binary significand
// (D2Q9: 4/9, 1/9, 1/36; D3Q27: 8/27 4^-k), so that the constants
// C_q(d) = d ln 2 - ln(m_q) of ln(f_q/w_q) share their second term.
template <int LAT>
__host__ __device__ constexpr bool uniform_weight_significand() {
  using L = Lattice<LAT>;
  double m0 = L::w(0);
  for (int e = exponent_of(m0); e > 0; --e) m0 *= 0.5;
  for (int e = exponent_of(L::w(0)); e < 0; ++e) m0 *= 2.0;
  for (int q = 1; q < L::Q; ++q) {
    double m = L::w(q);
    for (int e = exponent_of(L::w(q)); e > 0; --e) m *= 0.5;
    for (int e = exponent_of(L::w(q)); e < 0; ++e) m *= 2.0;
    if (m != m0) return false;
  }
  return true;
}

// v * 2^64 truncated to an integer, |v| < 2^-6 (zero for |v| < 2^-1022).
__device__ __forceinline__ long long fixed64(double v) {
  const long long b = __double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  const long long m = (b & 0x000fffffffffffffLL) | 0x0010000000000000LL;  // v = m 2^(e - 1075)
  const int sh = e - 1011;                                                 // v 2^64 = m 2^(e - 1011)
  long long a = sh >= 0 ? (m << min(sh, 10)) : (sh > -64 ? (m >> -sh) : 0LL);
  if (e == 0) a = 0;
  return b < 0 ? -a : a;
}

// With f_neq from double-float arithmetic (FP32 storage), each f_neq_q is off
// by at most 8 2^-48 rho w_q (1 + |P_q|) (eight roundings of 2^-48 on the
// operands' scale), so sum_q |delta f_neq_q| <= 8 2^-48 1.6 rho; through
// x (B1 + sum f_neq) with |ln(f/w)| <= 1: at most 2.5 x 2 x 4.6e-14 rho.
constexpr float kNeqDflBound = 2.3e-13f;

// FP32 storage forms B1 and M2 in double-float arithmetic (series_dfl): each
// ln(f/w) is within 7e-14 (the float pair of ln(1/inv_j), the exact
// reduction residual, the FP32 tail r'^2 (r'/3 - 1/2 - r'/4) with its
// roundings), so B1 is within 7.5e-14 rho rmax (products and sums add
// 2^-47 of the terms) and F within 2.5 times that; M2 carries a relative
// 1e-13 (the truncated 1/f = y0 (1 + e), double-float roundings), at most
// 3.2e-13 rho rmax^2 in F. FP16 storage keeps the FP64 sums (6e-13 rho rmax).
template <int LAT, int ST>
__device__ __forceinline__ double series_error_bound(float rabs, double rho) {
  const float r = rabs, rf = narrow_rn(rho);
  const float m = r <= kSeriesTierA ? 6.0e-6f * r * r * r : 1.2e-5f * (r * r) * (r * r) * r;
  const float dfl_term = (ST == ST_F32 && MLBM_NEQ_DFLOAT) ? kNeqDflBound : 0.0f;
  const float b1 = ST == ST_F32 ? fmaf(3.2e-13f, r, 2.0e-13f) * r : 6.0e-13f * r;
  return widen_exact(fmaf(rf, (b1 + m) + dfl_term, 1.0e-15f));
}

// B1 and the moments (series form), or r_q in place of f_neq_q in n[]
// (direct form).
template <int LAT, int ST, bool SERIES>
__device__ __forceinline__ HLowp<LAT, ST, SERIES> make_entropy_eval(const Pulled<LAT, ST>& P,
                                                                    double n[], float nfr[],
                                                                    float rabs,
                                                                    const LogEntry* tab,
                                                                    const LogEntryFine* fine,
                                                                    const double* lnw) {
  using L = Lattice<LAT>;
  HLowp<LAT, ST, SERIES> ev;
  double B1 = 0.0;
  if constexpr (SERIES) {
    const bool tierB = rabs > kSeriesTierA;
    double M2 = 0.0, M3 = 0.0, M4 = 0.0;
    float B1t = 0.0f, M2c = 0.0f, M3f = 0.0f, M4f = 0.0f, M5 = 0.0f, M6 = 0.0f, M7 = 0.0f,
          M8 = 0.0f;
    long long nd = 0;  // sum_q f_neq_q d_q 2^64 (lattices with one weight significand)
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      const double f = P.f64(q);
      const float nf = narrow_rn(n[q]);
      nfr[q] = nf;
      // B1 += f_neq ln(f/w): ln(f/w) = C_q(d) + T_j + log1p(r'), r' = m inv_j - 1
      {
        const int64_t bits = __double_as_longlong(f);
        const int d = (int)((bits >> 52) & 0x7ff) - (1023 + exponent_of(L::w(q)));
        const LogEntryFine t = fine[(bits >> 42) & (LOG_TABLE_FINE - 1)];
        const double m = __longlong_as_double((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
        const double rp = fma(m, t.inv, -1.0);
        if constexpr (uniform_weight_significand<LAT>()) {
          // sum_q f_neq_q C_q(d_q) = ln 2 sum_q f_neq_q d_q - ln(m) sum_q f_neq_q, and
          // sum_q f_neq_q = 0: the exponent term accumulates exactly in fixed point
          B1 = fma(n[q], t.hi + rp, B1);
          if (d == 1) nd += fixed64(n[q]);
          else if (d == -1) nd -= fixed64(n[q]);
          else if (d != 0) B1 = fma(n[q], exponent_as_double(d) * kLn2, B1);
        } else {
          double C;
          if (d >= -1 && d <= 1) C = lnw[3 * q + d + 1];
          else C = fma(exponent_as_double(d), kLn2, lnw[3 * q + 1]);
          B1 = fma(n[q], (C + t.hi) + rp, B1);
        }
        const float rpf = narrow_rn(rp);
        B1t = fmaf(nf, (rpf * rpf) * fmaf(rpf, 1.0f / 3.0f, -0.5f), B1t);
      }
      // moments
      const float y0f = rcp_sfu(P.f32(q));
      const double y0 = widen_exact(y0f);
      float e;
      if constexpr (ST == ST_F32) e = fmaf(-P.v[q], y0f, 1.0f);
      else e = narrow_rn(fma(-f, y0, 1.0));
      const double n2 = n[q] * n[q];
      M2 = fma(n2, y0, M2);
      const float rf = nf * y0f;
      M2c = fmaf(nf * rf, e, M2c);
      float t = nf * (rf * rf);  // f r^3
      if (tierB) {
        const double g = n[q] * fma(y0, widen_exact(e), y0);  // r_q
        const double p2 = g * n[q];
        M3 = fma(p2, g, M3);
        M4 = fma(p2 * g, g, M4);
      } else {
        M3f += t;
        M4f = fmaf(t, rf, M4f);
      }
      t *= rf * rf; M5 += t;  // f r^5
      t *= rf; M6 += t;
      t *= rf; M7 += t;
      t *= rf; M8 += t;
    }
    B1 += widen_exact(B1t);
    if constexpr (uniform_weight_significand<LAT>())
      B1 = fma((double)nd, kLn2 * 0x1p-64, B1);
    M2 += widen_exact(M2c);
    if (!tierB) { M3 = widen_exact(M3f); M4 = widen_exact(M4f); }
    ev.S = HSeries{B1, M2 * 0.5, M3 * (1.0 / 6.0), M4 * (1.0 / 12.0), M2, M3 * 0.5,
                   M4 * (1.0 / 3.0), M5 * (1.0f / 20.0f), M6 * (1.0f / 30.0f),
                   M7 * (1.0f / 42.0f), M8 * (1.0f / 56.0f), M5 * 0.25f, M6 * 0.2f,
                   M7 * (1.0f / 6.0f), M8 * (1.0f / 7.0f)};
  } else {
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      const double f = P.f64(q);
      B1 = fma(n[q], fast_log_short(f * (1.0 / L::w(q)), tab), B1);
      n[q] *= recip_refined(f, P.f32(q));
    }
  }
  ev.D = HLowpDirect<LAT, ST>{&P, n, B1, (double)rabs, tab};
  return ev;
}

// The moment-series coefficients of an FP32-storage node from f_neq in
// double-float form, with no FP64 arithmetic in the population loop:
//   B1 = sum_q f_neq_q ln(f_q/w_q), ln(f/w) = d ln2 - ln(m_q) + ln(1/inv_j)
//        + log1p(r'), r' = m inv_j - 1 (m the float mantissa of f, exact as
//        RN(m inv_j) - 1 plus the FMA residual), log1p(r') = r' + r'^2 (r'/3
//        - 1/2 - r'/4) with the tail in FP32; the d ln2 parts accumulate as
//        sum_q d_q f_neq_q, and on lattices with one weight significand the
//        -ln(m_q) parts cancel (sum_q f_neq_q = 0);
//   M2 = sum_q f_neq_q^2 / f_q with 1/f = y0 (1 + e), y0 the SFU reciprocal,
//        e = 1 - f y0 from one FMA;
// both as double-float sums (TwoSum on the running high part), rounded once
// to FP64 at the end. M3..M8 as in make_entropy_eval (FP32 sums in tier A,
// M3 and M4 in FP64 in tier B). The error bound is series_error_bound.
// One population's terms of make_series_dfl in the lanes of float pairs:
// lane x and lane y are two populations of the same weight (exponent d
// offsets and table constants alike), each lane the scalar sequence of
// operations, the sums kept per lane.
struct SeriesAcc2 {
  float2 bh, bl, eh, el, mh, ml, M3f, M4f, M5, M6, M7, M8;
};

template <int LAT>
__device__ __forceinline__ void series_terms2(float2 f, dfl2 n, int expw, const LogEntryFineF* fine,
                                              float2 C, SeriesAcc2& a) {
  constexpr bool kUniform = uniform_weight_significand<LAT>();
  const uint32_t bx = __float_as_uint(f.x), by = __float_as_uint(f.y);
  const int dx = (int)((bx >> 23) & 0xffu) - (127 + expw);
  const int dy = (int)((by >> 23) & 0xffu) - (127 + expw);
  const LogEntryFineF tx = fine[(bx >> 13) & (LOG_TABLE_FINE - 1)];
  const LogEntryFineF ty = fine[(by >> 13) & (LOG_TABLE_FINE - 1)];
  const float2 m = make_float2(__uint_as_float((bx & 0x7fffffu) | 0x3f800000u),
                               __uint_as_float((by & 0x7fffffu) | 0x3f800000u));
  const float2 inv = make_float2(tx.inv, ty.inv);
  const float2 thi = make_float2(tx.hi, ty.hi), tlo = make_float2(tx.lo, ty.lo);
  const float2 pr = mul2(m, inv);
  const float2 pe = fma2(m, inv, neg2(pr));
  const float2 pm1 = sub2(pr, bcast2(1.0f));
  const float2 rp = add2(pm1, pe);
  const float2 tail = mul2(mul2(rp, rp),
                           fma2(rp, fma2(rp, bcast2(-0.25f), bcast2(1.0f / 3.0f)), bcast2(-0.5f)));
  float2 Lh, Le, lo;
  if constexpr (kUniform) {
    two_sum2(thi, pm1, Lh, Le);
    lo = add2(add2(add2(tlo, Le), pe), tail);
  } else {
    const float2 Cx = bcast2(C.x), Cy = bcast2(C.y);
    float2 s1, e1;
    two_sum2(Cx, thi, s1, e1);
    two_sum2(s1, pm1, Lh, Le);
    lo = add2(add2(add2(add2(add2(Cy, tlo), e1), Le), pe), tail);
  }
  {  // B1 += f_neq ln(f/w)
    const float2 tp = mul2(n.hi, Lh);
    float2 te = fma2(n.hi, Lh, neg2(tp));
    te = fma2(n.hi, lo, fma2(n.lo, Lh, te));
    float2 e3;
    two_sum2(a.bh, tp, a.bh, e3);
    a.bl = add2(a.bl, add2(e3, te));
  }
  {  // sum_q d_q f_neq_q
    const float2 dd = sub2(make_float2(__int_as_float(0x4B400000 + dx), __int_as_float(0x4B400000 + dy)),
                           bcast2(12582912.0f));
    const float2 tp = mul2(n.hi, dd);
    const float2 te = fma2(n.lo, dd, fma2(n.hi, dd, neg2(tp)));
    float2 e3;
    two_sum2(a.eh, tp, a.eh, e3);
    a.el = add2(a.el, add2(e3, te));
  }
  const float2 y0 = make_float2(rcp_sfu(f.x), rcp_sfu(f.y));
  const float2 ee = fma2(neg2(f), y0, bcast2(1.0f));
  {  // M2 += f_neq^2 y0 (1 + e)
    const float2 sq = mul2(n.hi, n.hi);
    const float2 sqe = fma2(mul2(bcast2(2.0f), n.hi), n.lo, fma2(n.hi, n.hi, neg2(sq)));
    const float2 tq = mul2(sq, y0);
    float2 tqe = fma2(sq, y0, neg2(tq));
    tqe = fma2(tq, ee, fma2(sqe, y0, tqe));
    float2 e4;
    two_sum2(a.mh, tq, a.mh, e4);
    a.ml = add2(a.ml, add2(e4, tqe));
  }
  const float2 rf = mul2(n.hi, y0);
  float2 tt = mul2(n.hi, mul2(rf, rf));  // f r^3
  a.M3f = add2(a.M3f, tt);  // tier A (tier B: make_series_dfl's FP64 pass)
  a.M4f = fma2(tt, rf, a.M4f);
  tt = mul2(tt, mul2(rf, rf));
  a.M5 = add2(a.M5, tt);  // f r^5
  tt = mul2(tt, rf);
  a.M6 = add2(a.M6, tt);
  tt = mul2(tt, rf);
  a.M7 = add2(a.M7, tt);
  tt = mul2(tt, rf);
  a.M8 = add2(a.M8, tt);
}

// The moment-series coefficients of an FP32-storage node from f_neq in
// double-float form, with no FP64 arithmetic in the population loop:
//   B1 = sum_q f_neq_q ln(f_q/w_q), ln(f/w) = d ln2 - ln(m_q) + ln(1/inv_j)
//        + log1p(r'), r' = m inv_j - 1 (m the float mantissa of f, exact as
//        RN(m inv_j) - 1 plus the FMA residual), log1p(r') = r' + r'^2 (r'/3
//        - 1/2 - r'/4) with the tail in FP32; the d ln2 parts accumulate as
//        sum_q d_q f_neq_q, and on lattices with one weight significand the
//        -ln(m_q) parts cancel (sum_q f_neq_q = 0);
//   M2 = sum_q f_neq_q^2 / f_q with 1/f = y0 (1 + e), y0 the SFU reciprocal,
//        e = 1 - f y0 from one FMA;
// both as double-float sums (TwoSum on the running high part), rounded once
// to FP64 at the end. M3..M8 as in make_entropy_eval (FP32 sums in tier A,
// M3 and M4 in FP64 in tier B). The pair (q, opposite(q)) of each leader runs
// in the two lanes of packed FP32x2 instructions (series_terms2), the rest
// population in lane x ahead of the first pair; the lanes' sums are added at
// the end (two more double-float additions in the error bound). The error
// bound is series_error_bound.
template <int LAT>
__device__ __forceinline__ HSeries make_series_dfl(const Pulled<LAT, ST_F32>& P, const dfl nd[],
                                                   float nfr[], float rabs,
                                                   const LogEntryFineF* fine,
                                                   const float2* mconst) {
  using L = Lattice<LAT>;
  const bool tierB = rabs > kSeriesTierA;
  SeriesAcc2 a;
  a.bh = a.bl = a.eh = a.el = a.mh = a.ml = bcast2(0.0f);
  a.M3f = a.M4f = a.M5 = a.M6 = a.M7 = a.M8 = bcast2(0.0f);
  double M3 = 0.0, M4 = 0.0;
  {
    // the rest population in lane x, a zero term in lane y (f = 1, f_neq = 0:
    // every product with it is an exact zero)
    nfr[0] = nd[0].hi;
    const dfl2 n2 = dfl2_pack(nd[0], dfl{0.0f, 0.0f});
    series_terms2<LAT>(make_float2(P.v[0], 1.0f), n2, exponent_of(L::w(0)), fine, mconst[0], a);
  }
#pragma unroll
  for (int q = 1; q < L::Q; ++q) {
    if (!is_pair_leader<LAT>(q)) continue;
    const int qb = opposite<LAT>(q);
    nfr[q] = nd[q].hi;
    nfr[qb] = nd[qb].hi;
    series_terms2<LAT>(make_float2(P.v[q], P.v[qb]), dfl2_pack(nd[q], nd[qb]),
                       exponent_of(L::w(q)), fine, mconst[q], a);
  }
  // tier B: M3 and M4 in FP64 in a pass of their own (kept out of the packed
  // loop's code), the populations in the packed loop's order
  if (tierB) {
    auto fp64_terms = [&](float f, dfl n) {
      const float y0 = rcp_sfu(f);
      const float ee = fmaf(-f, y0, 1.0f);
      const double nq = widen_exact(n.hi) + widen_exact(n.lo);
      const double g = nq * fma(widen_exact(y0), widen_exact(ee), widen_exact(y0));  // r_q
      const double p2 = g * nq;
      M3 = fma(p2, g, M3);
      M4 = fma(p2 * g, g, M4);
    };
    fp64_terms(P.v[0], nd[0]);
#pragma unroll
    for (int q = 1; q < L::Q; ++q) {
      if (!is_pair_leader<LAT>(q)) continue;
      fp64_terms(P.v[q], nd[q]);
      fp64_terms(P.v[opposite<LAT>(q)], nd[opposite<LAT>(q)]);
    }
  }
  // B1 = (bh + bl) + ln2 (eh + el), M2 = mh + ml, over both lanes, each
  // rounded once to FP64
  auto lanes = [](float2 h, float2 l) {
    dfl x{h.x, l.x}, y{h.y, l.y};
    fast_two_sum(x.hi, x.lo, x.hi, x.lo);
    fast_two_sum(y.hi, y.lo, y.hi, y.lo);
    return dfl_add(x, y);
  };
  dfl B = lanes(a.bh, a.bl), E = lanes(a.eh, a.el), M = lanes(a.mh, a.ml);
  constexpr float kLn2F = 0x1.62e43p-1f;                  // RN_float(ln 2)
  constexpr float kLn2FLo = -0x1.05c610p-29f;             // ln 2 - kLn2F
  B = dfl_add(B, dfl_mul(E, dfl{kLn2F, kLn2FLo}));
  const double B1 = dfl_to_double(B);
  const double M2 = dfl_to_double(M);
  // the FP32 moments (tier A) scaled in FP32, M2 / 2 by an exponent step:
  // no FP64 multiply
  double a3, a4, b3, b4;
  if (!tierB) {
    const float m3 = a.M3f.x + a.M3f.y, m4 = a.M4f.x + a.M4f.y;
    a3 = widen_exact(m3 * (1.0f / 6.0f));
    a4 = widen_exact(m4 * (1.0f / 12.0f));
    b3 = widen_exact(m3 * 0.5f);
    b4 = widen_exact(m4 * (1.0f / 3.0f));
  } else {
    a3 = M3 * (1.0 / 6.0);
    a4 = M4 * (1.0 / 12.0);
    b3 = M3 * 0.5;
    b4 = M4 * (1.0 / 3.0);
  }
  const float M5 = a.M5.x + a.M5.y, M6 = a.M6.x + a.M6.y, M7 = a.M7.x + a.M7.y,
              M8 = a.M8.x + a.M8.y;
  return HSeries{B1, half_exact(M2), a3, a4, M2, b3, b4, M5 * (1.0f / 20.0f), M6 * (1.0f / 30.0f),
                 M7 * (1.0f / 42.0f), M8 * (1.0f / 56.0f), M5 * 0.25f, M6 * 0.2f,
                 M7 * (1.0f / 6.0f), M8 * (1.0f / 7.0f)};
}

// v * 2^60 as an exact integer for a float |v| < 4 (bits below 2^-60
// dropped, an absolute 1e-18); `bad` is set for larger or non-finite values.
__device__ __forceinline__ long long fixed60(float v, bool& bad) {
  const uint32_t b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 0xffu);
  bad |= e >= 129;
  const long long m = (long long)((b & 0x7fffffu) | (e ? 0x800000u : 0u));
  const int sh = e - 90;  // v = m 2^(e - 150)
  const long long a = sh >= 0 ? (m << (sh & 63)) : (m >> min(-sh, 63));
  return (b >> 31) ? -a : a;
}

// f 2^32 as an exact integer for a float f in [2^-9, 1): the significand
// with its leading one shifted left by e - 118 in [0, 8]; `bad` outside that
// range.
__device__ __forceinline__ long long fixed32(float v, bool& bad) {
  const uint32_t b = __float_as_uint(v);
  bad |= b - 0x3b000000u >= 0x04800000u;
  return (long long)(((b & 0x7fffffu) | 0x800000u) << (((b >> 23) - 118u) & 31u));
}

// rho (or rho - 1 for F16 storage, whose stored deviations sum to it) and
// the momentum as exact fixed-point sums of the stored values (2^-32 units
// for FP32 populations in [2^-9, 1), 2^-60 for the FP16 deviations), each
// rounded once to FP64; FP64 sums where a value is out of the fixed-point
// range.
template <int LAT, int ST>
__device__ __forceinline__ void moments_exact(const Pulled<LAT, ST>& P, double& rho, double& rhop,
                                              double j[3]) {
  using L = Lattice<LAT>;
  long long S = 0, J[3] = {0, 0, 0};
  bool bad = false;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    const long long a = ST == ST_F32 ? fixed32(P.v[q], bad) : fixed60(P.v[q], bad);
    S += a;
#pragma unroll
    for (int k = 0; k < L::D; ++k) {
      if (L::c(q, k) > 0) J[k] += a;
      if (L::c(q, k) < 0) J[k] -= a;
    }
  }
  if (!bad) {
    constexpr int kScale = ST == ST_F32 ? 32 : 60;
    const double Sd = ll_scaled(S, kScale);
    rho = ST == ST_F32 ? Sd : 1.0 + Sd;
    rhop = ST == ST_F32 ? Sd - 1.0 : Sd;
#pragma unroll
    for (int k = 0; k < 3; ++k) j[k] = ll_scaled(J[k], kScale);
  } else {
    rho = P.f64(0);
    j[0] = j[1] = j[2] = 0.0;
#pragma unroll
    for (int q = 1; q < L::Q; ++q) {
      const double f = P.f64(q);
      rho += f;
#pragma unroll
      for (int k = 0; k < L::D; ++k) {
        if (L::c(q, k) > 0) j[k] += f;
        if (L::c(q, k) < 0) j[k] -= f;
      }
    }
    rhop = rho - 1.0;
  }
}

// f_neq_q = f_q - rho w_q (1 + P_q) = (f_q - rho w_q) - rho w_q P_q with the
// TruncationMa3 polynomial in its pair form P(+-cu) = E +- O (Equilibrium.h:17-33).
// f_q - rho w_q is formed from the stored value: f_q - rho w_q for F32,
// (f_q - w_q) - (rho - 1) w_q for F16.
template <int LAT, int ST>
__device__ __forceinline__ void neq_pairs(const Pulled<LAT, ST>& P, double rho, double rhop,
                                          const double u[3], double n[]) {
  using L = Lattice<LAT>;
  const double u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double common = u2 * (1.125 * u2 - 1.5);
  const double A = fma(-6.75, u2, 4.5), B = fma(-4.5, u2, 3.0);
  auto base = [&](int q) {
    if constexpr (ST == ST_F32) return P.f64(q) - rho * L::w(q);
    else return widen_exact(P.v[q]) - rhop * L::w(q);
  };
  n[0] = fma(-rho * L::w(0), common, base(0));
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
      const double E = fma(c2, fma(3.375, c2, A), common);
      const double O = cu * fma(4.5, c2, B);
      const double rw = rho * L::w(q);
      n[q] = fma(-rw, E + O, base(q));
      n[qb] = fma(-rw, E - O, base(qb));
    }
  }
}

// The pair leaders of a lattice in population order (pairs (q, opposite(q))).
template <int LAT>
struct PairIndex {
  static constexpr int count() {
    int c = 0;
    for (int q = 1; q < Lattice<LAT>::Q; ++q) c += is_pair_leader<LAT>(q) ? 1 : 0;
    return c;
  }
  static constexpr int leader(int k) {
    int c = 0;
    for (int q = 1; q < Lattice<LAT>::Q; ++q) {
      if (!is_pair_leader<LAT>(q)) continue;
      if (c == k) return q;
      ++c;
    }
    return 0;
  }
};

// f_neq in double-float arithmetic (dfloat.cuh) for FP32 storage: the same
// pair form as neq_pairs, each operation on (hi, lo) float pairs, the result
// rounded once to FP64. Error: a few 2^-48 of rho w_q (1 + |P_q|) a
// population (bounded in series_error_bound), from ~20x fewer FP64-pipe
// cycles than the FP64 form. Two pairs run at a time in packed FP32x2 lanes
// (dfl2): each lane performs the scalar sequence of operations, so the
// values are those of the one-pair-at-a-time form.
template <int LAT>
__device__ __forceinline__ void neq_pairs_dfl(const Pulled<LAT, ST_F32>& P, double rho,
                                              const double u[3], dfl n[]) {
  using L = Lattice<LAT>;
  const dfl r = dfl_from(rho);
  const dfl ux = dfl_from(u[0]), uy = dfl_from(u[1]), uz = dfl_from(u[2]);
  const dfl uv[3] = {ux, uy, uz};
  dfl u2 = dfl_mul(ux, ux);
  if (L::D > 1) u2 = dfl_add(u2, dfl_mul(uy, uy));
  if (L::D > 2) u2 = dfl_add(u2, dfl_mul(uz, uz));
  const dfl common = dfl_mul(u2, dfl_add_f(dfl_mul_f(u2, 1.125f), -1.5f));
  const dfl A = dfl_add_f(dfl_mul_f(u2, -6.75f), 4.5f);
  const dfl B = dfl_add_f(dfl_mul_f(u2, -4.5f), 3.0f);
  auto rw_of = [&](int q) {
    const float wh = (float)L::w(q);
    const float wl = (float)(L::w(q) - (double)wh);
    return dfl_mul(r, dfl{wh, wl});
  };
  auto cu_of = [&](int q) {
    dfl cu{0.0f, 0.0f};
    bool first = true;
#pragma unroll
    for (int k = 0; k < L::D; ++k) {
      if (L::c(q, k) == 0) continue;
      const dfl t = L::c(q, k) > 0 ? uv[k] : dfl_neg(uv[k]);
      cu = first ? t : dfl_add(cu, t);
      first = false;
    }
    return cu;
  };
  {
    const dfl rw = rw_of(0);
    const dfl feq = dfl_add(rw, dfl_mul(rw, common));
    n[0] = dfl_add_f(dfl_neg(feq), P.v[0]);
  }
  constexpr int NP = PairIndex<LAT>::count();
  const dfl2 common2 = dfl2_pack(common, common), A2 = dfl2_pack(A, A), B2 = dfl2_pack(B, B);
#pragma unroll
  for (int k = 0; k + 1 < NP; k += 2) {
    const int qa = PairIndex<LAT>::leader(k), qb = PairIndex<LAT>::leader(k + 1);
    const dfl2 cu = dfl2_pack(cu_of(qa), cu_of(qb));
    const dfl2 c2 = dfl2_mul(cu, cu);
    const dfl2 E = dfl2_add(dfl2_mul(c2, dfl2_add(dfl2_mul_f(c2, bcast2(3.375f)), A2)), common2);
    const dfl2 O = dfl2_mul(cu, dfl2_add(dfl2_mul_f(c2, bcast2(4.5f)), B2));
    const dfl2 rw = dfl2_pack(rw_of(qa), rw_of(qb));
    const dfl2 A1 = dfl2_add(rw, dfl2_mul(rw, E));  // rho w (1 + E)
    const dfl2 B1 = dfl2_mul(rw, O);                // rho w O
    const dfl2 nA = dfl2_add_f(dfl2_neg(A1), make_float2(P.v[qa], P.v[qb]));
    const dfl2 nAb = dfl2_add_f(dfl2_neg(A1),
                                make_float2(P.v[opposite<LAT>(qa)], P.v[opposite<LAT>(qb)]));
    const dfl2 np = dfl2_sub(nA, B1);
    const dfl2 nm = dfl2_add(nAb, B1);
    n[qa] = dfl2_x(np);
    n[qb] = dfl2_y(np);
    n[opposite<LAT>(qa)] = dfl2_x(nm);
    n[opposite<LAT>(qb)] = dfl2_y(nm);
  }
  if constexpr (NP % 2 == 1) {
    const int q = PairIndex<LAT>::leader(NP - 1);
    const int qb = opposite<LAT>(q);
    const dfl cu = cu_of(q);
    const dfl c2 = dfl_mul(cu, cu);
    const dfl E = dfl_add(dfl_mul(c2, dfl_add(dfl_mul_f(c2, 3.375f), A)), common);
    const dfl O = dfl_mul(cu, dfl_add(dfl_mul_f(c2, 4.5f), B));
    const dfl rw = rw_of(q);
    const dfl A1 = dfl_add(rw, dfl_mul(rw, E));
    const dfl B1 = dfl_mul(rw, O);
    n[q] = dfl_sub(dfl_add_f(dfl_neg(A1), P.v[q]), B1);
    n[qb] = dfl_add(dfl_add_f(dfl_neg(A1), P.v[qb]), B1);
  }
}

// The same rounded once to FP64 (tests).
template <int LAT>
__device__ __forceinline__ void neq_pairs_dfl(const Pulled<LAT, ST_F32>& P, double rho,
                                              const double u[3], double n[]) {
  dfl nd[Lattice<LAT>::Q];
  neq_pairs_dfl<LAT>(P, rho, u, nd);
#pragma unroll
  for (int q = 0; q < Lattice<LAT>::Q; ++q) n[q] = dfl_to_double(nd[q]);
}

// The entropic step runs as two kernels. The main pass completes every node
// whose deviations allow the moment-series entropy function (all of them on
// resolved flows), the alpha = 2 shortcut and the alpha_max-limited nodes,
// and appends the others to a worklist; a persistent second pass finishes the
// listed nodes with the log1p form. Each kernel's register allocation then
// covers one form only (the series-only main pass fits 3 blocks of 128
// threads per SM without spills).
enum : int { ELBM_MAIN = 0, ELBM_DEFERRED = 1 };

template <int LAT, int FS, int ST, bool LEARNED, int MODE>
__device__ __forceinline__ void elbm_node(const typename Storage<ST>::T* __restrict__ prev,
                                          typename Storage<ST>::T* __restrict__ next,
                                          const StepParams& p, bool active, long long idx,
                                          const LogEntry* s_log, const LogEntryFine* s_fine,
                                          const double* s_lnw, const LogEntryFineF* s_finef,
                                          const float2* s_mconst, unsigned cnt[], bool& defer,
                                          bool& cold, double& mass,
                                          double& energy, double& mach, double& amin,
                                          double& amax) {
  using L = Lattice<LAT>;
  Pulled<LAT, ST> P;
  uint32_t x = 0, y = 0, z = 0;
  if (active) {
    node_coords(p, idx, x, y, z);
    const PullOffsets o = pull_offsets(p, x, y, z);
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      const auto* src = pop(prev, p.V, q) + o.at(L::c(q, 0), L::c(q, 1), L::c(q, 2));
      if constexpr (ST == ST_F32) P.v[q] = __ldg(src);
      else P.v[q] = __half2float(__ldg(src)) * (1.0f / (float)(1 << shift_exponent<LAT>(q)));
    }
  } else {
#pragma unroll
    for (int q = 0; q < L::Q; ++q) P.v[q] = ST == ST_F32 ? (float)L::w(q) : 0.0f;
  }
  // Learned guess: the network runs for the nodes without a solved alpha
  // from the previous step (the stored alpha is exactly 2 after
  // initialisation, a restart or an alpha = 2 fallback; a solved root is not
  // 2 to the last bit), or for every node with GUESS_LEARNED_EVERYWHERE; the
  // previous alpha is the guess elsewhere (the field holds alpha - 2, so
  // exactly 0 there). The inference is a warp tile
  // (every lane of a warp that has such a node takes part), on features
  // f_neq / rho from the FP32 deviations (computed before the FP64 part, so
  // that the inference and the FP64 f_neq are not live together).
  float learned = 0.0f;
  bool need_learned = false;
  if (LEARNED) {
    need_learned = active && (p.guess_mode == GUESS_LEARNED_EVERYWHERE ||
                              p.alpha_field_f32[idx] == 0.0f);
  }
  if (LEARNED && __any_sync(0xffffffffu, need_learned)) {
    float dv[L::Q], rhopf, rf, uf[3], deq[L::Q];
#pragma unroll
    for (int q = 0; q < L::Q; ++q) dv[q] = P.dev(q);
    moments_dev<LAT>(dv, rhopf, rf, uf);
    eq_dev<LAT>(rhopf, rf, uf, uf[0] * uf[0] + uf[1] * uf[1] + uf[2] * uf[2], deq);
    const float irf = 1.0f / rf;
    float xin[L::Q];
#pragma unroll
    for (int q = 0; q < L::Q; ++q) xin[q] = (dv[q] - deq[q]) * irf;
    learned = mlp_guess_block<L::Q>(reinterpret_cast<const MlpDev*>(p.mlp), xin);
  }
  if (!active) return;
  // rho, u and f_neq in FP64 from the exact stored values
  double rho, rhop, j[3], u[3];
  moments_exact<LAT, ST>(P, rho, rhop, j);
  const double ir = recip_refined(rho, narrow_rn(rho));
#pragma unroll
  for (int k = 0; k < 3; ++k) u[k] = j[k] * ir;
  // FP32 storage, main pass: f_neq stays in double-float form and the
  // series sums run on the FP32 pipe (make_series_dfl); otherwise FP64 f_neq
  constexpr bool kDfl = MODE == ELBM_MAIN && ST == ST_F32 && MLBM_NEQ_DFLOAT;
  double n[kDfl ? 1 : L::Q];
  dfl nd[kDfl ? L::Q : 1];
  if constexpr (kDfl) neq_pairs_dfl<LAT>(P, rho, u, nd);
  else neq_pairs<LAT, ST>(P, rho, rhop, u, n);
  auto nf_of = [&](int q) {
    if constexpr (kDfl) return nd[q].hi;
    else return narrow_rn(n[q]);
  };
  // r_q = n_q / f_q in FP32 for the bracket and the tests
  float rpos = 0.0f, rabs = 0.0f;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    const float rq = nf_of(q) * rcp_sfu(P.f32(q));
    rpos = fmaxf(rpos, rq);
    rabs = fmaxf(rabs, fabsf(rq));
  }
  // nf_q = f_neq_q rounded to FP32, all the update needs: the series form
  // fills it in its moment loop, past which the FP64 f_neq is dead
  float nf[L::Q];
  // alpha_max = min(2.5, 1 / max_q r_q) over r_q > 0 (Collision.h:305-326);
  // the deviation test |f_neq|/f <= threshold (Collision.h:284-303)
  const bool small = !(rabs > p.deviation_threshold_f);
  const double alphaMax = rpos > 0.4f ? widen_exact(__frcp_rn(rpos)) : 2.5;
  double alpha = 2.0;
  bool direct = false;  // n[] holds r_q instead of f_neq_q
  if (MODE == ELBM_MAIN && small) {
    ++cnt[CNT_SHORTCUT];
    alpha = 2.0;
#pragma unroll
    for (int q = 0; q < L::Q; ++q) nf[q] = nf_of(q);
  } else if (MODE == ELBM_MAIN && alphaMax < 2.0) {
    ++cnt[CNT_LIMITED];
    alpha = 0.95 * alphaMax;
#pragma unroll
    for (int q = 0; q < L::Q; ++q) nf[q] = nf_of(q);
  }
  else {
    const bool series = MODE == ELBM_MAIN && rabs <= kSeriesRmax;
    if (MODE == ELBM_MAIN && !series) {
      defer = true;
    } else {
      ++cnt[CNT_SOLVED];
      if (series) ++cnt[CNT_SERIES];
      direct = !series;
      const double prevA = 2.0 + widen_exact(p.alpha_field_f32[idx]);
      const double plain = p.guess_mode == GUESS_TWO ? 2.0 : prevA;
      const double guess = LEARNED && need_learned ? 2.0 + widen_exact(learned) : plain;
      if (LEARNED && need_learned) ++cnt[CNT_INFER];
      if constexpr (kDfl) {
        const HSeries ev = make_series_dfl<LAT>(P, nd, nf, rabs, s_finef, s_mconst);
        const double tol = p.newton_tol - series_error_bound<LAT, ST>(rabs, rho);
        alpha = residual_alpha_solve<HSeries, true>(ev, guess, plain, alphaMax, tol,
                                                    p.newton_maxit, p.bisect_maxit, cnt);
      } else if constexpr (MODE == ELBM_MAIN) {
        const auto ev = make_entropy_eval<LAT, ST, true>(P, n, nf, rabs, s_log, s_fine, s_lnw);
        const double tol = p.newton_tol - series_error_bound<LAT, ST>(rabs, rho);
        alpha = residual_alpha_solve<decltype(ev), true>(ev, guess, plain, alphaMax, tol,
                                                         p.newton_maxit, p.bisect_maxit, cnt);
      } else {
        const auto ev = make_entropy_eval<LAT, ST, false>(P, n, nf, rabs, s_log, s_fine, s_lnw);
        alpha = residual_alpha_solve<decltype(ev), true>(ev, guess, plain, alphaMax,
                                                         p.newton_tol - 4e-15, p.newton_maxit,
                                                         p.bisect_maxit, cnt);
      }
    }
  }
  if (!defer) {
    // update in FP32: f - alpha beta f_neq + S (Collision.h:243-258)
    // alpha beta in FP32 (2 beta = bgk_b_f exactly halved): its rounding
    // scales f_neq, a small part of the FP32-rounded update
    const float ab = narrow_rn(alpha) * (0.5f * p.bgk_b_f);
    float uf[3] = {0.0f, 0.0f, 0.0f}, Ff[3] = {0.0f, 0.0f, 0.0f}, rf = 1.0f, uF = 0.0f;
    PolyNode nu{0.0f, 0.0f}, nv{0.0f, 0.0f};
    float vf[3] = {0.0f, 0.0f, 0.0f};
    if (FS != FS_NONE) {
      node_force_float<L::D>(p, x, y, z, Ff);
#pragma unroll
      for (int k = 0; k < 3; ++k) uf[k] = narrow_rn(u[k]);
      rf = narrow_rn(rho);
      uF = uf[0] * Ff[0] + uf[1] * Ff[1] + uf[2] * Ff[2];
      if (FS == FS_EDM) {
        nu = poly_node(uf[0] * uf[0] + uf[1] * uf[1] + uf[2] * uf[2]);
        const float irf = 1.0f / rf;
#pragma unroll
        for (int k = 0; k < 3; ++k) vf[k] = fmaf(Ff[k], irf, uf[k]);
        nv = poly_node(vf[0] * vf[0] + vf[1] * vf[1] + vf[2] * vf[2]);
      }
    }
    float src[L::Q];
#pragma unroll
    for (int q = 0; q < L::Q; ++q) src[q] = 0.0f;
    if (FS == FS_GUO || FS == FS_EDM) {
      if (FS == FS_GUO) src[0] = -(p.guo_kt_f * (float)L::w(0)) * uF;
      else src[0] = (float)L::w(0) * rf * (nv.common - nu.common);
#pragma unroll
      for (int q = 1; q < L::Q; ++q) {
        if (is_pair_leader<LAT>(q)) {
          const int qb = opposite<LAT>(q);
          const float w = (float)L::w(q);
          if (FS == FS_GUO) {
            // S_q = kt w_q [(c_q - u).F + 3 (c_q.u)(c_q.F)] (ForcingScheme.h:100-117)
            const float cF = cdotf<LAT>(q, Ff);
            const float Es = fmaf(3.0f * cdotf<LAT>(q, uf), cF, -uF);
            const float kw = p.guo_kt_f * w;
            src[q] = kw * (Es + cF);
            src[qb] = kw * (Es - cF);
          } else {
            // S_q = f_eq(rho, u + F/rho) - f_eq(rho, u) (ForcingScheme.h:183-197)
            float E, O, Ev, Ov;
            poly_pair(nu, cdotf<LAT>(q, uf), E, O);
            poly_pair(nv, cdotf<LAT>(q, vf), Ev, Ov);
            const float wr = w * rf;
            src[q] = wr * ((Ev + Ov) - (E + O));
            src[qb] = wr * ((Ev - Ov) - (E - O));
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
      float nfq = nf[q];
      if constexpr (!kDfl) {
        if (direct) nfq = narrow_rn(n[q] * P.f64(q));
      }
      float rr = fmaf(-ab, nfq, P.v[q]);  // f (F32) or f - w (F16)
      if (FS == FS_GUO || FS == FS_EDM) rr += src[q];
      auto* dst = pop(next, p.V, q) + (uint32_t)idx;
      if constexpr (ST == ST_F32) *dst = rr;
      else *dst = __float2half_rn(rr * (float)(1 << shift_exponent<LAT>(q)));
    }
    // alpha persists as alpha - 2 in FP32: near 2 its rounding is ~1e-11
    // absolute, so the previous alpha stays a guess to FP64 accuracy
    const float stored = narrow_rn(alpha - 2.0);
    p.alpha_field_f32[idx] = stored;
    cold |= stored == 0.0f;
    if (p.diag) {
      const double a = 2.0 + widen_exact(stored);
      if (MODE == ELBM_MAIN) {  // one node a thread: no FP64 compares
        amin = a;
        amax = a;
      } else {
        amin = fmin(amin, a);
        amax = fmax(amax, a);
      }
    }
  }
  if (MODE == ELBM_MAIN) {
    {  // rho positive and finite, tested on its bits (no FP64 compare)
      const long long rb = __double_as_longlong(rho);
      if (rb <= 0 || rb >= 0x7ff0000000000000LL) atomicOr(p.err_word, ERR_NONFINITE);
    }
    if (p.store || p.diag) {
      // rho, u_hydro and F of every node; alpha by the kernel that solves it
      mass = rho;
      double F[3] = {0.0, 0.0, 0.0};
      if (FS != FS_NONE) node_force<L::D>(p, x, y, z, F);
      store_fields_f64<LAT>(p, idx, rho, u, F, FS != FS_NONE, alpha, energy, mach, !defer);
    }
  }
}

// Resident blocks per SM the main pass's register allocation is sized for:
// 4 blocks of 128 threads (128 registers, a few spills). Measured on the 512^3
// entropic workload, 4 blocks beat 3 (156 registers, no spills) for both
// variants: 1177 against 1078 MLUPS with the previous-alpha guess, 1096
// against 1004 with the learned guess; the extra warps hide the phases in
// which the FP64 pipe would otherwise idle (loads, inference).
#ifndef MLBM_ELBM_MIN_BLOCKS
#define MLBM_ELBM_MIN_BLOCKS 4
#endif
#ifndef MLBM_ELBM_MIN_BLOCKS_LEARNED
#define MLBM_ELBM_MIN_BLOCKS_LEARNED 4
#endif

template <int LAT, int FS, int ST, bool LEARNED>
__global__ void __launch_bounds__(128, LEARNED ? MLBM_ELBM_MIN_BLOCKS_LEARNED : MLBM_ELBM_MIN_BLOCKS) elbm_lowp_kernel(const typename Storage<ST>::T* __restrict__ prev,
                                                        typename Storage<ST>::T* __restrict__ next,
                                                        StepParams p) {
  // FP32 storage: the float table of the double-float series sums; FP16
  // storage: the FP64 table
  constexpr bool kDfl = ST == ST_F32 && MLBM_NEQ_DFLOAT;
  __shared__ __align__(16) LogEntryFineF s_finef[kDfl ? LOG_TABLE_FINE : 1];
  __shared__ float2 s_mconst[kDfl ? 27 : 1];
  __shared__ LogEntryFine s_fine[kDfl ? 1 : LOG_TABLE_FINE];
  __shared__ double s_lnw[kDfl ? 1 : LNW_CONSTS];
  if constexpr (kDfl)
    stage_log_table_fine_f(s_finef, s_mconst, reinterpret_cast<const FineTables*>(p.log_table_fine));
  else
    stage_log_table_fine(s_fine, s_lnw, reinterpret_cast<const LogEntryFine*>(p.log_table_fine));
  // the worklist counter of the next step (its last reader was the previous
  // step's second pass, which has completed)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    p.defer_count[p.parity ^ 1] = 0u;
    if (p.cold_flags) p.cold_flags[p.parity ^ 1] = 0u;
  }
  __syncthreads();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = idx < p.V;
  double mass = 0.0, energy = 0.0, mach = 0.0, amin = 1e300, amax = -1e300;
  unsigned cnt[CNT_COUNT] = {};
  bool defer = false, cold = false;
  elbm_node<LAT, FS, ST, LEARNED, ELBM_MAIN>(prev, next, p, active, idx, nullptr, s_fine, s_lnw,
                                             s_finef, s_mconst, cnt, defer, cold, mass, energy,
                                             mach, amin, amax);
  if (p.cold_flags && __any_sync(0xffffffffu, cold) && (threadIdx.x & 31) == 0)
    p.cold_flags[p.parity] = 1u;
  // warp-aggregated append to the worklist
  const unsigned m = __ballot_sync(0xffffffffu, defer);
  if (m) {
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(p.defer_count + p.parity, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (defer) p.defer_list[base + __popc(m & ((1u << lane) - 1u))] = (unsigned)idx;
  }
  add_counters(p.counters, cnt);
  if (p.diag) block_reduce_diag(mass, energy, mach, amin, amax, p.diag_partials);
}

// Second pass over the worklist (grid-stride; p.defer_blocks blocks).
template <int LAT, int FS, int ST, bool LEARNED>
__global__ void __launch_bounds__(128) elbm_lowp_deferred_kernel(const typename Storage<ST>::T* __restrict__ prev,
                                                                 typename Storage<ST>::T* __restrict__ next,
                                                                 StepParams p) {
  __shared__ LogEntry s_log[LOG_TABLE];
  stage_log_table(s_log, reinterpret_cast<const LogEntry*>(p.log_table));
  __syncthreads();
  const long long count = (long long)p.defer_count[p.parity];
  double mass = 0.0, energy = 0.0, mach = 0.0, amin = 1e300, amax = -1e300;
  unsigned cnt[CNT_COUNT] = {};
  bool cold = false;
  for (long long b = (long long)blockIdx.x * blockDim.x; b < count;
       b += (long long)gridDim.x * blockDim.x) {
    const long long i = b + threadIdx.x;
    const bool active = i < count;
    const long long idx = active ? (long long)p.defer_list[i] : 0;
    bool defer = false;
    elbm_node<LAT, FS, ST, LEARNED, ELBM_DEFERRED>(prev, next, p, active, idx, s_log, nullptr,
                                                   nullptr, nullptr, nullptr, cnt, defer, cold,
                                                   mass, energy, mach, amin, amax);
  }
  if (p.cold_flags && __any_sync(0xffffffffu, cold) && (threadIdx.x & 31) == 0)
    p.cold_flags[p.parity] = 1u;
  add_counters(p.counters, cnt);
  if (p.diag)
    block_reduce_diag(0.0, 0.0, 0.0, amin, amax,
                      p.diag_partials + (size_t)p.defer_slot0 * DIAG_FIELDS);
}

// ---- entropy-function test hook ---------------------------------------------
// F(x), F'(x) of nodes given as FP32 populations and FP64 f_neq, through the
// same construction as the step kernel; mode 0 picks the form as the kernel
// does, 1 forces the direct form, 2 the series form.
template <int LAT>
__global__ void entropy_test_kernel(const float* __restrict__ f, const double* __restrict__ fneq,
                                    long long nodes, const double* __restrict__ xs, int nx,
                                    int mode, const LogEntry* __restrict__ table,
                                    const LogEntryFine* __restrict__ table_fine,
                                    double* __restrict__ Fo, double* __restrict__ Do,
                                    int* __restrict__ series_out) {
  using L = Lattice<LAT>;
  __shared__ LogEntry s_log[LOG_TABLE];
  __shared__ __align__(16) LogEntryFineF s_finef[LOG_TABLE_FINE];
  __shared__ float2 s_mconst[27];
  stage_log_table(s_log, table);
  stage_log_table_fine_f(s_finef, s_mconst, reinterpret_cast<const FineTables*>(table_fine));
  __syncthreads();
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nodes) return;
  Pulled<LAT, ST_F32> P;
  double n[L::Q];
  float rabs = 0.0f, nf[L::Q];
#pragma unroll
  for (int q = 0; q < L::Q; ++q) {
    P.v[q] = f[s * L::Q + q];
    n[q] = fneq[s * L::Q + q];
    nf[q] = narrow_rn(n[q]);
    rabs = fmaxf(rabs, fabsf(nf[q] * rcp_sfu(P.v[q])));
  }
  const bool series = mode == 2 || (mode == 0 && rabs <= kSeriesRmax);
  if (series) {
    // the main pass's form: f_neq as double-float pairs, B1 and M2 in
    // double-float arithmetic
    dfl nd[L::Q];
#pragma unroll
    for (int q = 0; q < L::Q; ++q) nd[q] = dfl_from(n[q]);
    const HSeries ev = make_series_dfl<LAT>(P, nd, nf, rabs, s_finef, s_mconst);
    for (int i = 0; i < nx; ++i) ev(xs[i], Fo[s * nx + i], Do[s * nx + i]);
  } else {
    const auto ev = make_entropy_eval<LAT, ST_F32, false>(P, n, nf, rabs, s_log, nullptr, nullptr);
    for (int i = 0; i < nx; ++i) ev(xs[i], Fo[s * nx + i], Do[s * nx + i]);
  }
  series_out[s] = series ? 1 : 0;
}

// f_neq of nodes given as FP32 populations [nodes][Q], as the FP32-storage
// entropic main pass forms it (exact fixed-point moments, then double-float
// or FP64 pair form), for accuracy tests.
template <int LAT>
__global__ void neq_test_kernel(const float* __restrict__ f, long long nodes, int dfloat,
                                double* __restrict__ out) {
  using L = Lattice<LAT>;
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nodes) return;
  Pulled<LAT, ST_F32> P;
#pragma unroll
  for (int q = 0; q < L::Q; ++q) P.v[q] = f[s * L::Q + q];
  double rho, rhop, j[3], u[3], n[L::Q];
  moments_exact<LAT, ST_F32>(P, rho, rhop, j);
  const double ir = recip_refined(rho, narrow_rn(rho));
#pragma unroll
  for (int k = 0; k < 3; ++k) u[k] = j[k] * ir;
  if (dfloat) neq_pairs_dfl<LAT>(P, rho, u, n);
  else neq_pairs<LAT, ST_F32>(P, rho, rhop, u, n);
#pragma unroll
  for (int q = 0; q < L::Q; ++q) out[s * L::Q + q] = n[q];
}

// ---- init and conversions ---------------------------------------------------
// f_eq(rho, u) of the TruncationMa3 polynomial (Equilibrium.h:17-33) in its
// pair form, in double-float arithmetic (about 46 significant bits from the
// FP64 rho and u), rounded once into the storage format: the correctly rounded
// storage value of the exact equilibrium except for the rare values within
// ~2^-44 of a rounding boundary. The same polynomial in FP64 takes GB300's
// narrow FP64 pipe about ten times as long.
template <int LAT>
__device__ __forceinline__ dfl weight_dfl(int q) {
  const double w = Lattice<LAT>::w(q);
  const float h = (float)w;
  return {h, (float)(w - (double)h)};
}

template <int LAT, int ST>
__global__ void init_lowp_kernel(const double* __restrict__ rho, const double* __restrict__ u,
                                 typename Storage<ST>::T* __restrict__ f, long long V) {
  using L = Lattice<LAT>;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= V) return;
  dfl uu[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
#pragma unroll
  for (int k = 0; k < L::D; ++k) uu[k] = dfl_from(u[(long long)k * V + idx]);
  const dfl r = dfl_from(rho[idx]);
  dfl u2 = dfl_mul(uu[0], uu[0]);
#pragma unroll
  for (int k = 1; k < L::D; ++k) u2 = dfl_add(u2, dfl_mul(uu[k], uu[k]));
  // u^2 (1.125 u^2 - 1.5), 4.5 - 6.75 u^2, 3 - 4.5 u^2
  const dfl common = dfl_mul(u2, dfl_add_f(dfl_mul_f(u2, 1.125f), -1.5f));
  const dfl A = dfl_add_f(dfl_mul_f(u2, -6.75f), 4.5f);
  const dfl B = dfl_add_f(dfl_mul_f(u2, -4.5f), 3.0f);
  auto put = [&](int q, dfl P) {  // f_q = rho w_q P
    const dfl v = dfl_mul(dfl_mul(r, weight_dfl<LAT>(q)), P);
    auto* dst = pop(f, V, q) + (uint32_t)idx;
    if constexpr (ST == ST_F32) {
      *dst = __fadd_rn(v.hi, v.lo);
    } else {
      const dfl d = dfl_sub(v, weight_dfl<LAT>(q));
      *dst = __float2half_rn(__fadd_rn(d.hi, d.lo) * (float)(1 << shift_exponent<LAT>(q)));
    }
  };
  put(0, dfl_add_f(common, 1.0f));
#pragma unroll
  for (int q = 1; q < L::Q; ++q) {
    if (is_pair_leader<LAT>(q)) {
      const int qb = opposite<LAT>(q);
      dfl cu = {0.0f, 0.0f};
      bool first = true;
#pragma unroll
      for (int k = 0; k < L::D; ++k) {
        if (L::c(q, k) == 0) continue;
        const dfl t = L::c(q, k) > 0 ? uu[k] : dfl_neg(uu[k]);
        cu = first ? t : dfl_add(cu, t);
        first = false;
      }
      const dfl c2 = dfl_mul(cu, cu);
      const dfl E = dfl_add(dfl_mul(c2, dfl_add(dfl_mul_f(c2, 3.375f), A)), common);
      const dfl O = dfl_mul(cu, dfl_add(dfl_mul_f(c2, 4.5f), B));
      put(q, dfl_add_f(dfl_add(E, O), 1.0f));
      put(qb, dfl_add_f(dfl_sub(E, O), 1.0f));
    }
  }
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
    f[q] = load_f64<LAT, ST>(pop(prev, p.V, q) + o.at(L::c(q, 0), L::c(q, 1), L::c(q, 2)), q);
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
  alpha[s] = 2.0 + (double)p.alpha_field_f32[idx];
  solved[s] = (!small && alphaMax >= 2.0) ? 1 : 0;
}

// ---- host launchers -----------------------------------------------------------
template <int LAT, int FS, int ST>
static cudaError_t launch_lowp(int collision, const void* prev, void* next, const StepParams& p,
                               cudaStream_t s) {
  using T = typename Storage<ST>::T;
  if (collision == 0) {
    const int bs = 256;
    if (bgk_pairs(LAT, ST, p.lz)) {
      const unsigned grid = (unsigned)bgk_step_blocks(LAT, ST, p.V, p.lz);
      bgk_f16_pair_kernel<LAT, FS><<<grid, bs, 0, s>>>((const __half*)prev, (__half*)next, p);
    } else {
      const unsigned grid = (unsigned)((p.V + bs - 1) / bs);
      bgk_lowp_kernel<LAT, FS, ST><<<grid, bs, 0, s>>>((const T*)prev, (T*)next, p);
    }
  } else {
    const int bs = 128;
    const unsigned grid = (unsigned)((p.V + bs - 1) / bs);
    if (p.learned_kernel) {
      elbm_lowp_kernel<LAT, FS, ST, true><<<grid, bs, 0, s>>>((const T*)prev, (T*)next, p);
      elbm_lowp_deferred_kernel<LAT, FS, ST, true><<<p.defer_blocks, bs, 0, s>>>((const T*)prev, (T*)next, p);
    } else {
      elbm_lowp_kernel<LAT, FS, ST, false><<<grid, bs, 0, s>>>((const T*)prev, (T*)next, p);
      elbm_lowp_deferred_kernel<LAT, FS, ST, false><<<p.defer_blocks, bs, 0, s>>>((const T*)prev, (T*)next, p);
    }
  }
  return cudaGetLastError();
}

// This file is compiled once per (lattice, storage, forcing scheme) triple
// (MLBM_LAT = 0..3: D2Q9, D3Q19, D3Q27, D3Q15 -- the lattices of reach 1 with
// inv_cs2 = 3 and a conserving equilibrium, which this file's pair algebra and
// series form assume; MLBM_ST = 1 F32 or 2 F16-shifted; MLBM_FS = 0..3: None,
// Guo, Shan-Chen, EDM), so that the units build in parallel. Each unit holds
// the step kernels of its forcing scheme; the FS_NONE unit also holds the
// (lattice, storage) pair's dispatcher and the kernels that do not depend on
// the forcing scheme. misc.cu dispatches on the lattice and storage.
#if !defined(MLBM_LAT) || !defined(MLBM_ST) || !defined(MLBM_FS)
#error "compile step_lowp.cu with -DMLBM_LAT=<0..3> -DMLBM_ST=<1|2> -DMLBM_FS=<0..3>"
#endif
#define MLBM_CAT2(a, b, c, d) a##b##c##d
#define MLBM_CAT(a, b, c, d) MLBM_CAT2(a, b, c, d)
#define MLBM_FN(name) MLBM_CAT(name, MLBM_LAT, _S, MLBM_ST)
#define MLBM_FN_FS(fs) MLBM_CAT(MLBM_FN(step_lowp_L), _F, fs, )
using StT = typename Storage<MLBM_ST>::T;

// one forcing scheme's step launches
cudaError_t MLBM_FN_FS(0)(int collision, const void* prev, void* next, const StepParams& p,
                          cudaStream_t s);
cudaError_t MLBM_FN_FS(1)(int collision, const void* prev, void* next, const StepParams& p,
                          cudaStream_t s);
cudaError_t MLBM_FN_FS(2)(int collision, const void* prev, void* next, const StepParams& p,
                          cudaStream_t s);
cudaError_t MLBM_FN_FS(3)(int collision, const void* prev, void* next, const StepParams& p,
                          cudaStream_t s);

cudaError_t MLBM_FN_FS(MLBM_FS)(int collision, const void* prev, void* next, const StepParams& p,
                                cudaStream_t s) {
  return launch_lowp<MLBM_LAT, MLBM_FS, MLBM_ST>(collision, prev, next, p, s);
}

#if MLBM_FS == 0
cudaError_t MLBM_FN(step_lowp_L)(int collision, int fs, const void* prev, void* next,
                                 const StepParams& p, cudaStream_t s) {
  static_assert(FS_NONE == 0 && FS_GUO == 1 && FS_SHANCHEN == 2 && FS_EDM == 3,
                "the units are numbered by the forcing scheme's value");
  switch (fs) {
    case FS_NONE: return MLBM_FN_FS(0)(collision, prev, next, p, s);
    case FS_GUO: return MLBM_FN_FS(1)(collision, prev, next, p, s);
    case FS_SHANCHEN: return MLBM_FN_FS(2)(collision, prev, next, p, s);
    case FS_EDM: return MLBM_FN_FS(3)(collision, prev, next, p, s);
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

#if MLBM_ST == 1
cudaError_t MLBM_CAT(neq_test_L, MLBM_LAT, , )(const float* f, long long nodes, int dfloat,
                                              double* out, cudaStream_t s) {
  neq_test_kernel<MLBM_LAT><<<(unsigned)((nodes + 127) / 128), 128, 0, s>>>(f, nodes, dfloat, out);
  return cudaGetLastError();
}

cudaError_t MLBM_CAT(entropy_test_L, MLBM_LAT, , )(const float* f, const double* fneq, long long nodes,
                                                  const double* x, int nx, int mode,
                                                  const void* table, const void* table_fine,
                                                  double* F, double* D, int* series,
                                                  cudaStream_t s) {
  entropy_test_kernel<MLBM_LAT><<<(unsigned)((nodes + 127) / 128), 128, 0, s>>>(
      f, fneq, nodes, x, nx, mode, (const LogEntry*)table, (const LogEntryFine*)table_fine, F, D,
      series);
  return cudaGetLastError();
}
#endif

cudaError_t MLBM_FN(log_samples_lowp_L)(const void* prev, const StepParams& p,
                                        const long long* nodes, long long n, double* features,
                                        double* alpha, int* solved, cudaStream_t s) {
  samples_lowp_kernel<MLBM_LAT, MLBM_ST><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
      (const StT*)prev, p, nodes, n, features, alpha, solved);
  return cudaGetLastError();
}
#endif  // MLBM_FS == 0

}  // namespace mlbm
