// FP64-storage BGK step with the collision on the integer pipe.
//
// GB300 executes FP64 arithmetic at 1/73 of the FP32 rate, so the
// reference-order kernel (step_f64.cu, ~740 separately rounded FP64
// operations a node) is bound by that pipe at a few percent of HBM. This
// kernel keeps the FP64 populations in HBM and computes the same update,
//   f'_q = f_q + omega (f_eq_q - f_q) + S_q   (Collision.h:134-151, omega = 2 beta),
// in 64-bit fixed point on the integer pipe:
//   * F_q = f_q 2^60 (exact for f_q >= 2^-8, rounded below), D_q = F_q - W_q
//     with W_q = w_q 2^60, the reference's double weights exactly;
//   * rho and j = sum_q c_q f_q as exact integer sums (Moment.h:13-47);
//   * 1/rho by two Newton steps in 2^62 fixed point, u = j/rho in 2^64
//     fixed point;
//   * f_eq_q - f_q = [w_q rho - f_q + 3 w_q c_q.j] + w_q rho R_q, the linear
//     part of Equilibrium<TruncationMa3> (Equilibrium.h:17-33) exact from j,
//     R_q = 4.5 s^2 - 1.5 u^2 + 4.5 s^3 - 4.5 s u^2 + 1.125 u^4 - 6.75 s^2 u^2
//     + 3.375 s^4 (s = c_q.u) in 2^64 fixed point, the pair (q, -q) sharing
//     its even and odd parts;
//   * Guo's source ((1 - 1/(2 tau)) w_q 3) [(c_q - u).F + 3 (c_q.u)(c_q.F)]
//     (ForcingScheme.h:81-118) in fixed point;
//   * f'_q rounded once to FP64, to nearest even.
// Each fixed-point product carries at most 2^-64 relative to O(1) or one unit
// of 2^-60 absolute, so a population's update is within a few 2^-60 of the
// exact value of the reference's formula: within a few FP64 ulp of the
// reference's own result for populations above 2^-6 (the tests hold it to
// 1e-12 relative over hundreds of steps).
//
// Nodes outside the fixed-point ranges (a population outside [0, 2),
// |f_q - w_q| >= 1/4, rho outside (0.53, 2), |u| >= 0.1, |F_d| >= 1/8, or a
// non-finite value) take the reference-order arithmetic of ref_node.cuh: a
// warp with such a node computes all its nodes that way (bit-identical to the
// reference for them). Lattices D2Q9, D3Q19, D3Q27, D3Q15 (reach 1,
// inv_cs2 = 3); forcing None, Guo, Shan-Chen (EDM uses the reference-order
// kernel).
//
// This unit is compiled with -fmad=false for the reference-order fallback.

#include "common.cuh"
#include "kernels.h"
#include "ref_node.cuh"

namespace mlbm {
namespace fx {

// ---- 64-bit fixed-point helpers ---------------------------------------------

// high 64 bits of the signed 128-bit product (floor)
__device__ __forceinline__ long long mulhi(long long a, long long b) { return __mul64hi(a, b); }

// (a b + 2^63) >> 64: the product's high part rounded to nearest
__device__ __forceinline__ long long mulhi_rn(long long a, long long b) {
  const unsigned long long lo = (unsigned long long)a * (unsigned long long)b;
  return __mul64hi(a, b) + (long long)(lo >> 63);
}

// (a b) >> k for 0 < k < 64, from the signed 128-bit product (floor)
__device__ __forceinline__ long long mulshr(long long a, long long b, int k) {
  const unsigned long long lo = (unsigned long long)a * (unsigned long long)b;
  const long long hi = __mul64hi(a, b);
  return (long long)(((unsigned long long)hi << (64 - k)) | (lo >> k));
}

// v 2^S rounded to nearest for a double v; `bad` when v is not finite or
// |v| 2^S >= 2^62.
template <int S>
__device__ __forceinline__ long long to_fixed(double v, bool& bad) {
  const long long b = __double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  const long long m = (b & 0x000fffffffffffffLL) | 0x0010000000000000LL;  // |v| = m 2^(e - 1075)
  const int sh = e - 1075 + S;                                             // |v| 2^S = m 2^sh
  long long a;
  if (sh >= 0) {
    bad |= sh > 8;  // m < 2^53: m 2^8 < 2^61
    a = m << (sh & 15);
  } else if (sh > -62) {
    a = (m + (1LL << (-sh - 1))) >> (-sh);
  } else {
    a = 0;
  }
  if (e == 0) a = 0;  // zero and subnormals
  bad |= e == 0x7ff;
  return b < 0 ? -a : a;
}

// v 2^-S rounded to the nearest double (ties to even), |v| < 2^63.
template <int S>
__device__ __forceinline__ double to_double(long long v) {
  if (v == 0) return 0.0;
  const unsigned long long sign = v < 0 ? 0x8000000000000000ULL : 0ULL;
  const unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
  const int lz = __clzll((long long)a);
  const unsigned long long n = a << lz;  // leading one at bit 63
  unsigned long long mant = n >> 11;     // 53 bits
  const unsigned long long rest = n & 0x7ffULL;
  mant += (rest > 0x400ULL || (rest == 0x400ULL && (mant & 1ULL))) ? 1ULL : 0ULL;
  long long e = 63 - lz - S + 1023;      // the leading one is 2^(63 - lz - S)
  if (mant >> 53) {                      // rounded up to 2^53
    mant >>= 1;
    ++e;
  }
  return __longlong_as_double((long long)(sign | ((unsigned long long)e << 52) |
                                          (mant & 0x000fffffffffffffULL)));
}

// ---- lattice constants -------------------------------------------------------
template <int LAT>
struct FxConst {
  using L = Lattice<LAT>;
  // w_q 2^60 (exact: the double weight times a power of two is an integer)
  static constexpr long long W60(int q) { return (long long)(L::w(q) * 1152921504606846976.0); }
  // w_q 2^64 (< 2^63 for w_q < 1/2)
  static constexpr long long W64(int q) { return (long long)(L::w(q) * 18446744073709551616.0); }
  // 3 w_q 2^64 (moving populations: 3 w_q < 1/2)
  static constexpr long long W3_64(int q) {
    return (long long)(3.0 * L::w(q) * 18446744073709551616.0);
  }
  static constexpr long long sumW() {
    long long s = 0;
    for (int q = 0; q < L::Q; ++q) s += W60(q);
    return s;
  }
  // w_q sum_q' W_q' - W_q = w_q (sum W - 2^60): the rounding of the weights'
  // sum spread over the populations (a few units of 2^-60)
  static constexpr long long C(int q) {
    const double t = L::w(q) * (double)(sumW() - 1152921504606846976LL);
    return (long long)(t >= 0 ? t + 0.5 : t - 0.5);
  }
};

// The reference's BGK coefficients as fixed-point multipliers: omega T =
// a T + sign mulhi_rn(T, m) with m < 2^63 (StepParams fx_omega_*), and
// Guo's ((1 - 1/(2 tau)) w_q inv_cs2) in 2^62 fixed point (fx_guo62).

// One node in fixed point. Returns false, for every lane of the warp, when a
// lane of the warp is outside the fixed-point ranges (nothing is stored then);
// every lane of the warp must call it (inactive lanes with f = w).
template <int LAT, int FS>
__device__ __forceinline__ bool bgk_node_fixed(const double f[], const double F[3],
                                               const StepParams& p, long long idx, bool active,
                                               double* __restrict__ next, double& mass,
                                               double& energy, double& mach) {
  bool bad = false;
  using L = Lattice<LAT>;
  using K = FxConst<LAT>;
  constexpr int Q = L::Q;
  // populations as deviations from the weights, 2^60 fixed point
  long long Dq[Q];
  long long drho = 0, j[3] = {0, 0, 0};
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const long long Fq = to_fixed<60>(f[q], bad);
    bad |= Fq < 0;
    Dq[q] = Fq - K::W60(q);
    const long long ad = Dq[q] < 0 ? -Dq[q] : Dq[q];
    bad |= ad >= (1LL << 58);
    drho += Dq[q];
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(q, d) > 0) j[d] += Dq[q];
      if (L::c(q, d) < 0) j[d] -= Dq[q];
    }
  }
  const long long rhoF = K::sumW() + drho;  // rho 2^60
  bad |= rhoF <= (1LL << 59) + (1LL << 55) || rhoF >= (1LL << 61);
#pragma unroll
  for (int d = 0; d < L::D; ++d) bad |= (j[d] < 0 ? -j[d] : j[d]) >= (1LL << 58);  // |u| < 1/2
  // forces, 2^64 fixed point
  long long Fx[3] = {0, 0, 0};
  if (FS == FS_GUO) {
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      Fx[d] = to_fixed<64>(F[d], bad);
      const long long a = Fx[d] < 0 ? -Fx[d] : Fx[d];
      bad |= a >= (1LL << 62);
    }
  }
  if (__any_sync(0xffffffffu, bad)) return false;  // the warp takes the reference arithmetic

  // 1/rho in 2^62: float seed (2^-22), two Newton steps in fixed point
  long long R;
  {
    const float r = (float)(rhoF >> 37) * 0x1p-23f;  // rho to ~2^-22 (rhoF >> 37 < 2^24)
    const float y = __frcp_rn(r);
    R = (long long)__float2int_rn(y * 0x1p30f) << 32;  // y 2^62
#pragma unroll
    for (int it = 0; it < 2; ++it) {
      // e = (1 - rho R) 2^62 = (2^122 - rhoF R) >> 60
      const unsigned long long lo = (unsigned long long)rhoF * (unsigned long long)R;
      const long long hi = __mul64hi(rhoF, R);
      const long long hd = (1LL << 58) - hi - (lo != 0ULL ? 1 : 0);
      const unsigned long long ld = 0ULL - lo;
      const long long e = (long long)(((unsigned long long)hd << 4) | (ld >> 60));
      R += mulshr(R, e, 62);
    }
  }
  // u = j / rho in 2^64 fixed point: (j 2^60)(R 2^62) >> 58
  long long u[3] = {0, 0, 0};
  long long u2 = 0;
#pragma unroll
  for (int d = 0; d < L::D; ++d) {
    u[d] = mulshr(j[d], R, 58);
    u2 += mulhi(u[d], u[d]);
  }
  const bool fast = u2 < 184467440737095516LL;  // |u|^2 < 0.01
  if (!__all_sync(0xffffffffu, fast)) return false;
  const long long u4 = mulhi(u2, u2);
  // Guo: u.F (2^64)
  long long uF = 0;
  if (FS == FS_GUO) {
#pragma unroll
    for (int d = 0; d < L::D; ++d) uF += mulhi(u[d], Fx[d]);
  }
  const long long drho_w = drho;  // w_q delta rho via W64
  // omega multiplier
  const long long om = p.fx_omega_m;
  const int oa = p.fx_omega_a, os = p.fx_omega_sign;
  auto update = [&](int q, long long T, long long S) {
    const long long m = mulhi_rn(T, om);
    long long dq = (oa == 0 ? 0 : (oa == 1 ? T : 2 * T)) + (os > 0 ? m : -m);
    dq += S;
    const long long Fq = K::W60(q) + Dq[q] + dq;
    if (active) pop(next, p.V, q)[(uint32_t)idx] = to_double<60>(Fq);
  };
  // rest population: s = 0, R_0 = -1.5 u^2 + 1.125 u^4
  {
    const long long wr = mulhi(rhoF, K::W64(0));  // w_0 rho 2^60
    const long long R0 = ((-3 * u2) >> 1) + ((9 * u4) >> 3);
    const long long T1 = K::C(0) + mulhi_rn(drho_w, K::W64(0)) - Dq[0];
    const long long T2 = mulhi_rn(wr, R0);
    long long S = 0;
    if (FS == FS_GUO) S = (mulhi_rn(-uF, p.fx_guo62[0]) + 2) >> 2;
    update(0, T1 + T2, S);
  }
#pragma unroll
  for (int q = 1; q < Q; ++q) {
    if (!is_pair_leader<LAT>(q)) continue;
    const int qb = opposite<LAT>(q);
    long long s = 0, cj = 0, cF = 0;
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(q, d) > 0) { s += u[d]; cj += j[d]; cF += Fx[d]; }
      if (L::c(q, d) < 0) { s -= u[d]; cj -= j[d]; cF -= Fx[d]; }
    }
    const long long s2 = mulhi(s, s);
    const long long s2u2 = mulhi(s2, u2);
    const long long s4 = mulhi(s2, s2);
    // even part 4.5 s^2 - 1.5 u^2 + 1.125 u^4 - 6.75 s^2 u^2 + 3.375 s^4,
    // odd part (without the linear term) 4.5 s (s^2 - u^2)
    const long long E = ((9 * s2 - 3 * u2) >> 1) + ((9 * u4 - 54 * s2u2 + 27 * s4) >> 3);
    const long long O = (9 * mulhi(s, s2 - u2)) >> 1;
    const long long wr = mulhi(rhoF, K::W64(q));  // w_q rho 2^60
    const long long Tp2 = mulhi_rn(wr, E + O), Tm2 = mulhi_rn(wr, E - O);
    const long long lin = mulhi_rn(cj, K::W3_64(q));  // 3 w_q c_q.j 2^60
    const long long base = K::C(q) + mulhi_rn(drho_w, K::W64(q));
    const long long Tp1 = base - Dq[q] + lin, Tm1 = base - Dq[qb] - lin;
    long long Sp = 0, Sm = 0;
    if (FS == FS_GUO) {
      // ((c - u) + 3 (c.u) c).F = c.F - u.F + 3 s c.F (2^64); times guo_k (2^62) >> 66
      const long long e3 = 3 * mulhi(s, cF);
      Sp = (mulhi_rn(cF - uF + e3, p.fx_guo62[q]) + 2) >> 2;
      Sm = (mulhi_rn(-cF - uF + e3, p.fx_guo62[qb]) + 2) >> 2;
    }
    update(q, Tp1 + Tp2, Sp);
    update(qb, Tm1 + Tm2, Sm);
  }
  // stored fields and diagnostics (store / diagnostics steps only): FP64
  if (active && (p.store || p.diag)) {
    const double rho = to_double<60>(rhoF);
    double ud[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < L::D; ++d) ud[d] = to_double<64>(u[d]);
    double Fd[3] = {F[0], F[1], F[2]};
    store_node_fields<LAT>(p, idx, rho, ud, Fd, FS != FS_NONE, 2.0, energy, mach);
    mass = rho;
  }
  return true;
}

}  // namespace fx

template <int LAT, int FS>
__global__ void __launch_bounds__(256, 2) bgk_f64x_kernel(const double* __restrict__ prev,
                                                       double* __restrict__ next, StepParams p) {
  using L = Lattice<LAT>;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = idx < p.V;
  double mass = 0.0, energy = 0.0, mach = 0.0;
  uint32_t x = 0, y = 0, z = 0;
  double f[L::Q];
  double F[3] = {0.0, 0.0, 0.0};
  if (active) {
    node_coords(p, idx, x, y, z);
    const auto o = pull_offsets(p, x, y, z);
    pull<LAT>(prev, p.V, o, f);
    if (FS != FS_NONE) node_force<L::D>(p, x, y, z, F);
  } else {
#pragma unroll
    for (int q = 0; q < L::Q; ++q) f[q] = L::w(q);
  }
  const bool done = fx::bgk_node_fixed<LAT, FS>(f, F, p, idx, active, next, mass, energy, mach);
  if (!done && active) bgk_node_reference<LAT, FS>(prev, next, p, idx, x, y, z, mass, energy, mach);
  if (p.diag) block_reduce_diag(mass, energy, mach, 2.0, 2.0, p.diag_partials);
}

// ---- host-side launcher -------------------------------------------------------
template <int LAT, int FS>
static cudaError_t launch_f64x(const double* prev, double* next, const StepParams& p,
                               cudaStream_t s) {
  const unsigned grid = (unsigned)((p.V + 255) / 256);
  bgk_f64x_kernel<LAT, FS><<<grid, 256, 0, s>>>(prev, next, p);
  return cudaGetLastError();
}

#ifndef MLBM_LAT
#error "compile step_f64x.cu with -DMLBM_LAT=<0..3>"
#endif
#define MLBM_CAT2(a, b) a##b
#define MLBM_CAT(a, b) MLBM_CAT2(a, b)

// BGK with FP64 storage, fixed-point collision: forcing None, Guo or
// Shan-Chen (cudaErrorInvalidValue for EDM, which the caller runs with the
// reference-order kernel).
cudaError_t MLBM_CAT(step_f64x_L, MLBM_LAT)(int forcing, const double* prev, double* next,
                                              const StepParams& p, cudaStream_t s) {
  switch (forcing) {
    case FS_NONE: return launch_f64x<MLBM_LAT, FS_NONE>(prev, next, p, s);
    case FS_GUO: return launch_f64x<MLBM_LAT, FS_GUO>(prev, next, p, s);
    case FS_SHANCHEN: return launch_f64x<MLBM_LAT, FS_SHANCHEN>(prev, next, p, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace mlbm
