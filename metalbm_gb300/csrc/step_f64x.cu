// FP64-storage BGK step with the collision on the integer pipe.
//
// GB300 executes FP64 arithmetic at 1/73 of the FP32 rate, so the
// reference-order kernel (step_f64.cu, ~740 separately rounded FP64
// operations a node) is bound by that pipe at a few percent of HBM. This
// kernel keeps the FP64 populations in HBM and computes the same update,
//   f'_q = f_q + omega (f_eq_q - f_q) + S_q   (Collision.h:134-151, omega = 2 beta),
// in 64-bit fixed point:
//   * F_q = f_q 2^60 from the double's bits (exact for f_q >= 2^-8, rounded
//     below);
//   * rho and j = sum_q c_q f_q as exact integer sums (Moment.h:13-47);
//   * 1/rho by two Newton steps in 2^61 fixed point from an FP32 seed,
//     u = j / rho in 2^62 fixed point;
//   * f_eq_q - f_q = w_q rho (1 + 3 s + R_q) - f_q with s = c_q.u and
//     R_q = 4.5 s^2 - 1.5 u^2 + 4.5 s^3 - 4.5 s u^2 + 1.125 u^4 - 6.75 s^2 u^2
//     + 3.375 s^4, Equilibrium<TruncationMa3> (Equilibrium.h:17-33), in 2^62
//     fixed point, w_q rho from the reference's double weights exactly, the
//     pair (q, -q) sharing the even and odd parts of 3 s + R_q;
//   * Guo's source ((1 - 1/(2 tau)) w_q 3) [(c_q - u).F + 3 (c_q.u)(c_q.F)]
//     (ForcingScheme.h:81-118);
//   * f'_q 2^62 = (1 - omega) 4 F_q + Omega_q (1 + E_q +- O_q) + S_q for the
//     moving populations (Omega_q = omega w_q rho, once per weight), and
//     4 F_0 + a T_0 + (omega - a) T_0 + S_0 for the rest population (T_0 =
//     f_eq_0 - f_0, a the integer nearest omega), rounded once to FP64, to
//     nearest even (the one FP64-pipe instruction a population).
// Every product is of two values below 2^62 in magnitude held as 31-bit
// halves, (a_h 2^31 + a_l)(b_h 2^31 + b_l) 2^-62 = a_h b_h + (a_h b_l + a_l b_h)
// 2^-31 with the product of the low halves dropped: three 32 x 32 -> 64-bit
// integer multiply-adds, within one unit of 2^-62 of the exact product (GB300
// emulates a 64 x 64-bit high product in several times as many
// instructions). A population's update is then within a few units of 2^-62 of
// the exact value of the reference's formula, about one FP64 ulp of the
// smallest populations (the tests hold the state to 1e-12 relative over
// hundreds of steps).
//
// Nodes outside the fixed-point ranges (a population outside [0, 1/2) for
// Q > 15, [0, 1) for D2Q9 and D3Q15, so that the unsigned sum of the F_q stays
// below 2^64; rho outside (0.53, 2); |j| >= 1/4; |u| >= 0.1; |F_d| >= 1/8; a new
// population outside [2^-30, 1); or a non-finite value) take the reference-order arithmetic of ref_node.cuh: a
// warp with such a node computes all its nodes that way (bit-identical to the
// reference for them), rewriting whatever the fixed-point pass stored.
// Lattices D2Q9, D3Q19, D3Q27, D3Q15 (reach 1, inv_cs2 = 3); forcing None,
// Guo, Shan-Chen (EDM uses the reference-order kernel).
//
// This unit is compiled with -fmad=false for the reference-order fallback.

#include "common.cuh"
#include "kernels.h"
#include "ref_node.cuh"

namespace mlbm {
namespace fx {

// ---- 64-bit fixed-point helpers ---------------------------------------------

// x = h 2^31 + l with 0 <= l < 2^31, for |x| < 2^62
struct S31 {
  int h, l;
};
__device__ __forceinline__ S31 split(long long x) {
  return S31{(int)(x >> 31), (int)((unsigned)x & 0x7fffffffu)};
}
__host__ __device__ constexpr S31 csplit(long long x) {
  return S31{(int)(x >> 31), (int)(x & 0x7fffffffLL)};
}

// a b 2^-62 within one unit (|error| < 1): the low halves' product dropped,
// the middle terms' sum rounded
__device__ __forceinline__ long long mul62(S31 a, S31 b) {
  const long long mid = (long long)a.h * b.l + ((long long)a.l * b.h + (1LL << 30));
  return (long long)a.h * b.h + (mid >> 31);
}
// a b 2^-60 within one unit
__device__ __forceinline__ long long mul60(S31 a, S31 b) {
  const long long mid = (long long)a.h * b.l + ((long long)a.l * b.h + (1LL << 28));
  return ((long long)a.h * b.h << 2) + (mid >> 29);
}

// x >> s for any s (PTX clamps shift amounts above 64: 0)
__device__ __forceinline__ unsigned long long shr_u64(unsigned long long x, unsigned s) {
  unsigned long long r;
  asm("shr.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(s));
  return r;
}

// |v| 2^S rounded to nearest (ties away) from the double's bits b, for
// |v| 2^S < 2^62 (the caller checks the exponent range); zero and
// subnormals give 0.
template <int S>
__device__ __forceinline__ unsigned long long abs_to_fixed(unsigned long long b) {
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  const unsigned long long t = (b << 11) | 0x8000000000000000ULL;  // 1.m 2^63
  // |v| 2^S = t 2^(e - 1086 + S)
  return (shr_u64(t, 1085u - S - e) + 1ULL) >> 1;
}

// X 2^-62 rounded to the nearest double (ties to even) for X in [2^32, 2^62);
// `bad` otherwise. The integer-to-double conversion runs on the FP64 pipe
// (2 a clock per SM on GB300, idle in this kernel; measured 4 % faster than
// rounding with integer instructions), the scaling by 2^-62 is an exponent
// subtraction.
__device__ __forceinline__ double fixed62_to_double(long long X, bool& bad) {
  const unsigned hi = (unsigned)((unsigned long long)X >> 32);
  bad |= hi - 1u >= 0x3fffffffu;
  return __longlong_as_double(__double_as_longlong(__ll2double_rn(X)) - (62LL << 52));
}

// v 2^-S rounded to the nearest double (ties to even), any |v| < 2^63 (the
// stored fields and diagnostics).
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
  // w_q 2^63 (exact: the double weight times a power of two is an integer;
  // < 2^62 for w_q < 1/2)
  static constexpr long long W63(int q) { return (long long)(L::w(q) * 9223372036854775808.0); }
  // populations below 2^-1 (Q > 15) or 2^0: the high word's bound, and the
  // new populations' bound in 2^62 fixed point
  static constexpr unsigned kFmaxHi = L::Q > 15 ? 0x3fe00000u : 0x3ff00000u;
};

// The reference's BGK coefficients in fixed point: omega T = a T + mul62(T,
// omega - a) (StepParams fx_omega_a, fx_omega_s31), and Guo's
// ((1 - 1/(2 tau)) w_q inv_cs2) 2^62 (fx_guo_s31), split on the host.

// One node in fixed point. Returns false, for every lane of the warp, when a
// lane of the warp is outside the fixed-point ranges; every lane of the warp
// must call it (inactive lanes with f = w). On false the caller recomputes the
// warp's nodes in the reference order (populations this pass stored are
// rewritten).
template <int LAT, int FS>
__device__ __forceinline__ bool bgk_node_fixed(const double f[], const double F[3],
                                               const StepParams& p, long long idx, bool active,
                                               double* __restrict__ next, double& mass,
                                               double& energy, double& mach) {
  bool bad = false;
  using L = Lattice<LAT>;
  using K = FxConst<LAT>;
  constexpr int Q = L::Q;
  // populations in 2^60 fixed point, their exact sums
  unsigned long long Fq[Q];
  unsigned long long rhoF = 0;
  long long j[3] = {0, 0, 0};
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(f[q]);
    bad |= (unsigned)(b >> 32) >= K::kFmaxHi;  // negative, too large, inf, NaN
    Fq[q] = abs_to_fixed<60>(b);
    rhoF += Fq[q];
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(q, d) > 0) j[d] += (long long)Fq[q];
      if (L::c(q, d) < 0) j[d] -= (long long)Fq[q];
    }
  }
  constexpr unsigned long long kRhoLo = (1ULL << 59) + (1ULL << 55);  // rho > 0.53
  bad |= rhoF - kRhoLo >= (1ULL << 61) - kRhoLo;                      // rho < 2
#pragma unroll
  for (int d = 0; d < L::D; ++d)
    bad |= (unsigned long long)(j[d] + (1LL << 58)) >= (1ULL << 59);  // |j| < 1/4
  // forces, 2^62 fixed point
  long long Fx[3] = {0, 0, 0};
  if (FS == FS_GUO) {
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(F[d]);
      bad |= ((unsigned)(b >> 32) & 0x7fffffffu) >= 0x3fc00000u;  // |F| < 1/8, finite
      const long long a = (long long)abs_to_fixed<62>(b);
      Fx[d] = (long long)b < 0 ? -a : a;
    }
  }
  if (__any_sync(0xffffffffu, bad)) return false;  // the warp takes the reference arithmetic

  // 1/rho in 2^61: FP32 seed (~2^-21), two Newton steps
  const S31 rho61 = split((long long)(rhoF << 1));
  long long R;
  {
    const unsigned x = (unsigned)(rhoF >> 38);  // rho 2^22, < 2^23
    const float rf = __uint_as_float(0x4b000000u | x) - 8388608.0f;
    const float y = __frcp_rn(rf);              // 2^-22 / rho
    R = (long long)__float2uint_rn(y * 0x1p53f) << 30;
#pragma unroll
    for (int it = 0; it < 2; ++it) {
      const S31 Rs = split(R);
      const long long e = (1LL << 62) - mul60(rho61, Rs);  // (1 - rho R) 2^62
      R += mul62(Rs, split(e));
    }
  }
  // u = j / rho in 2^62 fixed point
  const S31 Rs = split(R);
  long long u[3] = {0, 0, 0};
  S31 us[3];
  long long u2 = 0;
#pragma unroll
  for (int d = 0; d < L::D; ++d) {
    u[d] = mul62(split(j[d] << 3), Rs);
    us[d] = split(u[d]);
    u2 += mul62(us[d], us[d]);
  }
  const bool fast = u2 < 46116860184273879LL;  // |u|^2 < 0.01
  if (!__all_sync(0xffffffffu, fast)) return false;
  const S31 u2s = split(u2);
  const long long u4 = mul62(u2s, u2s);
  // the node's part of R_q: -1.5 u^2 + 1.125 u^4
  const long long P0 = ((-3 * u2) >> 1) + ((9 * u4) >> 3);
  // Guo: u.F (2^62)
  long long uF = 0;
  if (FS == FS_GUO) {
#pragma unroll
    for (int d = 0; d < L::D; ++d) uF += mul62(us[d], split(Fx[d]));
  }
  const int oa = p.fx_omega_a;
  const S31 om = S31{p.fx_omega_s31[0], p.fx_omega_s31[1]};
  const S31 c1mw = S31{p.fx_1mw_s31[0], p.fx_1mw_s31[1]};
  bool out_bad = false;
  auto store = [&](int q, long long X) {
    const double r = fixed62_to_double(X, out_bad);
    if (active) pop(next, p.V, q)[(uint32_t)idx] = r;
  };
  // new population q from T = (f_eq_q - f_q) 2^62 and the source S (2^62):
  // (f + omega T + S) 2^62, summed modulo 2^64 (a value outside (-2, 2) wraps
  // to one that fails the range check)
  auto update = [&](int q, long long T, long long S) {
    store(q, (long long)((Fq[q] << 2) + (unsigned long long)(oa * T) +
                         (unsigned long long)mul62(split(T), om) + (unsigned long long)S));
  };
  // the moving populations as (1 - omega) f + omega w rho (1 + E +- O) + S,
  // Omega = omega w rho per weight (< 1/2 for the moving weights, rho < 2):
  // two products a population instead of three
  auto update_moving = [&](int q, S31 Omega_s, long long Omega, long long EO, long long S) {
    store(q, (long long)((unsigned long long)mul62(split((long long)(Fq[q] << 2)), c1mw) +
                         (unsigned long long)Omega + (unsigned long long)mul62(Omega_s, split(EO)) +
                         (unsigned long long)S));
  };
  // rest population: s = 0, R_0 = -1.5 u^2 + 1.125 u^4
  {
    const long long wr = mul62(rho61, csplit(K::W63(0)));  // w_0 rho 2^62
    const long long T = wr - (long long)(Fq[0] << 2) + mul62(split(wr), split(P0));
    long long S = 0;
    if (FS == FS_GUO) S = mul62(split(-uF), S31{p.fx_guo_s31[0][0], p.fx_guo_s31[0][1]});
    update(0, T, S);
  }
#pragma unroll
  for (int q = 1; q < Q; ++q) {
    if (!is_pair_leader<LAT>(q)) continue;
    const int qb = opposite<LAT>(q);
    long long s = 0, cF = 0;
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      if (L::c(q, d) > 0) { s += u[d]; cF += Fx[d]; }
      if (L::c(q, d) < 0) { s -= u[d]; cF -= Fx[d]; }
    }
    const S31 ss = split(s);
    const long long s2 = mul62(ss, ss);
    const S31 s2s = split(s2);
    // even part 4.5 s^2 + P0 + s^2 (3.375 s^2 - 6.75 u^2), odd part
    // 3 s + 4.5 s (s^2 - u^2)
    const long long E = ((9 * s2) >> 1) + P0 + mul62(s2s, split((27 * s2 - 54 * u2) >> 3));
    const long long O = 3 * s + ((9 * mul62(ss, split(s2 - u2))) >> 1);
    const long long wrv = mul62(rho61, csplit(K::W63(q)));  // w_q rho 2^62 (w_q = w_-q)
    const long long Omega = oa * wrv + mul62(split(wrv), om);  // omega w_q rho 2^62
    const S31 Omega_s = split(Omega);
    long long Sp = 0, Sm = 0;
    if (FS == FS_GUO) {
      // ((c - u) + 3 (c.u) c).F = c.F - u.F + 3 s c.F
      const long long e3 = 3 * mul62(ss, split(cF));
      Sp = mul62(split(cF - uF + e3), S31{p.fx_guo_s31[q][0], p.fx_guo_s31[q][1]});
      Sm = mul62(split(-cF - uF + e3), S31{p.fx_guo_s31[qb][0], p.fx_guo_s31[qb][1]});
    }
    update_moving(q, Omega_s, Omega, E + O, Sp);
    update_moving(qb, Omega_s, Omega, E - O, Sm);
  }
  if (__any_sync(0xffffffffu, out_bad)) return false;
  // stored fields and diagnostics (store / diagnostics steps only): FP64
  if (active && (p.store || p.diag)) {
    const double rho = to_double<60>((long long)rhoF);
    double ud[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < L::D; ++d) ud[d] = to_double<62>(u[d]);
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
