// Per-node arithmetic of the FP64 kernels in the reference's operation order
// (shared by step_f64.cu and step_f64x.cu; both are compiled with
// -fmad=false so every multiply and add below is a separately rounded IEEE
// operation, left to right as in the cited C++ expressions, and BGK results
// are bit-identical to the reference CPU build). Rearrangements used here are
// exact: products by +-1 are sign changes, additions of the zero products of
// c_d = 0 are dropped (x + 0 = x), and the odd/even powers of c.u are shared
// between the populations q and -q (c.u changes sign exactly).
#pragma once

#include "common.cuh"

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
// One node of the reference-order BGK step: pull, moments, force,
// equilibrium, collide and stream, optional stored fields and diagnostics.
template <int LAT, int FS>
__device__ __forceinline__ void bgk_node_reference(const double* __restrict__ prev,
                                                   double* __restrict__ next, const StepParams& p,
                                                   long long idx, uint32_t x, uint32_t y,
                                                   uint32_t z, double& mass, double& energy,
                                                   double& mach) {
  using L = Lattice<LAT>;
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

}  // namespace mlbm
