// Shared device-side definitions of the mlbm kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lattice.cuh"

namespace mlbm {

enum : int { FS_NONE = 0, FS_GUO = 1, FS_SHANCHEN = 2, FS_EDM = 3 };
// FORCE_FIELD: the per-node force read from force_field [D][V] (the spectral
// forces, Force.h:294-626, computed into that array before each step)
enum : int { FORCE_NONE = 0, FORCE_CONSTANT = 1, FORCE_SINUSOIDAL = 2, FORCE_KOLMOGOROV = 3,
             FORCE_FIELD = 7 };
enum : int { ALPHA_REFERENCE = 0, ALPHA_RESIDUAL = 1 };
enum : int { GUESS_PREVIOUS = 0, GUESS_TWO = 1, GUESS_LEARNED = 2, GUESS_LEARNED_EVERYWHERE = 3 };

enum : unsigned { ERR_NONFINITE = 1u, ERR_DENSITY = 2u };

// Unsigned division by a runtime constant with a multiply-high
// (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994): q = (umulhi(n, m) + n) >> s for n < 2^31.
struct FastDiv {
  uint32_t d, m, s;
  __host__ void init(uint32_t divisor) {
    d = divisor;
    s = 0;
    while ((1u << s) < divisor) ++s;
    const uint64_t one = 1;
    m = (uint32_t)(((one << 32) * ((one << s) - divisor)) / divisor + 1);
    if (divisor == 1) { m = 0; s = 0; }
  }
  __device__ __forceinline__ uint32_t div(uint32_t n) const {
    return (__umulhi(n, m) + n) >> s;
  }
};

// Per-step parameters, passed by value to every step kernel.
struct StepParams {
  long long V;               // nodes
  uint32_t lx, ly, lz;
  FastDiv div_lz, div_ly;    // node index -> (x, y, z)
  // relaxation
  double tau, beta;
  double bgk_a, bgk_b;       // (1 - 2 beta), 2 beta  (Collision.h:145-149)
  double guo_k[kMaxQ];       // ((1 - 1/(2 tau)) w_q) inv_cs2  (ForcingScheme.h:115-116)
  // force
  int force_type;
  int kol_axis, kol_comp;
  double amp[3];
  const double* force_table[3];  // per-axis host-computed sin profiles (device)
  const double* force_field;     // [D][V] per-node force of FORCE_FIELD (device)
  const float* force_field_f;    // its float copy (FP32/FP16 storage)
  // float copies for the low-precision kernels, which execute no FP64
  // instruction on their common path (a double->float conversion runs on
  // GB300's narrow FP64 pipe)
  const float* force_table_f[3];
  float amp_f[3];
  float bgk_b_f;             // 2 beta
  float guo_kt_f;            // (1 - 1/(2 tau)) 3; S_q = kt w_q [...]
  // FP64 BGK in fixed point (step_f64x.cu): omega = a + (omega - a) with
  // (omega - a) 2^62 as 31-bit halves (high, low), and
  // ((1 - 1/(2 tau)) w_q inv_cs2) 2^62 likewise; fx_ok = 0 when omega is
  // outside (0, 2) or a Guo factor is not below 1 (the kernel's ranges)
  int fx_ok;
  int fx_omega_a;
  int fx_omega_s31[2];
  int fx_1mw_s31[2];         // (1 - omega) 2^62 as 31-bit halves
  int fx_guo_s31[kMaxQ][2];
  // entropic solver
  int alpha_mode, guess_mode;
  double newton_tol;
  int newton_maxit;
  int bisect_maxit;          // cap of the bracketed solver (RESIDUAL mode)
  double deviation_threshold;
  float deviation_threshold_f;
  // optional outputs on this step
  int store;                 // write rho, u_hydro, alpha(, force) fields
  int diag;                  // fused diagnostics reduction
  double* rho_out;
  double* u_out;             // [D][V]
  double* force_out;         // [D][V]
  double* alpha_field;       // FP64 storage: per-node alpha (read guess, write result)
  float* alpha_field_f32;    // FP32/FP16 storage: per-node alpha - 2
  double* diag_partials;     // per block: mass, energy, max_mach, alpha_min, alpha_max
  unsigned long long* counters;  // solver counters (see CNT_*)
  unsigned* err_word;
  const void* mlp;           // device MlpDev* (learned guess)
  const void* log_table;     // device LogEntry[LOG_TABLE] (fastlog.cuh)
  const void* log_table_fine;  // device LogEntryFine[LOG_TABLE_FINE] + double[LNW_CONSTS] (fastlog.cuh)
  // entropic FP32/FP16 step: worklist of the nodes left to the second pass
  unsigned* defer_list;      // [V] node indices
  unsigned* defer_count;     // [2] list lengths, used by alternating steps
  int parity;                // step number & 1
  // learned guess: 1 when this step launches the kernels with the network;
  // cold_flags[parity] is set when the step stores a node without a solved
  // alpha (alpha exactly 2), cold_flags[parity ^ 1] cleared for the next step
  int learned_kernel;
  unsigned* cold_flags;
  int defer_blocks;          // grid of the second pass
  int defer_slot0;           // its first block's slot in diag_partials
};

enum : int {
  CNT_SOLVED = 0, CNT_ITER = 1, CNT_HITS = 2, CNT_BISECT = 3, CNT_FALLBACK = 4,
  CNT_LIMITED = 5, CNT_SHORTCUT = 6, CNT_SERIES = 7, CNT_INFER = 8, CNT_COUNT = 9
};
constexpr int DIAG_FIELDS = 5;

// Source node of the pulled population with velocity (cx, cy, cz): periodic
// neighbour offsets along each axis, formed once per node.
template <int R>
struct PullOffsetsR {
  // node-index offsets within one population array (V < 2^31): 32-bit, so a
  // source address is one 32-bit three-input add and one wide multiply-add
  // onto the population's base pointer. Index c + R holds the offset of the
  // node x - c (periodic) for a velocity component c in [-R, R].
  uint32_t ox[2 * R + 1];
  uint32_t oy[2 * R + 1];
  uint32_t oz[2 * R + 1];
  __device__ __forceinline__ uint32_t at(int cx, int cy, int cz) const {
    return ox[cx + R] + oy[cy + R] + oz[cz + R];
  }
};
using PullOffsets = PullOffsetsR<1>;

// Base of population q's array (uniform across the grid) indexed with a
// 32-bit node index.
template <class T>
__device__ __forceinline__ T* pop(T* base, long long V, int q) {
  return base + (long long)q * V;
}

__device__ __forceinline__ void node_coords(const StepParams& p, long long idx, uint32_t& x,
                                            uint32_t& y, uint32_t& z) {
  const uint32_t i = (uint32_t)idx;
  const uint32_t t = p.div_lz.div(i);
  z = i - t * p.lz;
  x = p.div_ly.div(t);
  y = t - x * p.ly;
}

__device__ __forceinline__ PullOffsets pull_offsets(const StepParams& p, uint32_t x, uint32_t y,
                                                    uint32_t z) {
  PullOffsets o;
  const uint32_t sx = p.ly * p.lz;
  const uint32_t xp = (x + 1 == p.lx) ? 0 : x + 1, xm = (x == 0) ? p.lx - 1 : x - 1;
  const uint32_t yp = (y + 1 == p.ly) ? 0 : y + 1, ym = (y == 0) ? p.ly - 1 : y - 1;
  const uint32_t zp = (z + 1 == p.lz) ? 0 : z + 1, zm = (z == 0) ? p.lz - 1 : z - 1;
  o.ox[0] = xp * sx; o.ox[1] = x * sx; o.ox[2] = xm * sx;
  o.oy[0] = yp * p.lz; o.oy[1] = y * p.lz; o.oy[2] = ym * p.lz;
  o.oz[0] = zp; o.oz[1] = z; o.oz[2] = zm;
  return o;
}

// Offsets for lattices that reach R > 1 nodes (D2Q13, D3Q33; the reference's
// halo of width R, Lattice.h:225-228, 719-722): (x - c) mod L by integer
// division, valid for any length >= 1. Those lattices run only in the FP64
// kernels, where the divisions are a small share of the node's work.
template <int R>
__device__ __forceinline__ PullOffsetsR<R> pull_offsets_r(const StepParams& p, uint32_t x,
                                                        uint32_t y, uint32_t z) {
  if constexpr (R == 1) {
    return pull_offsets(p, x, y, z);
  } else {
    PullOffsetsR<R> o;
    const uint32_t sx = p.ly * p.lz;
#pragma unroll
    for (int c = -R; c <= R; ++c) {
      o.ox[c + R] = ((x + R * p.lx - c) % p.lx) * sx;
      o.oy[c + R] = ((y + R * p.ly - c) % p.ly) * p.lz;
      o.oz[c + R] = (z + R * p.lz - c) % p.lz;
    }
    return o;
  }
}

// Per-node body force (Force.h:137-292). The sine profiles are tabulated on
// the host with the reference's expression amplitude * sin(i*2*pi/lambda)
// (Force.h:213, 266), so the device reads the very same doubles.
template <int D>
__device__ __forceinline__ void node_force(const StepParams& p, uint32_t x, uint32_t y,
                                           uint32_t z, double F[3]) {
  F[0] = 0.0; F[1] = 0.0; F[2] = 0.0;
  switch (p.force_type) {
    case FORCE_CONSTANT:
#pragma unroll
      for (int d = 0; d < D; ++d) F[d] = p.amp[d];
      break;
    case FORCE_SINUSOIDAL:
      F[0] = __ldg(p.force_table[0] + x);
      F[1] = __ldg(p.force_table[1] + y);
      if (D == 3) F[2] = __ldg(p.force_table[2] + z);
      break;
    case FORCE_KOLMOGOROV: {
      const uint32_t c = p.kol_axis == 0 ? x : (p.kol_axis == 1 ? y : z);
      const double v = __ldg(p.force_table[0] + c);
      F[0] = p.kol_comp == 0 ? v : 0.0;
      F[1] = p.kol_comp == 1 ? v : 0.0;
      F[2] = p.kol_comp == 2 ? v : 0.0;
      break;
    }
    case FORCE_FIELD: {  // Force<Generic>::setForce (Force.h:36-45)
      const uint32_t i = (x * p.ly + y) * p.lz + z;
#pragma unroll
      for (int d = 0; d < D; ++d) F[d] = __ldg(p.force_field + (long long)d * p.V + i);
      break;
    }
    default:
      break;
  }
}

// float -> double, exact, with integer operations: a conversion instruction
// between FP32 and FP64 executes on the FP64 path, which GB300 narrows to a
// small fraction of the FP32 rate. Valid for finite, normal, nonzero floats
// (populations); anything else takes the conversion instruction.
__device__ __forceinline__ double widen_exact(float v) {
  const uint32_t b = __float_as_uint(v);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)v;
  const uint32_t hi = (b & 0x80000000u) | (((b & 0x7fffffffu) >> 3) + (896u << 20));
  const uint32_t lo = b << 29;
  return __hiloint2double((int)hi, (int)lo);
}

// double -> float, round to nearest even, with integer operations (same
// reason); results outside the normal float range take the instruction.
__device__ __forceinline__ float narrow_rn(double x) {
  const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  if (e <= 896u || e >= 1151u) return (float)x;  // not a normal float after rounding
  uint32_t bits = ((((hi & 0x7fffffffu) - (896u << 20)) << 3) | (lo >> 29));
  const uint32_t rem = lo & 0x1fffffffu;
  bits += (rem > 0x10000000u || (rem == 0x10000000u && (bits & 1u))) ? 1u : 0u;
  return __uint_as_float(bits | (hi & 0x80000000u));
}

// v 2^-k for an integer v (|v| < 2^63, 0 < k <= 60): one rounding (the
// conversion), the scaling an exponent subtraction instead of an FP64 multiply.
__device__ __forceinline__ double ll_scaled(long long v, int k) {
  const double d = (double)v;
  return v == 0 ? 0.0 : __longlong_as_double(__double_as_longlong(d) - ((long long)k << 52));
}

// x / 2 for a positive normal or zero double, exactly, by an exponent step
// (values below 2^-1021 take the multiply).
__device__ __forceinline__ double half_exact(double x) {
  const long long b = __double_as_longlong(x);
  return ((b >> 52) & 0x7ff) > 1 ? __longlong_as_double(b - (1LL << 52)) : x * 0.5;
}

// Order-preserving integer key of a double, so that maxima and minima are
// integer operations (GB300 runs FP64 compares on its narrow FP64 path):
// non-negative values keep their bit pattern, negative ones are mirrored.
__device__ __forceinline__ long long dkey(double x) {
  const long long b = __double_as_longlong(x);
  return b >= 0 ? b : b ^ 0x7fffffffffffffffLL;
}
__device__ __forceinline__ double dkey_value(long long k) {
  return __longlong_as_double(k >= 0 ? k : k ^ 0x7fffffffffffffffLL);
}

// Block reduction of the diagnostics, written to partials[blockIdx.x]
// (blocks of at most 256 threads). Sums in a fixed order — each lane of warp
// 0 adds its column of the block's values in warp order, then a shuffle
// tree — so the result does not depend on scheduling; maxima and minima on
// integer keys.
__device__ __forceinline__ void block_reduce_diag(double mass, double energy, double mach,
                                                  double amin, double amax, double* partials) {
  __shared__ double sh_sum[2][256];
  __shared__ long long sh_key[3][8];
  long long kmach = dkey(mach), kmin = dkey(amin), kmax = dkey(amax);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    kmach = max(kmach, __shfl_down_sync(0xffffffffu, kmach, o));
    kmin = min(kmin, __shfl_down_sync(0xffffffffu, kmin, o));
    kmax = max(kmax, __shfl_down_sync(0xffffffffu, kmax, o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  sh_sum[0][threadIdx.x] = mass;
  sh_sum[1][threadIdx.x] = energy;
  if (lane == 0) {
    sh_key[0][warp] = kmach; sh_key[1][warp] = kmin; sh_key[2][warp] = kmax;
  }
  __syncthreads();
  if (warp == 0) {
    double m = 0.0, e = 0.0;
    for (int w = 0; w < nw; ++w) {
      m += sh_sum[0][w * 32 + lane];
      e += sh_sum[1][w * 32 + lane];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      m += __shfl_down_sync(0xffffffffu, m, o);
      e += __shfl_down_sync(0xffffffffu, e, o);
    }
    kmach = lane < nw ? sh_key[0][lane] : dkey(0.0);
    kmin = lane < nw ? sh_key[1][lane] : dkey(1e300);
    kmax = lane < nw ? sh_key[2][lane] : dkey(-1e300);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
      kmach = max(kmach, __shfl_down_sync(0xffffffffu, kmach, o));
      kmin = min(kmin, __shfl_down_sync(0xffffffffu, kmin, o));
      kmax = max(kmax, __shfl_down_sync(0xffffffffu, kmax, o));
    }
    if (lane == 0) {
      double* o = partials + (size_t)blockIdx.x * DIAG_FIELDS;
      o[0] = m; o[1] = e; o[2] = dkey_value(kmach); o[3] = dkey_value(kmin); o[4] = dkey_value(kmax);
    }
  }
}

// Warp-aggregated add of the solver counters.
__device__ __forceinline__ void add_counters(unsigned long long* counters, const unsigned c[CNT_COUNT]) {
#pragma unroll
  for (int k = 0; k < CNT_COUNT; ++k) {
    unsigned v = c[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(counters + k, (unsigned long long)v);
  }
}

}  // namespace mlbm
