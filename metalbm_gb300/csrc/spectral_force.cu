// Spectral forces (Force.h:294-626): ConstantShell, EnergyRemoval and
// Turbulent2D as a per-node force field [D][V] that the step kernels read
// (FORCE_FIELD in node_force / node_force_float).
//
// The reference computes them with FFTW r2c/c2r transforms on the host
// (Transformer.h:19-110). Here:
//   * ConstantShell (and Turbulent2D's injection part): the spectrum A on the
//     shell kmin^2 <= |k|^2 <= kmax^2 (integer wavenumbers, Force.h:339-347,
//     386), made solenoidal by the curl i k x T (3-D, Transformer.h:207-272)
//     or (i k_y psi, -i k_x psi) (2-D, Transformer.h:298-387), divided by the
//     node count (the backward transform's normalisation,
//     Transformer.h:98-108): one batched cuFFT Z2D at creation.
//   * EnergyRemoval (and Turbulent2D's removal part): -A_d times the momentum
//     rho u of the last stored fields filtered to the shell (Force.h:442-532).
//     Shells up to k = 5 use the separable partial transforms below (sums
//     along the contiguous axis, then the two others, the filter, and back;
//     FP32 per-node stages for FP32/FP16 storage); larger shells use batched
//     cuFFT D2Z, one filter pass and Z2D.
// Every spectrum stays Hermitian: the reference's partner writes on the
// k_y = k_z = 0 row of 3-D lattices, which index y = L_y and land one row off
// (or past the array), are not reproduced. Shells stay below the Nyquist
// wavenumber (checked by the caller).

#include <cufft.h>

#include <cmath>
#include <cstdio>
#include <new>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "mlbm/mlbm.h"

namespace mlbm {

// Half-spectrum geometry: extents of the r2c output, last axis halved.
struct SpecGrid {
  int D;
  int lx, ly, lz;   // real extents (lz = 1 in 2-D)
  int hx, hy, hz;   // complex extents: (lx, ly, lz/2+1) or (lx, ly/2+1, 1)
  long long nspec;  // hx * hy * hz
};

__device__ __forceinline__ void mode_wavenumbers(const SpecGrid& g, long long m, int k[3]) {
  const int iz = (int)(m % g.hz);
  const long long t = m / g.hz;
  const int iy = (int)(t % g.hy);
  const int ix = (int)(t / g.hy);
  k[0] = ix <= g.lx / 2 ? ix : ix - g.lx;
  if (g.D == 2) {
    k[1] = iy;  // halved axis: 0 .. ly/2
    k[2] = 0;
  } else {
    k[1] = iy <= g.ly / 2 ? iy : iy - g.ly;
    k[2] = iz;  // halved axis: 0 .. lz/2
  }
}

__device__ __forceinline__ bool in_shell(const int k[3], int kmin, int kmax) {
  const long long k2 = (long long)k[0] * k[0] + (long long)k[1] * k[1] + (long long)k[2] * k[2];
  return k2 >= (long long)kmin * kmin && k2 <= (long long)kmax * kmax;
}

// ConstantShell spectrum after MakeIncompressible, times `scale` (1/V).
__global__ void shell_injection_kernel(SpecGrid g, double ax, double ay, double az, int kmin,
                                       int kmax, double scale, cufftDoubleComplex* out) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= g.nspec) return;
  int k[3];
  mode_wavenumbers(g, m, k);
  const bool s = in_shell(k, kmin, kmax);
  if (g.D == 2) {
    const double psi = s ? ax * scale : 0.0;
    out[m] = make_cuDoubleComplex(0.0, (double)k[1] * psi);
    out[g.nspec + m] = make_cuDoubleComplex(0.0, -(double)k[0] * psi);
  } else {
    const double tx = s ? ax * scale : 0.0, ty = s ? ay * scale : 0.0, tz = s ? az * scale : 0.0;
    const double kx = k[0], ky = k[1], kz = k[2];
    out[m] = make_cuDoubleComplex(0.0, ky * tz - kz * ty);
    out[g.nspec + m] = make_cuDoubleComplex(0.0, kz * tx - kx * tz);
    out[2 * g.nspec + m] = make_cuDoubleComplex(0.0, kx * ty - ky * tx);
  }
}

// momentum [D][V] = rho * u_d of the stored fields (Force.h:451-460)
__global__ void momentum_kernel(const double* __restrict__ rho, const double* __restrict__ u,
                                double* __restrict__ mom, int D, long long V) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V) return;
  const double r = rho[i];
  for (int d = 0; d < D; ++d) mom[(long long)d * V + i] = r * u[(long long)d * V + i];
}

// spec_d <- (shell ? -A_d spec_d : 0) * scale (+ injection_d)
__global__ void removal_filter_kernel(SpecGrid g, cufftDoubleComplex* __restrict__ spec,
                                      const cufftDoubleComplex* __restrict__ inject, double rx,
                                      double ry, double rz, int kmin, int kmax, double scale) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= g.nspec) return;
  int k[3];
  mode_wavenumbers(g, m, k);
  const bool s = in_shell(k, kmin, kmax);
  const double a[3] = {rx, ry, rz};
  for (int d = 0; d < g.D; ++d) {
    const long long j = (long long)d * g.nspec + m;
    const double c = s ? -a[d] * scale : 0.0;
    cufftDoubleComplex v = spec[j];
    v = make_cuDoubleComplex(c * v.x, c * v.y);
    if (inject) v = make_cuDoubleComplex(v.x + inject[j].x, v.y + inject[j].y);
    spec[j] = v;
  }
}

// ---- Removal on a small shell: separable partial transforms ----------------
// The removal shell is a handful of modes (|k| <= K, K <= kSparseMaxK), so
// instead of two full FP64 FFTs of D components (FP64-bound on GB300) the
// momentum spectrum is formed only on the box [-KA, KA] x [-K, K] x [0, K]:
// sums along the contiguous axis first (one warp per line), then along the
// two others; the filtered modes go back the same way. The lattice is seen as
// A x B x C with the halved axis C last: 3-D (lx, ly, lz), 2-D (1, lx, ly)
// with KA = 0. Per node: D (K + 1) complex multiply-adds each way.
constexpr int kSparseMaxK = 5;

struct SepGrid {
  int A, B, C, D, K, KA;
  long long V;
  const double2* twA;  // (cos, sin)(2 pi j / n), j < n
  const double2* twB;
  const double2* twC;
  const float2* twCf;  // float copy of twC (FP32/FP16-storage updates)
};

// e^{+2 pi i k j / n}
__device__ __forceinline__ double2 twiddle(const double2* t, int k, int j, int n) {
  const long long km = ((long long)k % n + n) % n;
  return __ldg(t + (km * j) % n);
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmul_conj(double2 a, double2 b) {  // a * conj(b)
  return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// P1[line][kc][d] = sum_c rho u_d e^{-2 pi i kc c / C}, one warp per line
template <int K>
__global__ void __launch_bounds__(256) sep_forward_c(SepGrid g, const double* __restrict__ rho,
                                                     const double* __restrict__ u,
                                                     double2* __restrict__ P1) {
  const int lane = threadIdx.x & 31;
  const long long line = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (line >= (long long)g.A * g.B) return;  // uniform across the warp
  double ar[3][K + 1], ai[3][K + 1];
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int k = 0; k <= K; ++k) ar[d][k] = ai[d][k] = 0.0;
  // running twiddle indices (k c) mod C, advanced by (32 k) mod C per stride
  int idx[K + 1], step[K + 1];
#pragma unroll
  for (int k = 0; k <= K; ++k) {
    idx[k] = (k * lane) % g.C;
    step[k] = (32 * k) % g.C;
  }
  for (int c = lane; c < g.C; c += 32) {
    const long long i = line * g.C + c;
    const double r = rho[i];
    double m[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) m[d] = d < g.D ? r * u[(long long)d * g.V + i] : 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) ar[d][0] += m[d];  // k = 0: twiddle 1
#pragma unroll
    for (int k = 1; k <= K; ++k) {
      const double2 w = __ldg(g.twC + idx[k]);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        ar[d][k] += m[d] * w.x;
        ai[d][k] -= m[d] * w.y;
      }
    }
#pragma unroll
    for (int k = 1; k <= K; ++k) {
      idx[k] += step[k];
      if (idx[k] >= g.C) idx[k] -= g.C;
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int k = 0; k <= K; ++k)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ar[d][k] += __shfl_down_sync(0xffffffffu, ar[d][k], o);
        ai[d][k] += __shfl_down_sync(0xffffffffu, ai[d][k], o);
      }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k <= K; ++k)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        if (d < g.D) P1[(line * (K + 1) + k) * g.D + d] = make_double2(ar[d][k], ai[d][k]);
  }
}

// P2[a][kb][kc][d] = sum_b P1[a][b][kc][d] e^{-2 pi i kb b / B}; one warp per
// output, the lanes splitting the sum (fixed reduction order)
__device__ __forceinline__ double2 warp_sum2(double2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  return v;
}

__global__ void sep_forward_b(SepGrid g, const double2* __restrict__ P1, double2* __restrict__ P2) {
  const int nk = 2 * g.K + 1, nc = g.K + 1;
  const int lane = threadIdx.x & 31;
  const long long t = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (t >= (long long)g.A * nk * nc * g.D) return;  // uniform across the warp
  const int d = (int)(t % g.D);
  const int kc = (int)((t / g.D) % nc);
  const int kbi = (int)((t / ((long long)g.D * nc)) % nk);
  const long long a = t / ((long long)g.D * nc * nk);
  const int kbm = ((kbi - g.K) % g.B + g.B) % g.B;
  double2 acc = make_double2(0.0, 0.0);
  for (int b = lane; b < g.B; b += 32) {
    const double2 v = P1[((a * g.B + b) * nc + kc) * g.D + d];
    const int e = (int)(((long long)kbm * b) % g.B);
    const double2 p = cmul_conj(v, __ldg(g.twB + e));
    acc.x += p.x;
    acc.y += p.y;
  }
  acc = warp_sum2(acc);
  if (lane == 0) P2[t] = acc;
}

// modes of the box: sum over a (one warp per mode), then the removal filter
// -A_d/V on the shell (0 elsewhere), doubled for kc > 0 (each stands for k and -k)
__global__ void sep_modes(SepGrid g, const double2* __restrict__ P2, double2* __restrict__ Ch,
                          double rx, double ry, double rz, int kmin, int kmax, double inv_v) {
  const int nk = 2 * g.K + 1, nc = g.K + 1, na = 2 * g.KA + 1;
  const int lane = threadIdx.x & 31;
  const long long t = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (t >= (long long)na * nk * nc * g.D) return;  // uniform across the warp
  const int d = (int)(t % g.D);
  const int kc = (int)((t / g.D) % nc);
  const int kbi = (int)((t / ((long long)g.D * nc)) % nk);
  const int kai = (int)(t / ((long long)g.D * nc * nk));
  const int ka = kai - g.KA, kb = kbi - g.K;
  const int kam = (ka % g.A + g.A) % g.A;
  double2 acc = make_double2(0.0, 0.0);
  for (int a = lane; a < g.A; a += 32) {
    const double2 v = P2[(((long long)a * nk + kbi) * nc + kc) * g.D + d];
    const int e = (int)(((long long)kam * a) % g.A);
    const double2 p = cmul_conj(v, __ldg(g.twA + e));
    acc.x += p.x;
    acc.y += p.y;
  }
  acc = warp_sum2(acc);
  if (lane != 0) return;
  const long long k2 = (long long)ka * ka + (long long)kb * kb + (long long)kc * kc;
  const bool s = k2 >= (long long)kmin * kmin && k2 <= (long long)kmax * kmax;
  const double amp = d == 0 ? rx : (d == 1 ? ry : rz);
  const double c = s ? -amp * inv_v * (kc > 0 ? 2.0 : 1.0) : 0.0;
  Ch[t] = make_double2(c * acc.x, c * acc.y);
}

// R1[a][kb][kc][d] = sum_ka Ch[ka][kb][kc][d] e^{+2 pi i ka a / A}
__global__ void sep_inverse_a(SepGrid g, const double2* __restrict__ Ch, double2* __restrict__ R1) {
  const int nk = 2 * g.K + 1, nc = g.K + 1, na = 2 * g.KA + 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)g.A * nk * nc * g.D) return;
  const long long inner = t % ((long long)nk * nc * g.D);  // (kb, kc, d)
  const int a = (int)(t / ((long long)nk * nc * g.D));
  double2 acc = make_double2(0.0, 0.0);
  for (int kai = 0; kai < na; ++kai) {
    const double2 p = cmul(Ch[(long long)kai * nk * nc * g.D + inner], twiddle(g.twA, kai - g.KA, a, g.A));
    acc.x += p.x;
    acc.y += p.y;
  }
  R1[t] = acc;
}

// R2[a][b][kc][d] = sum_kb R1[a][kb][kc][d] e^{+2 pi i kb b / B}
__global__ void sep_inverse_b(SepGrid g, const double2* __restrict__ R1, double2* __restrict__ R2,
                              float2* __restrict__ R2f) {
  const int nk = 2 * g.K + 1, nc = g.K + 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)g.A * g.B * nc * g.D) return;
  const int d = (int)(t % g.D);
  const int kc = (int)((t / g.D) % nc);
  const long long ab = t / ((long long)g.D * nc);
  const int b = (int)(ab % g.B);
  const long long a = ab / g.B;
  double2 acc = make_double2(0.0, 0.0);
  for (int kbi = 0; kbi < nk; ++kbi) {
    const double2 p = cmul(R1[((a * nk + kbi) * nc + kc) * g.D + d], twiddle(g.twB, kbi - g.K, b, g.B));
    acc.x += p.x;
    acc.y += p.y;
  }
  if (R2f)
    R2f[t] = make_float2(narrow_rn(acc.x), narrow_rn(acc.y));
  else
    R2[t] = acc;
}

// field_d = injection_d + Re sum_kc R2[line][kc][d] e^{+2 pi i kc c / C}
template <int K>
__global__ void __launch_bounds__(256) sep_synthesis(SepGrid g, const double2* __restrict__ R2,
                                                     const double* __restrict__ inj,
                                                     double* __restrict__ field) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.V) return;
  const long long line = i / g.C;
  const int c = (int)(i - line * g.C);
  double2 w[K + 1];
  int e = 0;  // (k c) mod C, by repeated addition of c < C
#pragma unroll
  for (int k = 1; k <= K; ++k) {
    e += c;
    if (e >= g.C) e -= g.C;
    w[k] = __ldg(g.twC + e);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (d >= g.D) break;
    double f = inj ? inj[(long long)d * g.V + i] : 0.0;
    f += __ldg(R2 + (line * (K + 1)) * g.D + d).x;  // k = 0: twiddle 1
#pragma unroll
    for (int k = 1; k <= K; ++k) {
      const double2 z = __ldg(R2 + (line * (K + 1) + k) * g.D + d);
      f += z.x * w[k].x - z.y * w[k].y;
    }
    field[(long long)d * g.V + i] = f;
  }
}

// FP32 variants of the two per-node stages, for FP32/FP16 storage: the
// kernels read a float field, so the sums need FP32 accuracy only (about
// 1e-6 relative on a force that is itself ~1e-8 of the populations), and FP32
// runs at ~73x the FP64 rate. The FP64 field kept for stored fields is the
// exact widening of the float one; the middle stages (a few thousand modes)
// stay FP64.
template <int K>
__global__ void __launch_bounds__(256) sep_forward_c_f(SepGrid g, const double* __restrict__ rho,
                                                       const double* __restrict__ u,
                                                       double2* __restrict__ P1) {
  const int lane = threadIdx.x & 31;
  const long long line = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (line >= (long long)g.A * g.B) return;  // uniform across the warp
  float ar[3][K + 1], ai[3][K + 1];
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int k = 0; k <= K; ++k) ar[d][k] = ai[d][k] = 0.0f;
  int idx[K + 1], step[K + 1];
#pragma unroll
  for (int k = 0; k <= K; ++k) {
    idx[k] = (k * lane) % g.C;
    step[k] = (32 * k) % g.C;
  }
  for (int c = lane; c < g.C; c += 32) {
    const long long i = line * g.C + c;
    const float r = narrow_rn(rho[i]);
    float m[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) m[d] = d < g.D ? r * narrow_rn(u[(long long)d * g.V + i]) : 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) ar[d][0] += m[d];
#pragma unroll
    for (int k = 1; k <= K; ++k) {
      const float2 w = __ldg(g.twCf + idx[k]);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        ar[d][k] = fmaf(m[d], w.x, ar[d][k]);
        ai[d][k] = fmaf(-m[d], w.y, ai[d][k]);
      }
    }
#pragma unroll
    for (int k = 1; k <= K; ++k) {
      idx[k] += step[k];
      if (idx[k] >= g.C) idx[k] -= g.C;
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int k = 0; k <= K; ++k)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ar[d][k] += __shfl_down_sync(0xffffffffu, ar[d][k], o);
        ai[d][k] += __shfl_down_sync(0xffffffffu, ai[d][k], o);
      }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k <= K; ++k)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        if (d < g.D)
          P1[(line * (K + 1) + k) * g.D + d] = make_double2(widen_exact(ar[d][k]), widen_exact(ai[d][k]));
  }
}

template <int K>
__global__ void __launch_bounds__(256) sep_synthesis_f(SepGrid g, const float2* __restrict__ R2f,
                                                       const float* __restrict__ inj,
                                                       float* __restrict__ field_f,
                                                       double* __restrict__ field) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.V) return;
  const long long line = i / g.C;
  const int c = (int)(i - line * g.C);
  float2 w[K + 1];
  int e = 0;
#pragma unroll
  for (int k = 1; k <= K; ++k) {
    e += c;
    if (e >= g.C) e -= g.C;
    w[k] = __ldg(g.twCf + e);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (d >= g.D) break;
    float f = inj ? inj[(long long)d * g.V + i] : 0.0f;
    f += __ldg(R2f + (line * (K + 1)) * g.D + d).x;
#pragma unroll
    for (int k = 1; k <= K; ++k) {
      const float2 z = __ldg(R2f + (line * (K + 1) + k) * g.D + d);
      f = fmaf(z.x, w[k].x, fmaf(-z.y, w[k].y, f));
    }
    field_f[(long long)d * g.V + i] = f;
    field[(long long)d * g.V + i] = widen_exact(f);
  }
}

// float copy of the field for the FP32/FP16-storage kernels (integer-bit
// rounding: conversion instructions run on the narrow FP64 path)
__global__ void narrow_field_kernel(const double* __restrict__ in, float* __restrict__ out,
                                    long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = narrow_rn(in[i]);
}

struct SpectralForce {
  int force = 0;
  SpecGrid g{};
  long long V = 0;
  bool time_dependent = false;
  bool sparse = false;                   // removal by the separable partial transforms
  cufftHandle fwd = 0, inv = 0;
  bool have_fwd = false, have_inv = false;
  cufftDoubleComplex* spec = nullptr;    // [D][nspec] work spectrum (cuFFT removal)
  cufftDoubleComplex* inject = nullptr;  // [D][nspec] injection spectrum (cuFFT removal)
  double* inj_field = nullptr;           // [D][V] injection field (separable removal)
  float* inj_field_f = nullptr;          // its float copy (FP32 updates)
  bool single = false;                   // FP32 separable updates (FP32/FP16 storage)
  float2* twf = nullptr;                 // float twiddle table of the C axis
  float2* R2f = nullptr;
  double* mom = nullptr;                 // [D][V]
  double* field = nullptr;               // [D][V]
  float* field_f = nullptr;              // [D][V] float copy, or null
  SepGrid sg{};
  double2* tw = nullptr;                 // twiddle tables A | B | C
  double2 *P1 = nullptr, *P2 = nullptr, *Ch = nullptr, *R1 = nullptr, *R2 = nullptr;
  double ramp[3] = {0, 0, 0};
  int rkmin = 0, rkmax = 0;
};

static int sf_fail(char* err, size_t n, const char* what, int code) {
  if (err && n) std::snprintf(err, n, "%s (%d)", what, code);
  return 1;
}

void spectral_force_destroy(SpectralForce* sf) {
  if (!sf) return;
  if (sf->have_fwd) cufftDestroy(sf->fwd);
  if (sf->have_inv) cufftDestroy(sf->inv);
  void* ptrs[] = {sf->spec, sf->inject, sf->inj_field, sf->inj_field_f, sf->twf, sf->R2f,
                  sf->mom, sf->field, sf->field_f, sf->tw,
                  sf->P1, sf->P2, sf->Ch, sf->R1, sf->R2};
  for (void* p : ptrs) cudaFree(p);
  delete sf;
}

const double* spectral_force_field(const SpectralForce* sf) { return sf->field; }
const float* spectral_force_field_f(const SpectralForce* sf) { return sf->field_f; }
bool spectral_force_time_dependent(const SpectralForce* sf) { return sf->time_dependent; }

static unsigned blocks_for(long long n) { return (unsigned)((n + 255) / 256); }

// (cos, sin)(2 pi j / n) rounded from extended precision
static void twiddle_table(std::vector<double2>& t, int n) {
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int j = 0; j < n; ++j) {
    const long double x = two_pi * (long double)j / (long double)n;
    t.push_back(make_double2((double)std::cos(x), (double)std::sin(x)));
  }
}

static int setup_sparse(SpectralForce* sf, cudaStream_t st, char* err, size_t errlen) {
  const SpecGrid& g = sf->g;
  SepGrid& s = sf->sg;
  s.D = g.D;
  s.V = sf->V;
  if (g.D == 2) { s.A = 1; s.B = g.lx; s.C = g.ly; } else { s.A = g.lx; s.B = g.ly; s.C = g.lz; }
  s.K = sf->rkmax;
  s.KA = g.D == 2 ? 0 : s.K;
  std::vector<double2> t;
  twiddle_table(t, s.A);
  twiddle_table(t, s.B);
  twiddle_table(t, s.C);
  const long long nk = 2 * s.K + 1, nc = s.K + 1, na = 2 * s.KA + 1;
  cudaError_t e;
  if ((e = cudaMalloc(&sf->tw, sizeof(double2) * t.size())) != cudaSuccess ||
      (e = cudaMalloc(&sf->P1, sizeof(double2) * s.A * s.B * nc * s.D)) != cudaSuccess ||
      (e = cudaMalloc(&sf->R2, sizeof(double2) * s.A * s.B * nc * s.D)) != cudaSuccess ||
      (e = cudaMalloc(&sf->P2, sizeof(double2) * s.A * nk * nc * s.D)) != cudaSuccess ||
      (e = cudaMalloc(&sf->R1, sizeof(double2) * s.A * nk * nc * s.D)) != cudaSuccess ||
      (e = cudaMalloc(&sf->Ch, sizeof(double2) * na * nk * nc * s.D)) != cudaSuccess)
    return sf_fail(err, errlen, "device allocation failed", (int)e);
  if ((e = cudaMemcpy(sf->tw, t.data(), sizeof(double2) * t.size(), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return sf_fail(err, errlen, "twiddle upload failed", (int)e);
  s.twA = sf->tw;
  s.twB = sf->tw + s.A;
  s.twC = sf->tw + s.A + s.B;
  s.twCf = nullptr;
  if (sf->single) {
    std::vector<float2> tf;
    for (int j = 0; j < s.C; ++j) {
      const double2 v = t[s.A + s.B + j];
      tf.push_back(make_float2((float)v.x, (float)v.y));
    }
    if ((e = cudaMalloc(&sf->twf, sizeof(float2) * s.C)) != cudaSuccess ||
        (e = cudaMalloc(&sf->R2f, sizeof(float2) * s.A * s.B * nc * s.D)) != cudaSuccess)
      return sf_fail(err, errlen, "device allocation failed", (int)e);
    if ((e = cudaMemcpy(sf->twf, tf.data(), sizeof(float2) * s.C, cudaMemcpyHostToDevice)) !=
        cudaSuccess)
      return sf_fail(err, errlen, "twiddle upload failed", (int)e);
    s.twCf = sf->twf;
    if (sf->inj_field) {
      const long long n = sf->V * s.D;
      if ((e = cudaMalloc(&sf->inj_field_f, sizeof(float) * n)) != cudaSuccess)
        return sf_fail(err, errlen, "device allocation failed", (int)e);
      // on the handle's stream, after the transform that produced inj_field
      narrow_field_kernel<<<blocks_for(n), 256, 0, st>>>(sf->inj_field, sf->inj_field_f, n);
      count_launches(1);
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess)
        return sf_fail(err, errlen, "injection narrowing failed", (int)e);
    }
  }
  return 0;
}

static void narrow_field(SpectralForce* sf, cudaStream_t s) {
  if (!sf->field_f) return;
  const long long n = sf->V * sf->g.D;
  narrow_field_kernel<<<blocks_for(n), 256, 0, s>>>(sf->field, sf->field_f, n);
  count_launches(1);
}

int spectral_force_create(SpectralForce** out, int force, int D, int lx, int ly, int lz,
                          const double amp[3], int kmin, int kmax, const double ramp[3],
                          int rkmin, int rkmax, int want_float, cudaStream_t s, char* err,
                          size_t errlen) {
  *out = nullptr;
  SpectralForce* sf = new (std::nothrow) SpectralForce();
  if (!sf) return sf_fail(err, errlen, "host allocation failed", 0);
  sf->force = force;
  SpecGrid& g = sf->g;
  g.D = D;
  g.lx = lx; g.ly = ly; g.lz = D == 2 ? 1 : lz;
  g.hx = lx;
  g.hy = D == 2 ? ly / 2 + 1 : ly;
  g.hz = D == 2 ? 1 : lz / 2 + 1;
  g.nspec = (long long)g.hx * g.hy * g.hz;
  sf->V = (long long)lx * ly * g.lz;
  sf->time_dependent = force != MLBM_FORCE_CONSTANT_SHELL;
  sf->sparse = sf->time_dependent && rkmax <= kSparseMaxK;
  sf->single = sf->sparse && want_float;
  for (int d = 0; d < 3; ++d) sf->ramp[d] = ramp[d];
  sf->rkmin = rkmin;
  sf->rkmax = rkmax;
  const double scale = 1.0 / (double)sf->V;
  const bool injection = force != MLBM_FORCE_ENERGY_REMOVAL;
  auto bail = [&](const char* what, int code) {
    spectral_force_destroy(sf);
    return sf_fail(err, errlen, what, code);
  };

  cudaError_t e;
  if ((e = cudaMalloc(&sf->field, sizeof(double) * sf->V * D)) != cudaSuccess ||
      (want_float && (e = cudaMalloc(&sf->field_f, sizeof(float) * sf->V * D)) != cudaSuccess))
    return bail("device allocation failed", (int)e);
  int n[3] = {lx, ly, lz};
  cufftResult r;
  const bool need_inv = injection || !sf->sparse;
  if (need_inv) {
    if ((r = cufftPlanMany(&sf->inv, D, n, nullptr, 1, (int)g.nspec, nullptr, 1, (int)sf->V,
                           CUFFT_Z2D, D)) != CUFFT_SUCCESS)
      return bail("cufftPlanMany Z2D failed", (int)r);
    sf->have_inv = true;
    if ((r = cufftSetStream(sf->inv, s)) != CUFFT_SUCCESS) return bail("cufftSetStream failed", (int)r);
    if ((e = cudaMalloc(&sf->spec, sizeof(cufftDoubleComplex) * g.nspec * D)) != cudaSuccess)
      return bail("device allocation failed", (int)e);
  }
  if (injection) {
    shell_injection_kernel<<<blocks_for(g.nspec), 256, 0, s>>>(g, amp[0], amp[1], amp[2], kmin,
                                                               kmax, scale, sf->spec);
    count_launches(1);
  }
  if (force == MLBM_FORCE_CONSTANT_SHELL || (injection && sf->sparse)) {
    // the injection field, transformed back once
    double* dst = force == MLBM_FORCE_CONSTANT_SHELL ? sf->field : nullptr;
    if (!dst) {
      if ((e = cudaMalloc(&sf->inj_field, sizeof(double) * sf->V * D)) != cudaSuccess)
        return bail("device allocation failed", (int)e);
      dst = sf->inj_field;
    }
    if ((r = cufftExecZ2D(sf->inv, sf->spec, dst)) != CUFFT_SUCCESS)
      return bail("cufftExecZ2D failed", (int)r);
    if (dst == sf->field) narrow_field(sf, s);
  }
  if (sf->sparse) {
    if (setup_sparse(sf, s, err, errlen)) {
      spectral_force_destroy(sf);
      return 1;
    }
  } else if (sf->time_dependent) {
    if ((r = cufftPlanMany(&sf->fwd, D, n, nullptr, 1, (int)sf->V, nullptr, 1, (int)g.nspec,
                           CUFFT_D2Z, D)) != CUFFT_SUCCESS)
      return bail("cufftPlanMany D2Z failed", (int)r);
    sf->have_fwd = true;
    if ((r = cufftSetStream(sf->fwd, s)) != CUFFT_SUCCESS) return bail("cufftSetStream failed", (int)r);
    if ((e = cudaMalloc(&sf->mom, sizeof(double) * sf->V * D)) != cudaSuccess)
      return bail("device allocation failed", (int)e);
    if (injection) {
      // the injection spectrum is kept: Z2D overwrites its input every step
      if ((e = cudaMalloc(&sf->inject, sizeof(cufftDoubleComplex) * g.nspec * D)) != cudaSuccess)
        return bail("device allocation failed", (int)e);
      if ((e = cudaMemcpyAsync(sf->inject, sf->spec, sizeof(cufftDoubleComplex) * g.nspec * D,
                             cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
      return bail("injection copy failed", (int)e);
    }
  }
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return bail("spectral setup failed", (int)e);
  if (sf->sparse || !sf->time_dependent) {
    // the spectrum buffer and inverse plan served the injection only
    cudaFree(sf->spec);
    sf->spec = nullptr;
    if (sf->have_inv) cufftDestroy(sf->inv);
    sf->have_inv = false;
  }
  *out = sf;
  return 0;
}

template <int K>
static void launch_sparse(SpectralForce* sf, const double* rho, const double* u, cudaStream_t s) {
  const SepGrid& g = sf->sg;
  const long long lines = (long long)g.A * g.B;
  if (sf->single)
    sep_forward_c_f<K><<<(unsigned)((lines + 7) / 8), 256, 0, s>>>(g, rho, u, sf->P1);
  else
    sep_forward_c<K><<<(unsigned)((lines + 7) / 8), 256, 0, s>>>(g, rho, u, sf->P1);
  const long long nk = 2 * g.K + 1, nc = g.K + 1, na = 2 * g.KA + 1;
  // one warp per output: 8 outputs per 256-thread block
  sep_forward_b<<<(unsigned)((g.A * nk * nc * g.D + 7) / 8), 256, 0, s>>>(g, sf->P1, sf->P2);
  sep_modes<<<(unsigned)((na * nk * nc * g.D + 7) / 8), 256, 0, s>>>(
      g, sf->P2, sf->Ch, sf->ramp[0], sf->ramp[1], sf->ramp[2], sf->rkmin, sf->rkmax,
      1.0 / (double)sf->V);
  sep_inverse_a<<<blocks_for(g.A * nk * nc * g.D), 256, 0, s>>>(g, sf->Ch, sf->R1);
  sep_inverse_b<<<blocks_for(lines * nc * g.D), 256, 0, s>>>(g, sf->R1, sf->R2,
                                                             sf->single ? sf->R2f : nullptr);
  if (sf->single)
    sep_synthesis_f<K><<<blocks_for(g.V), 256, 0, s>>>(g, sf->R2f, sf->inj_field_f, sf->field_f,
                                                       sf->field);
  else
    sep_synthesis<K><<<blocks_for(g.V), 256, 0, s>>>(g, sf->R2, sf->inj_field, sf->field);
  count_launches(6);
}

int spectral_force_update(SpectralForce* sf, const double* rho, const double* u, cudaStream_t s,
                          char* err, size_t errlen) {
  if (!sf->time_dependent) return 0;
  if (sf->sparse) {
    switch (sf->sg.K) {
      case 0: launch_sparse<0>(sf, rho, u, s); break;
      case 1: launch_sparse<1>(sf, rho, u, s); break;
      case 2: launch_sparse<2>(sf, rho, u, s); break;
      case 3: launch_sparse<3>(sf, rho, u, s); break;
      case 4: launch_sparse<4>(sf, rho, u, s); break;
      default: launch_sparse<5>(sf, rho, u, s); break;
    }
  } else {
    const SpecGrid& g = sf->g;
    momentum_kernel<<<blocks_for(sf->V), 256, 0, s>>>(rho, u, sf->mom, g.D, sf->V);
    count_launches(1);
    cufftResult r;
    if ((r = cufftExecD2Z(sf->fwd, sf->mom, sf->spec)) != CUFFT_SUCCESS)
      return sf_fail(err, errlen, "cufftExecD2Z failed", (int)r);
    removal_filter_kernel<<<blocks_for(g.nspec), 256, 0, s>>>(
        g, sf->spec, sf->inject, sf->ramp[0], sf->ramp[1], sf->ramp[2], sf->rkmin, sf->rkmax,
        1.0 / (double)sf->V);
    count_launches(1);
    if ((r = cufftExecZ2D(sf->inv, sf->spec, sf->field)) != CUFFT_SUCCESS)
      return sf_fail(err, errlen, "cufftExecZ2D failed", (int)r);
  }
  if (!sf->single) narrow_field(sf, s);  // the FP32 updates write the float field directly
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return sf_fail(err, errlen, cudaGetErrorString(e), (int)e);
  return 0;
}

}  // namespace mlbm
