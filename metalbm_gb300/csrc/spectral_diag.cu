// Spectral analyses of the stored fields on the device: the vorticity by the
// spectral curl, total energy and enstrophy, and the shell energy spectrum,
// as the reference's Routine computes them after a stored step
// (Routine.h:69-72, 126-131; AnalysisList.h:55-73, 135-171).
//
//   * forward transforms: unnormalised real-to-complex over the lattice
//     (Transformer.h:38-112), one batched cuFFT D2Z of the D velocity
//     components;
//   * wavenumbers: the signed integers k_d = i_d for i_d <= L_d / 2, else
//     i_d - L_d, the halved last axis 0 .. L_last / 2 (Transformer.h:146-151);
//   * curl (Transformer.h:118-295): omega_hat = i k x u_hat per component,
//     brought back by cuFFT Z2D, divided by V for the normalised backward
//     transform and by V once more (Curl::normalize, Transformer.h:181-187,
//     285-294). In 2-D the reference keeps the real part of i k x u_hat only
//     (its imaginary part is multiplied by 0, Transformer.h:160-164); that
//     spectrum is real and even in k, so any complex-to-real transform of it
//     agrees;
//   * TotalEnergy (1/V) sum 1/2 rho |u|^2 and TotalEnstrophy
//     (1/V) sum 1/2 |omega|^2 (Analysis.h:33-98);
//   * PowerSpectra (Analysis.h:122-177): for every half-spectrum mode,
//     coef * sum_d |u_hat_d|^2 with coef = 1/2 on the k_last = 0 plane and 1
//     elsewhere, added to shell floor(|k|) below the reference's shell count
//     max(L_x, min(L_y, L_z)) / 2 (FourierDomain.h:77-79, whose arrayMax
//     recursion takes the minimum of the remaining lengths, Helpers.h:37-39),
//     divided by V.
// Sums are fixed-order block reductions (reproducible run to run), except the
// spectrum's per-block shell histograms, which add in shared memory in
// arrival order (reproducible to rounding); the blocks' histograms are then
// summed in block order.

#include <cufft.h>

#include <cstdio>
#include <new>

#include "common.cuh"
#include "kernels.h"

namespace mlbm {

namespace {

constexpr int kThreads = 256;
constexpr int kSpecBlocks = 512;  // fixed, so the summation order does not depend on the GPU

struct DiagGrid {
  int D;
  int lx, ly, lz;  // real extents (lz = 1 in 2-D)
  int hx, hy, hz;  // half-spectrum extents
  long long V, nspec;
  int nshells;
};

__device__ __forceinline__ void wavenumbers(const DiagGrid& g, long long m, int k[3]) {
  const int iz = (int)(m % g.hz);
  const long long t = m / g.hz;
  const int iy = (int)(t % g.hy);
  const int ix = (int)(t / g.hy);
  k[0] = ix <= g.lx / 2 ? ix : ix - g.lx;
  if (g.D == 2) {
    k[1] = iy;  // the halved axis
    k[2] = 0;
  } else {
    k[1] = iy <= g.ly / 2 ? iy : iy - g.ly;
    k[2] = iz;  // the halved axis
  }
}

// floor(sqrt(n)) for n < 2^40 without rounding surprises
__device__ __forceinline__ int isqrt(long long n) {
  long long s = (long long)sqrt((double)n);
  while (s * s > n) --s;
  while ((s + 1) * (s + 1) <= n) ++s;
  return (int)s;
}

// Per-block shell histograms of coef * sum_d |u_hat_d|^2.
__global__ void __launch_bounds__(kThreads) spectrum_kernel(DiagGrid g,
                                                            const cufftDoubleComplex* __restrict__ uh,
                                                            double* __restrict__ partial) {
  extern __shared__ double hist[];
  for (int s = threadIdx.x; s < g.nshells; s += blockDim.x) hist[s] = 0.0;
  __syncthreads();
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < g.nspec;
       m += (long long)gridDim.x * blockDim.x) {
    int k[3];
    wavenumbers(g, m, k);
    const int shell = isqrt((long long)k[0] * k[0] + (long long)k[1] * k[1] + (long long)k[2] * k[2]);
    if (shell >= g.nshells) continue;
    double e = 0.0;
    for (int d = 0; d < g.D; ++d) {
      const cufftDoubleComplex v = uh[(long long)d * g.nspec + m];
      e += v.x * v.x + v.y * v.y;
    }
    const bool last_zero = (g.D == 2 ? k[1] : k[2]) == 0;
    atomicAdd(&hist[shell], last_zero ? 0.5 * e : e);
  }
  __syncthreads();
  for (int s = threadIdx.x; s < g.nshells; s += blockDim.x)
    partial[(long long)blockIdx.x * g.nshells + s] = hist[s];
}

// spectrum[s] = (sum over blocks, in block order) / V
__global__ void spectrum_finalize_kernel(const double* __restrict__ partial, int nblocks,
                                         int nshells, double inv_volume, double* __restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nshells) return;
  double acc = 0.0;
  for (int b = 0; b < nblocks; ++b) acc += partial[(long long)b * nshells + s];
  out[s] = acc * inv_volume;
}

// One component of omega_hat = i k x u_hat (2-D: the real part of the one
// component only).
__global__ void curl_kernel(DiagGrid g, const cufftDoubleComplex* __restrict__ uh, int c,
                            cufftDoubleComplex* __restrict__ wh) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= g.nspec) return;
  int k[3];
  wavenumbers(g, m, k);
  auto u = [&](int d) { return uh[(long long)d * g.nspec + m]; };
  // a x b component c with a = k, b = u_hat: (k_i b_j - k_j b_i), (i, j) cyclic after c
  int i, j;
  if (g.D == 2) { i = 0; j = 1; }
  else { i = (c + 1) % 3; j = (c + 2) % 3; }
  const cufftDoubleComplex bi = u(i), bj = u(j);
  const double zr = k[i] * bj.x - k[j] * bi.x, zi = k[i] * bj.y - k[j] * bi.y;
  // i z = -zi + i zr
  cufftDoubleComplex w;
  w.x = -zi;
  w.y = g.D == 2 ? 0.0 : zr;
  wh[m] = w;
}

// w *= scale in place; per-block sums of w^2 (fixed order: each thread's
// strided terms in order, then a shared-memory tree).
__global__ void __launch_bounds__(kThreads) scale_square_kernel(double* __restrict__ w, long long n,
                                                                 double scale,
                                                                 double* __restrict__ partial) {
  __shared__ double sh[kThreads];
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = w[i] * scale;
    w[i] = v;
    acc += v * v;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// per-block sums of 1/2 rho |u|^2
__global__ void __launch_bounds__(kThreads) energy_kernel(const double* __restrict__ rho,
                                                           const double* __restrict__ u, int D,
                                                           long long V,
                                                           double* __restrict__ partial) {
  __shared__ double sh[kThreads];
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < V;
       i += (long long)gridDim.x * blockDim.x) {
    double u2 = 0.0;
    for (int d = 0; d < D; ++d) {
      const double v = u[(long long)d * V + i];
      u2 += v * v;
    }
    acc += 0.5 * rho[i] * u2;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// out[slot] (+)= scale * sum of the partials in block order
__global__ void sum_partials_kernel(const double* __restrict__ partial, int n, double scale,
                                    int accumulate, double* __restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double acc = 0.0;
  for (int b = 0; b < n; ++b) acc += partial[b];
  *out = accumulate ? *out + acc * scale : acc * scale;
}

unsigned blocks_for(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace

struct SpectralDiag {
  DiagGrid g{};
  cufftHandle fwd = 0, inv = 0;
  bool have_fwd = false, have_inv = false;
  cufftDoubleComplex* uh = nullptr;  // [D][nspec]
  cufftDoubleComplex* wh = nullptr;  // [nspec], one curl component
  double* w = nullptr;               // [V], one vorticity component
  double* partial = nullptr;         // block partials (max of the reductions)
  double* out = nullptr;             // energy, enstrophy, spectrum[nshells]
};

static int sd_fail(char* err, size_t errlen, const char* what, int code) {
  std::snprintf(err, errlen, "%s (%d)", what, code);
  return 1;
}

void spectral_diag_destroy(SpectralDiag* sd) {
  if (!sd) return;
  if (sd->have_fwd) cufftDestroy(sd->fwd);
  if (sd->have_inv) cufftDestroy(sd->inv);
  cudaFree(sd->uh);
  cudaFree(sd->wh);
  cudaFree(sd->w);
  cudaFree(sd->partial);
  cudaFree(sd->out);
  delete sd;
}

int spectral_diag_shells(int D, int lx, int ly, int lz) {
  const int l3 = D == 2 ? 1 : lz;
  const int inner = ly < l3 ? ly : l3;
  return (lx > inner ? lx : inner) / 2;
}

int spectral_diag_create(SpectralDiag** out, int D, int lx, int ly, int lz, cudaStream_t s,
                         char* err, size_t errlen) {
  SpectralDiag* sd = new (std::nothrow) SpectralDiag();
  if (!sd) return sd_fail(err, errlen, "host allocation failed", 0);
  DiagGrid& g = sd->g;
  g.D = D;
  g.lx = lx; g.ly = ly; g.lz = D == 2 ? 1 : lz;
  g.hx = lx;
  g.hy = D == 2 ? ly / 2 + 1 : ly;
  g.hz = D == 2 ? 1 : lz / 2 + 1;
  g.V = (long long)g.lx * g.ly * g.lz;
  g.nspec = (long long)g.hx * g.hy * g.hz;
  g.nshells = spectral_diag_shells(D, lx, ly, lz);
  auto bail = [&](const char* what, int code) {
    spectral_diag_destroy(sd);
    return sd_fail(err, errlen, what, code);
  };
  if (g.nspec > 0x7fffffffLL || g.V > 0x7fffffffLL)
    return bail("lattice too large for the spectral analyses", 0);
  const long long npart = (long long)kSpecBlocks * (g.nshells > 1 ? g.nshells : 1);
  cudaError_t e;
  if ((e = cudaMalloc(&sd->uh, sizeof(cufftDoubleComplex) * g.nspec * D)) != cudaSuccess ||
      (e = cudaMalloc(&sd->wh, sizeof(cufftDoubleComplex) * g.nspec)) != cudaSuccess ||
      (e = cudaMalloc(&sd->w, sizeof(double) * g.V)) != cudaSuccess ||
      (e = cudaMalloc(&sd->partial, sizeof(double) * (npart > kSpecBlocks ? npart : kSpecBlocks))) !=
          cudaSuccess ||
      (e = cudaMalloc(&sd->out, sizeof(double) * (2 + g.nshells))) != cudaSuccess) {
    cudaGetLastError();
    return bail("device allocation failed", (int)e);
  }
  int n[3] = {g.lx, g.ly, g.lz};
  cufftResult r;
  if ((r = cufftPlanMany(&sd->fwd, D, n, nullptr, 1, (int)g.V, nullptr, 1, (int)g.nspec,
                         CUFFT_D2Z, D)) != CUFFT_SUCCESS)
    return bail("cufftPlanMany D2Z failed", (int)r);
  sd->have_fwd = true;
  if ((r = cufftPlanMany(&sd->inv, D, n, nullptr, 1, (int)g.nspec, nullptr, 1, (int)g.V,
                         CUFFT_Z2D, 1)) != CUFFT_SUCCESS)
    return bail("cufftPlanMany Z2D failed", (int)r);
  sd->have_inv = true;
  if ((r = cufftSetStream(sd->fwd, s)) != CUFFT_SUCCESS ||
      (r = cufftSetStream(sd->inv, s)) != CUFFT_SUCCESS)
    return bail("cufftSetStream failed", (int)r);
  *out = sd;
  return 0;
}

int spectral_diag_nshells(const SpectralDiag* sd) { return sd->g.nshells; }
long long spectral_diag_volume(const SpectralDiag* sd) { return sd->g.V; }
const double* spectral_diag_results(const SpectralDiag* sd) { return sd->out; }
const double* spectral_diag_vorticity(const SpectralDiag* sd) { return sd->w; }

// Energy, the spectrum and the forward transforms (results in out[0] and
// out[2..]); the curl and enstrophy come component by component from
// spectral_diag_curl.
int spectral_diag_run(SpectralDiag* sd, const double* rho, const double* u, cudaStream_t s,
                      char* err, size_t errlen) {
  const DiagGrid& g = sd->g;
  const double inv_v = 1.0 / (double)g.V;
  energy_kernel<<<kSpecBlocks, kThreads, 0, s>>>(rho, u, g.D, g.V, sd->partial);
  sum_partials_kernel<<<1, 32, 0, s>>>(sd->partial, kSpecBlocks, inv_v, 0, sd->out);
  cufftResult r;
  // the plan reads u through a const-less pointer; cuFFT D2Z does not write its input
  if ((r = cufftExecD2Z(sd->fwd, const_cast<double*>(u), sd->uh)) != CUFFT_SUCCESS)
    return sd_fail(err, errlen, "cufftExecD2Z failed", (int)r);
  if (g.nshells > 0) {
    spectrum_kernel<<<kSpecBlocks, kThreads, sizeof(double) * g.nshells, s>>>(g, sd->uh,
                                                                             sd->partial);
    spectrum_finalize_kernel<<<(g.nshells + 127) / 128, 128, 0, s>>>(
        sd->partial, kSpecBlocks, g.nshells, inv_v, sd->out + 2);
  }
  count_launches(g.nshells > 0 ? 4 : 2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return sd_fail(err, errlen, cudaGetErrorString(e), (int)e);
  return 0;
}

// Vorticity component c (0 in 2-D) into spectral_diag_vorticity(); its
// 1/2 |omega_c|^2 / V added to out[1] (c = 0 starts the sum).
int spectral_diag_curl(SpectralDiag* sd, int c, cudaStream_t s, char* err, size_t errlen) {
  const DiagGrid& g = sd->g;
  const double inv_v = 1.0 / (double)g.V;
  curl_kernel<<<blocks_for(g.nspec), kThreads, 0, s>>>(g, sd->uh, c, sd->wh);
  cufftResult r;
  if ((r = cufftExecZ2D(sd->inv, sd->wh, sd->w)) != CUFFT_SUCCESS)
    return sd_fail(err, errlen, "cufftExecZ2D failed", (int)r);
  // the normalised backward transform (1/V) and Curl::normalize (1/V again)
  scale_square_kernel<<<kSpecBlocks, kThreads, 0, s>>>(sd->w, g.V, inv_v * inv_v, sd->partial);
  sum_partials_kernel<<<1, 32, 0, s>>>(sd->partial, kSpecBlocks, 0.5 * inv_v, c > 0 ? 1 : 0,
                                       sd->out + 1);
  count_launches(3);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return sd_fail(err, errlen, cudaGetErrorString(e), (int)e);
  return 0;
}

}  // namespace mlbm
