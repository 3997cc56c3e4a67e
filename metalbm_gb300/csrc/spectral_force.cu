// Spectral forces (Force.h:294-626): ConstantShell, EnergyRemoval and
// Turbulent2D as a per-node force field [D][V] that the FP64 step kernels
// read (FORCE_FIELD in node_force).
//
// The reference computes them with FFTW r2c/c2r transforms on the host
// (Transformer.h:19-110). Here the transforms are cuFFT D2Z/Z2D plans batched
// over the D components, and everything between them is one kernel pass over
// the half spectrum:
//   * ConstantShell: the spectrum A on the shell kmin^2 <= |k|^2 <= kmax^2
//     (integer wavenumbers, Force.h:339-347, 386), made solenoidal by the curl
//     i k x T (3-D, Transformer.h:207-272) or (i k_y psi, -i k_x psi) (2-D,
//     Transformer.h:298-387), divided by the node count (the backward
//     transform's normalisation, Transformer.h:98-108) and transformed back
//     once, at creation;
//   * EnergyRemoval: every step, the momentum rho u of the last stored fields
//     (Force.h:442-463), forward transform, -A_d on the shell and 0 elsewhere
//     (Force.h:496-532), divided by the node count, backward transform;
//   * Turbulent2D: the two added (Force.h:596-612), in the spectrum, so one
//     backward transform serves both.
// Every spectrum stays Hermitian: the reference's partner writes on the
// k_y = k_z = 0 row of 3-D lattices, which index y = L_y and land one row off
// (or past the array), are not reproduced. Shells stay below the Nyquist
// wavenumber (checked by the caller).

#include <cufft.h>

#include <cstdio>
#include <new>

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

struct SpectralForce {
  int force = 0;
  SpecGrid g{};
  long long V = 0;
  bool time_dependent = false;
  cufftHandle fwd = 0, inv = 0;
  bool have_fwd = false, have_inv = false;
  cufftDoubleComplex* spec = nullptr;    // [D][nspec] work spectrum
  cufftDoubleComplex* inject = nullptr;  // [D][nspec] injection spectrum (Turbulent2D)
  double* mom = nullptr;                 // [D][V]
  double* field = nullptr;               // [D][V]
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
  cudaFree(sf->spec);
  cudaFree(sf->inject);
  cudaFree(sf->mom);
  cudaFree(sf->field);
  delete sf;
}

const double* spectral_force_field(const SpectralForce* sf) { return sf->field; }
bool spectral_force_time_dependent(const SpectralForce* sf) { return sf->time_dependent; }

static unsigned blocks_for(long long n) { return (unsigned)((n + 255) / 256); }

int spectral_force_create(SpectralForce** out, int force, int D, int lx, int ly, int lz,
                          const double amp[3], int kmin, int kmax, const double ramp[3],
                          int rkmin, int rkmax, cudaStream_t s, char* err, size_t errlen) {
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
  for (int d = 0; d < 3; ++d) sf->ramp[d] = ramp[d];
  sf->rkmin = rkmin;
  sf->rkmax = rkmax;
  const double scale = 1.0 / (double)sf->V;

  int n[3] = {lx, ly, lz};
  cufftResult r;
  if ((r = cufftPlanMany(&sf->inv, D, n, nullptr, 1, (int)g.nspec, nullptr, 1, (int)sf->V,
                         CUFFT_Z2D, D)) != CUFFT_SUCCESS) {
    spectral_force_destroy(sf);
    return sf_fail(err, errlen, "cufftPlanMany Z2D failed", (int)r);
  }
  sf->have_inv = true;
  cufftSetStream(sf->inv, s);
  cudaError_t e;
  if ((e = cudaMalloc(&sf->spec, sizeof(cufftDoubleComplex) * g.nspec * D)) != cudaSuccess ||
      (e = cudaMalloc(&sf->field, sizeof(double) * sf->V * D)) != cudaSuccess) {
    spectral_force_destroy(sf);
    return sf_fail(err, errlen, "device allocation failed", (int)e);
  }
  const bool injection = force != MLBM_FORCE_ENERGY_REMOVAL;
  if (injection) {
    shell_injection_kernel<<<blocks_for(g.nspec), 256, 0, s>>>(g, amp[0], amp[1], amp[2], kmin,
                                                               kmax, scale, sf->spec);
    count_launches(1);
  }
  if (force == MLBM_FORCE_CONSTANT_SHELL) {
    // time-independent: one backward transform, then only the field is kept
    if ((r = cufftExecZ2D(sf->inv, sf->spec, sf->field)) != CUFFT_SUCCESS) {
      spectral_force_destroy(sf);
      return sf_fail(err, errlen, "cufftExecZ2D failed", (int)r);
    }
    cudaStreamSynchronize(s);
    cudaFree(sf->spec);
    sf->spec = nullptr;
    *out = sf;
    return 0;
  }
  if ((r = cufftPlanMany(&sf->fwd, D, n, nullptr, 1, (int)sf->V, nullptr, 1, (int)g.nspec,
                         CUFFT_D2Z, D)) != CUFFT_SUCCESS) {
    spectral_force_destroy(sf);
    return sf_fail(err, errlen, "cufftPlanMany D2Z failed", (int)r);
  }
  sf->have_fwd = true;
  cufftSetStream(sf->fwd, s);
  if ((e = cudaMalloc(&sf->mom, sizeof(double) * sf->V * D)) != cudaSuccess) {
    spectral_force_destroy(sf);
    return sf_fail(err, errlen, "device allocation failed", (int)e);
  }
  if (injection) {
    // the injection spectrum is kept: Z2D overwrites its input every step
    if ((e = cudaMalloc(&sf->inject, sizeof(cufftDoubleComplex) * g.nspec * D)) != cudaSuccess) {
      spectral_force_destroy(sf);
      return sf_fail(err, errlen, "device allocation failed", (int)e);
    }
    cudaMemcpyAsync(sf->inject, sf->spec, sizeof(cufftDoubleComplex) * g.nspec * D,
                    cudaMemcpyDeviceToDevice, s);
  }
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) {
    spectral_force_destroy(sf);
    return sf_fail(err, errlen, "injection spectrum failed", (int)e);
  }
  *out = sf;
  return 0;
}

int spectral_force_update(SpectralForce* sf, const double* rho, const double* u, cudaStream_t s,
                          char* err, size_t errlen) {
  if (!sf->time_dependent) return 0;
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
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return sf_fail(err, errlen, cudaGetErrorString(e), (int)e);
  return 0;
}

}  // namespace mlbm
