// Small kernels shared by every storage format: the fixed-order reduction of
// the per-block diagnostics partials, and the sample-logger dispatch.

#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "fastlog.cuh"
#include "kernels.h"

namespace mlbm {

// One block of 256 threads: each thread folds a strided subset of the
// partials in index order, then a fixed tree; the result does not depend on
// scheduling, so a diagnostics value is reproducible run to run.
__device__ __forceinline__ void finalize_diag_body(const double* __restrict__ partials, int nblocks,
                                                   double* __restrict__ out, bool root) {
  __shared__ double sh[DIAG_FIELDS][256];
  double m = 0.0, e = 0.0, mach = 0.0, amin = 1e300, amax = -1e300;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double* p = partials + (size_t)b * DIAG_FIELDS;
    m += p[0];
    e += p[1];
    mach = fmax(mach, p[2]);
    amin = fmin(amin, p[3]);
    amax = fmax(amax, p[4]);
  }
  sh[0][threadIdx.x] = m; sh[1][threadIdx.x] = e; sh[2][threadIdx.x] = mach;
  sh[3][threadIdx.x] = amin; sh[4][threadIdx.x] = amax;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
      sh[2][threadIdx.x] = fmax(sh[2][threadIdx.x], sh[2][threadIdx.x + w]);
      sh[3][threadIdx.x] = fmin(sh[3][threadIdx.x], sh[3][threadIdx.x + w]);
      sh[4][threadIdx.x] = fmax(sh[4][threadIdx.x], sh[4][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int k = 0; k < DIAG_FIELDS; ++k) out[k] = sh[k][0];
    // the nodes contribute |u|^2 / c_s^2; sqrt is monotonic and correctly
    // rounded, so the root of the maximum is the maximum of the roots
    if (root) out[2] = sqrt(sh[2][0]);
  }
}

__global__ void finalize_diag_kernel(const double* __restrict__ partials, int nblocks,
                                     double* __restrict__ out) {
  finalize_diag_body(partials, nblocks, out, true);
}

__global__ void fast_log_kernel(const double* __restrict__ x, double* __restrict__ out, long long n,
                                const LogEntry* __restrict__ table) {
  __shared__ LogEntry tab[LOG_TABLE];
  stage_log_table(tab, table);
  __syncthreads();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = fast_log(x[i], tab);
}

cudaError_t fast_log_eval(const double* x, double* out, long long n, const void* table,
                          cudaStream_t s) {
  fast_log_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, out, n,
                                                             (const LogEntry*)table);
  return cudaGetLastError();
}

// First level for long partial lists: block b folds the partials
// [b * chunk, (b + 1) * chunk) with the same fixed-order fold and tree, into
// one partial of its own; finalize_diag_kernel then folds those. The
// partition depends only on the list's length, so the result is still the
// same run to run.
__global__ void fold_diag_kernel(const double* __restrict__ partials, int nblocks, int chunk,
                                 double* __restrict__ folded) {
  const int b0 = blockIdx.x * chunk;
  const int n = min(chunk, nblocks - b0);
  finalize_diag_body(partials + (size_t)b0 * DIAG_FIELDS, n, folded + (size_t)blockIdx.x * DIAG_FIELDS,
                     false);
}

// Partial lists up to this length are folded by one block; longer ones by
// kFoldBlocks blocks first (the handle's partials buffer has room for the
// folded list behind the longest list it holds).
constexpr int kFoldThreshold = 8192;
constexpr int kFoldBlocks = 512;

int finalize_diag_scratch(int nblocks) { return nblocks > kFoldThreshold ? kFoldBlocks : 0; }

cudaError_t finalize_diag(const double* partials, int nblocks, double* out, cudaStream_t s) {
  finalize_diag_kernel<<<1, 256, 0, s>>>(partials, nblocks, out);
  return cudaGetLastError();
}

cudaError_t finalize_diag_fold(double* partials, int nblocks, double* out, cudaStream_t s) {
  if (nblocks <= kFoldThreshold) return finalize_diag(partials, nblocks, out, s);
  const int chunk = (nblocks + kFoldBlocks - 1) / kFoldBlocks;
  const int used = (nblocks + chunk - 1) / chunk;
  double* folded = partials + (size_t)nblocks * DIAG_FIELDS;
  fold_diag_kernel<<<used, 256, 0, s>>>(partials, nblocks, chunk, folded);
  finalize_diag_kernel<<<1, 256, 0, s>>>(folded, used, out);
  return cudaGetLastError();
}

int finalize_diag_launches(int nblocks) { return nblocks > kFoldThreshold ? 2 : 1; }

// Fill of the per-node alpha field: FP64 storage keeps alpha, the other
// storage formats alpha - 2 in float.
__global__ void fill_alpha_kernel(double* __restrict__ a64, float* __restrict__ a32, long long n,
                                  double v64, float v32) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (a64) a64[i] = v64;
  else a32[i] = v32;
}

// Copy of n doubles between any two addresses kernels can access (device
// memory, page-locked or, on NVLink-C2C systems, pageable host memory):
// 16-byte accesses when both ends are 16-byte aligned, grid-stride over a
// grid of a few blocks per SM.
__global__ void copy_doubles_kernel(const double* __restrict__ src, double* __restrict__ dst,
                                    long long n, int vec) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (vec) {
    const long long n2 = n / 2;
    const double2* s2 = reinterpret_cast<const double2*>(src);
    double2* d2 = reinterpret_cast<double2*>(dst);
    for (long long k = i; k < n2; k += stride) d2[k] = s2[k];
    if (i == 0 && (n & 1)) dst[n - 1] = src[n - 1];
  } else {
    for (long long k = i; k < n; k += stride) dst[k] = src[k];
  }
}

cudaError_t copy_doubles(const double* src, double* dst, long long n, cudaStream_t s) {
  int dev = 0, sms = 1;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    sms = 1;
  }
  const int vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0;
  const long long work = vec ? n / 2 : n;
  const long long blocks = std::min<long long>((long long)sms * 8, std::max<long long>(1, (work + 255) / 256));
  copy_doubles_kernel<<<(unsigned)blocks, 256, 0, s>>>(src, dst, n, vec);
  return cudaGetLastError();
}

cudaError_t fill_alpha_field(double* a64, float* a32, long long n, double value, cudaStream_t s) {
  fill_alpha_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a64, a32, n, value,
                                                                 (float)(value - 2.0));
  return cudaGetLastError();
}

#define MLBM_BY_LAT(L, CALL0, CALL1, CALL2) \
  switch (L) { case 0: return CALL0; case 1: return CALL1; case 2: return CALL2; } \
  return cudaErrorInvalidValue;
// the FP64 units exist for all six lattices (0..5)
#define MLBM_BY_LAT6(L, F, ARGS) \
  switch (L) { \
    case 0: return F##_L0 ARGS; case 1: return F##_L1 ARGS; case 2: return F##_L2 ARGS; \
    case 3: return F##_L3 ARGS; case 4: return F##_L4 ARGS; case 5: return F##_L5 ARGS; \
  } \
  return cudaErrorInvalidValue;
// the FP32 / FP16 units exist for D2Q9, D3Q19, D3Q27 and D3Q15 (0..3)
#define MLBM_BY_LAT4(L, C0, C1, C2, C3) \
  switch (L) { case 0: return C0; case 1: return C1; case 2: return C2; case 3: return C3; } \
  return cudaErrorInvalidValue;
#define MLBM_BY_LAT_ST(L, S, F, ARGS) \
  if (S == 1) { MLBM_BY_LAT4(L, F##_L0_S1 ARGS, F##_L1_S1 ARGS, F##_L2_S1 ARGS, F##_L3_S1 ARGS) } \
  if (S == 2) { MLBM_BY_LAT4(L, F##_L0_S2 ARGS, F##_L1_S2 ARGS, F##_L2_S2 ARGS, F##_L3_S2 ARGS) } \
  return cudaErrorInvalidValue;

cudaError_t entropy_test(int lattice, const float* f, const double* fneq, long long nodes,
                         const double* x, int nx, int mode, const void* table,
                         const void* table_fine, double* F, double* D, int* series,
                         cudaStream_t s) {
  MLBM_BY_LAT(lattice, entropy_test_L0(f, fneq, nodes, x, nx, mode, table, table_fine, F, D, series, s),
              entropy_test_L1(f, fneq, nodes, x, nx, mode, table, table_fine, F, D, series, s),
              entropy_test_L2(f, fneq, nodes, x, nx, mode, table, table_fine, F, D, series, s))
}

cudaError_t neq_test(int lattice, const float* f, long long nodes, int dfloat, double* out,
                     cudaStream_t s) {
  MLBM_BY_LAT(lattice, neq_test_L0(f, nodes, dfloat, out, s), neq_test_L1(f, nodes, dfloat, out, s),
              neq_test_L2(f, nodes, dfloat, out, s))
}

cudaError_t alpha_solve_test(int lattice, const double* f, const double* fneq,
                             const double* guess, long long n, const StepParams& p, double* alpha,
                             int* flags, cudaStream_t s) {
  MLBM_BY_LAT6(lattice, alpha_solve_test, (f, fneq, guess, n, p, alpha, flags, s))
}

cudaError_t step_f64x(int lattice, int forcing, const double* prev, double* next,
                      const StepParams& p, cudaStream_t s) {
  MLBM_BY_LAT4(lattice, step_f64x_L0(forcing, prev, next, p, s),
               step_f64x_L1(forcing, prev, next, p, s), step_f64x_L2(forcing, prev, next, p, s),
               step_f64x_L3(forcing, prev, next, p, s))
}

cudaError_t step_f64(int lattice, int collision, int forcing, const double* prev, double* next,
                     const StepParams& p, cudaStream_t s) {
  MLBM_BY_LAT6(lattice, step_f64, (collision, forcing, prev, next, p, s))
}

cudaError_t init_f64(int lattice, const double* rho, const double* u, double* f, long long V,
                     cudaStream_t s) {
  MLBM_BY_LAT6(lattice, init_f64, (rho, u, f, V, s))
}

cudaError_t step_lowp(int lattice, int collision, int forcing, int storage, const void* prev,
                      void* next, const StepParams& p, cudaStream_t s) {
  MLBM_BY_LAT_ST(lattice, storage, step_lowp, (collision, forcing, prev, next, p, s))
}

cudaError_t init_lowp(int lattice, int storage, const double* rho, const double* u, void* f,
                      long long V, cudaStream_t s) {
  MLBM_BY_LAT_ST(lattice, storage, init_lowp, (rho, u, f, V, s))
}

cudaError_t lowp_to_f64(int lattice, int storage, const void* f, int q, double* out, long long V,
                        cudaStream_t s) {
  MLBM_BY_LAT_ST(lattice, storage, lowp_to_f64, (f, q, out, V, s))
}

cudaError_t f64_to_lowp(int lattice, int storage, const double* in, int q, void* f, long long V,
                        cudaStream_t s) {
  MLBM_BY_LAT_ST(lattice, storage, f64_to_lowp, (in, q, f, V, s))
}

cudaError_t log_samples(int lattice, int storage, const void* prev, const StepParams& p,
                        const long long* nodes, long long n, double* features, double* alpha,
                        int* solved, cudaStream_t s) {
  if (storage == 0) {
    MLBM_BY_LAT6(lattice, log_samples_f64,
                 ((const double*)prev, p, nodes, n, features, alpha, solved, s))
  }
  MLBM_BY_LAT_ST(lattice, storage, log_samples_lowp,
                 (prev, p, nodes, n, features, alpha, solved, s))
}

}  // namespace mlbm
