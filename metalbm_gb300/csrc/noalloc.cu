// Allocation-free entry point: one FP64 BGK pull step with fused diagnostics
// on caller-owned device buffers (mlbm_step_f64_noalloc in mlbm.h).
//
// Some callers cannot allocate device memory at all: code running inside a
// host framework that owns every device allocation through its own pool, a
// step replayed from a captured sequence where a cudaMalloc is not allowed,
// or embedded callers with a fixed device-memory budget. The handle API
// (mlbm_create) allocates the populations, fields and the diagnostics scratch;
// this entry point takes the populations (and the force profile) as the
// caller's device buffers and keeps the one piece of scratch the kernel needs
// (the per-block diagnostics partials of the fused reduction) in a
// file-scope __device__ array that every GPU loading the library holds until
// the process exits.
//
// It launches the same FP64 BGK kernel (bit-identical to the reference) and
// the same fixed-order diagnostics reduction as mlbm_step with
// MLBM_STEP_DIAGNOSTICS; nothing is allocated on any call.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>

#include "../../include/mlbm/mlbm.h"
#include "kernels.h"

namespace mlbm {
void set_global_error(const char* message);
void count_launches(unsigned n);
}  // namespace mlbm

using namespace mlbm;

namespace {

constexpr int kBlock = 256;              // nodes per block of the BGK kernel
constexpr int kMaxBlocks = 65536;        // partial slots in the scratch array
constexpr long long kMaxNodes = (long long)kMaxBlocks * kBlock;  // 16,777,216 = 256^3

// Scratch of the fused diagnostics: one slot of DIAG_FIELDS doubles per block
// (2.5 MiB), plus the device error word. Shared by every call on a device.
static __device__ __align__(256) double g_noalloc_partials[kMaxBlocks * DIAG_FIELDS];
static __device__ __align__(256) unsigned int g_noalloc_error_word;

struct Scratch {
  double* partials = nullptr;
  unsigned int* error_word = nullptr;
};

int noalloc_fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int noalloc_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  set_global_error(buf);
  return code;
}

// With the calling thread's current device current: the device addresses of
// the scratch symbols. In host code the symbols' names are host-side
// stand-ins, not device addresses, so the kernels get these pointers instead.
// The first call on a device loads this library's device code there (the
// set-up); later lookups read a table on the host and allocate nothing. The
// address is looked up on every call rather than cached, because a device
// reset or a new primary context reloads the module, possibly elsewhere.
int scratch_for_current_device(Scratch* out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(MLBM_ERR_NO_DEVICE, "no current CUDA device: %s", cudaGetErrorString(e));
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_partials);
  if (e != cudaSuccess)
    return noalloc_fail(MLBM_ERR_CUDA, "cudaGetSymbolAddress(partials) on device %d failed: %s", dev,
                        cudaGetErrorString(e));
  out->partials = static_cast<double*>(p);
  e = cudaGetSymbolAddress(&p, g_noalloc_error_word);
  if (e != cudaSuccess)
    return noalloc_fail(MLBM_ERR_CUDA, "cudaGetSymbolAddress(error word) on device %d failed: %s", dev,
                        cudaGetErrorString(e));
  out->error_word = static_cast<unsigned int*>(p);
  return MLBM_OK;
}

}  // namespace

// ((1 - 1/(2 tau)) w_q) inv_cs2 of the Guo source, from the lattice tables
template <int LAT>
static void guo_factors(StepParams& p, double tau) {
  for (int q = 0; q < Lattice<LAT>::Q; ++q)
    p.guo_k[q] = (1.0 - 1.0 / (2.0 * tau)) * Lattice<LAT>::w(q) * Lattice<LAT>::ics;
}

extern "C" int mlbm_step_f64_noalloc(const mlbm_config* cfg, const double* f_in, double* f_out,
                                     const double* force_profile, double* diag_out,
                                     unsigned int* error_word_out, void* stream) {
  if (!cfg) return noalloc_fail(MLBM_ERR_INVALID, "null configuration");
  const mlbm_config& c = *cfg;
  if (c.lattice < MLBM_D2Q9 || c.lattice > MLBM_D3Q33)
    return noalloc_fail(MLBM_ERR_INVALID, "bad lattice %d", c.lattice);
  if (c.collision != MLBM_BGK)
    return noalloc_fail(MLBM_ERR_INVALID, "the allocation-free step is the BGK collision only");
  if (c.storage != MLBM_STORAGE_F64)
    return noalloc_fail(MLBM_ERR_INVALID, "the allocation-free step uses FP64 storage only");
  if (c.forcing_scheme < 0 || c.forcing_scheme > 3 || c.force < 0 || c.force > 3)
    return noalloc_fail(MLBM_ERR_INVALID, "bad forcing scheme or force");
  if (!(c.relaxation_time > 0.5) || !std::isfinite(c.relaxation_time))
    return noalloc_fail(MLBM_ERR_INVALID, "relaxation time must be > 0.5 (got %g)", c.relaxation_time);
  static const int kD[6] = {2, 3, 3, 3, 2, 3}, kQ[6] = {9, 19, 27, 15, 13, 33};
  const int D = kD[c.lattice];
  const int Q = kQ[c.lattice];
  const long long L[3] = {c.length[0], c.length[1], D == 2 ? 1 : c.length[2]};
  for (int d = 0; d < 3; ++d)
    if (L[d] < 1 || L[d] > 65536) return noalloc_fail(MLBM_ERR_INVALID, "bad length[%d] = %lld", d, L[d]);
  const long long V = L[0] * L[1] * L[2];
  if (V > kMaxNodes)
    return noalloc_fail(MLBM_ERR_INVALID,
                        "lattice of %lld nodes exceeds the allocation-free limit of %lld nodes "
                        "(%d diagnostics slots of %d nodes); use mlbm_create/mlbm_step",
                        V, kMaxNodes, kMaxBlocks, kBlock);
  if (!f_in || !f_out || !diag_out) return noalloc_fail(MLBM_ERR_INVALID, "null buffer");
  if (f_in == f_out) return noalloc_fail(MLBM_ERR_INVALID, "f_in and f_out must be distinct buffers");
  const bool tabulated = c.force == MLBM_FORCE_SINUSOIDAL || c.force == MLBM_FORCE_KOLMOGOROV;
  if (tabulated && !force_profile)
    return noalloc_fail(MLBM_ERR_INVALID, "this force needs the caller's force profile");
  if (c.force == MLBM_FORCE_KOLMOGOROV &&
      (c.kolmogorov_axis < 0 || c.kolmogorov_axis >= D || c.kolmogorov_component < 0 ||
       c.kolmogorov_component >= D))
    return noalloc_fail(MLBM_ERR_INVALID, "bad Kolmogorov axis/component");

  Scratch scratch;
  int rc = scratch_for_current_device(&scratch);
  if (rc != MLBM_OK) return rc;
  const Scratch* s = &scratch;

  // Step parameters, formed as mlbm_create forms them.
  StepParams p{};
  p.V = V;
  p.lx = (uint32_t)L[0]; p.ly = (uint32_t)L[1]; p.lz = (uint32_t)L[2];
  p.div_lz.init(p.lz);
  p.div_ly.init(p.ly);
  p.tau = c.relaxation_time;
  p.beta = (double)1.0 / (2.0 * c.relaxation_time);  // Collision.h:122
  p.bgk_a = 1. - 2. * p.beta;
  p.bgk_b = 2. * p.beta;
  switch (c.lattice) {  // ForcingScheme.h:115-116
    case MLBM_D2Q9: guo_factors<LAT_D2Q9>(p, c.relaxation_time); break;
    case MLBM_D3Q19: guo_factors<LAT_D3Q19>(p, c.relaxation_time); break;
    case MLBM_D3Q27: guo_factors<LAT_D3Q27>(p, c.relaxation_time); break;
    case MLBM_D3Q15: guo_factors<LAT_D3Q15>(p, c.relaxation_time); break;
    case MLBM_D2Q13: guo_factors<LAT_D2Q13>(p, c.relaxation_time); break;
    default: guo_factors<LAT_D3Q33>(p, c.relaxation_time); break;
  }
  p.force_type = c.force;
  p.kol_axis = c.kolmogorov_axis;
  p.kol_comp = c.kolmogorov_component;
  for (int d = 0; d < 3; ++d) p.amp[d] = d < D ? c.force_amplitude[d] : 0.0;
  if (c.force == MLBM_FORCE_KOLMOGOROV) {
    p.force_table[0] = force_profile;
  } else if (c.force == MLBM_FORCE_SINUSOIDAL) {
    p.force_table[0] = force_profile;
    p.force_table[1] = force_profile + L[0];
    p.force_table[2] = D == 3 ? force_profile + L[0] + L[1] : nullptr;
  }
  p.store = 0;
  p.diag = 1;
  p.diag_partials = s->partials;
  p.err_word = s->error_word;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(s->error_word, 0, sizeof(unsigned int), st);
  if (e != cudaSuccess) return noalloc_fail(MLBM_ERR_CUDA, "clearing the error word: %s", cudaGetErrorString(e));
  e = step_f64(c.lattice, 0, c.forcing_scheme, f_in, f_out, p, st);
  if (e != cudaSuccess) return noalloc_fail(MLBM_ERR_CUDA, "step kernel: %s", cudaGetErrorString(e));
  const int nblocks = (int)((V + kBlock - 1) / kBlock);
  e = finalize_diag(s->partials, nblocks, diag_out, st);
  if (e != cudaSuccess) return noalloc_fail(MLBM_ERR_CUDA, "diagnostics: %s", cudaGetErrorString(e));
  count_launches(2);
  if (error_word_out) {
    e = cudaMemcpyAsync(error_word_out, s->error_word, sizeof(unsigned int), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return noalloc_fail(MLBM_ERR_CUDA, "error word copy: %s", cudaGetErrorString(e));
  }
  return MLBM_OK;
}
