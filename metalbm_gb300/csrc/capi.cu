// C ABI of the fused collide-and-stream pull step (include/mlbm/mlbm.h).
//
// Host side of the drop-in: it owns the device buffers of one periodic
// lattice (what Distribution and FieldList own in the reference,
// Distribution.h:14-43, FieldList.h:22-86), converts host arrays between the
// dense and the reference's padded layout, and enqueues the step kernels on
// one CUDA stream. Errors are returned as status codes with a message; no
// call aborts the process.

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mlbm/mlbm.h"
#include "../../include/mlbm/mlbm_testing.h"
#include "kernels.h"
#include "fastlog.cuh"
#include "mlp_device.cuh"
#include "mlp_train.h"

using namespace mlbm;

namespace {

std::atomic<unsigned long long> g_launches{0};
std::mutex g_create_error_mutex;
std::string g_create_error;

const int kQ[6] = {9, 19, 27, 15, 13, 33};
const int kD[6] = {2, 3, 3, 3, 2, 3};
const double kPi = 3.14159265358979323846;

}  // namespace

namespace mlbm {
void count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
// Error message of a call made without a handle (mlbm_last_error(NULL)).
void set_global_error(const char* message) {
  std::lock_guard<std::mutex> lk(g_create_error_mutex);
  g_create_error = message;
}
}  // namespace mlbm

struct mlbm_handle {
  mlbm_config cfg{};
  int Q = 0, D = 0;
  long long V = 0;
  uint32_t lx = 0, ly = 0, lz = 0;
  int storage = 0;
  size_t elem = 8;  // bytes per stored population value
  void* f[2] = {nullptr, nullptr};
  int cur = 0;      // f[cur] holds the current populations
  double* rho = nullptr;
  double* u = nullptr;
  double* force = nullptr;
  double* alpha = nullptr;      // FP64 storage
  float* alpha32 = nullptr;     // low-precision storage
  double* force_table[3] = {nullptr, nullptr, nullptr};
  float* force_table_f[3] = {nullptr, nullptr, nullptr};
  double* partials = nullptr;
  int partial_blocks = 0;
  int main_blocks = 0;          // blocks of the (first) step kernel
  // entropic FP32/FP16 step: second-pass worklist
  unsigned* defer_list = nullptr;
  unsigned* defer_count = nullptr;  // [2] worklist lengths, [2] cold-node flags (by parity)
  // learned guess: nodes without a solved alpha may exist (after init, a
  // restart, set_alpha, or a step that stored alpha = 2)
  bool alpha_cold = true;
  bool learned_now = false;  // the steps being enqueued run the network
  int defer_blocks = 0;
  double* diag_dev = nullptr;
  unsigned long long* counters = nullptr;
  unsigned* err_word = nullptr;
  double* staging = nullptr;    // V doubles
  MlpDev* mlp = nullptr;
  LogEntry* log_table = nullptr;
  LogEntryFine* log_table_fine = nullptr;
  bool have_model = false;
  long long* sample_nodes = nullptr;
  long long n_samples = 0;
  double* sample_feat = nullptr;
  double* sample_alpha = nullptr;
  int* sample_solved = nullptr;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  long long steps = 0;
  bool diag_valid = false;
  bool fields_valid = false;
  StepParams base{};
  SpectralForce* spectral = nullptr;  // spectral forces (FP64 storage)
  SpectralDiag* sdiag = nullptr;      // spectral analyses, created on first use
  // the stored fields changed since the time-dependent force was computed
  // from them (its only inputs): recompute before the next step
  bool force_stale = true;
  std::string error;
};

static int fail(mlbm_handle* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) {
    h->error = buf;
  } else {
    std::lock_guard<std::mutex> lk(g_create_error_mutex);
    g_create_error = buf;
  }
  return code;
}

#define MLBM_CUDA(h, call)                                                              \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail((h), MLBM_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));  \
  } while (0)

static int device_alloc(mlbm_handle* h, void** p, size_t bytes) {
  if (bytes == 0) { *p = nullptr; return MLBM_OK; }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(h, MLBM_ERR_ALLOC, "cudaMalloc of %zu bytes failed: %s", bytes,
                cudaGetErrorString(e));
  }
  return MLBM_OK;
}

// ---- layouts -----------------------------------------------------------------
// Reference layout (lSD, Domain.h:42-92 + FFTW padding): the last active
// dimension padded to 2*(N/2+1); component stride = padded volume.
struct RefLayout {
  long long px, py, pz;  // padded extents
  long long volume;
};
static RefLayout ref_layout(const mlbm_handle* h) {
  RefLayout r;
  r.px = h->lx;
  if (h->D == 2) {
    r.py = 2 * (h->ly / 2 + 1);
    r.pz = 1;
  } else {
    r.py = h->ly;
    r.pz = 2 * (h->lz / 2 + 1);
  }
  r.volume = r.px * r.py * r.pz;
  return r;
}

// Copy ncomp components between dense [c][V] and reference [c][padded].
static void dense_from_ref(const mlbm_handle* h, const double* ref, double* dense, int ncomp) {
  const RefLayout r = ref_layout(h);
  for (int c = 0; c < ncomp; ++c)
    for (uint32_t x = 0; x < h->lx; ++x)
      for (uint32_t y = 0; y < h->ly; ++y)
        for (uint32_t z = 0; z < h->lz; ++z)
          dense[(long long)c * h->V + ((long long)x * h->ly + y) * h->lz + z] =
              ref[(long long)c * r.volume + (x * r.py + y) * r.pz + z];
}
static void ref_from_dense(const mlbm_handle* h, const double* dense, double* ref, int ncomp) {
  const RefLayout r = ref_layout(h);
  for (int c = 0; c < ncomp; ++c)
    for (uint32_t x = 0; x < h->lx; ++x)
      for (uint32_t y = 0; y < h->ly; ++y)
        for (uint32_t z = 0; z < h->lz; ++z)
          ref[(long long)c * r.volume + (x * r.py + y) * r.pz + z] =
              dense[(long long)c * h->V + ((long long)x * h->ly + y) * h->lz + z];
}

// The address through which kernels on `device` access the n doubles at
// `host`, when they can: page-locked (registered) host memory whose
// registration covers the first and the last element, or any host memory on
// a device that accesses pageable memory through the host's page tables
// (NVLink-C2C systems). nullptr otherwise (device memory included).
static double* device_view(int device, const double* host, size_t n) {
  int pageable = 0, host_tables = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess ||
      cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                             device) != cudaSuccess) {
    cudaGetLastError();
    pageable = host_tables = 0;
  }
  cudaPointerAttributes a{}, b{};
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess ||
      cudaPointerGetAttributes(&b, host + (n - 1)) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return nullptr;
  if (a.type == cudaMemoryTypeHost && b.type == cudaMemoryTypeHost && a.devicePointer &&
      b.devicePointer &&
      (const char*)b.devicePointer - (const char*)a.devicePointer ==
          (std::ptrdiff_t)((n - 1) * sizeof(double)))
    return (double*)a.devicePointer;
  if (pageable && host_tables && a.type == cudaMemoryTypeUnregistered &&
      b.type == cudaMemoryTypeUnregistered)
    return const_cast<double*>(host);
  return nullptr;
}

// Upload ncomp host components (given layout) into device dense memory. A
// dense array that kernels can read in place is moved by a copy kernel over
// the host link (on GB300 systems several times the rate that the copy
// engines reach from 64 KiB-page host memory); others by cudaMemcpyAsync.
static int upload(mlbm_handle* h, const double* host, double* dev, int ncomp, int layout) {
  const size_t bytes = sizeof(double) * (size_t)h->V * ncomp;
  if (layout == MLBM_LAYOUT_DENSE) {
    if (const double* view = device_view(h->cfg.device, host, (size_t)h->V * ncomp)) {
      cudaError_t e = copy_doubles(view, dev, h->V * ncomp, h->stream);
      count_launches(1);
      if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "host copy: %s", cudaGetErrorString(e));
    } else {
      MLBM_CUDA(h, cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, h->stream));
    }
    MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
    return MLBM_OK;
  }
  std::vector<double> tmp;
  try { tmp.resize((size_t)h->V * ncomp); } catch (...) {
    return fail(h, MLBM_ERR_ALLOC, "host staging of %zu bytes failed", bytes);
  }
  dense_from_ref(h, host, tmp.data(), ncomp);
  MLBM_CUDA(h, cudaMemcpyAsync(dev, tmp.data(), bytes, cudaMemcpyHostToDevice, h->stream));
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  return MLBM_OK;
}

static int download(mlbm_handle* h, const double* dev, double* host, int ncomp, int layout) {
  const size_t bytes = sizeof(double) * (size_t)h->V * ncomp;
  if (layout == MLBM_LAYOUT_DENSE) {
    if (double* view = device_view(h->cfg.device, host, (size_t)h->V * ncomp)) {
      cudaError_t e = copy_doubles(dev, view, h->V * ncomp, h->stream);
      count_launches(1);
      if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "host copy: %s", cudaGetErrorString(e));
    } else {
      MLBM_CUDA(h, cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, h->stream));
    }
    MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
    return MLBM_OK;
  }
  std::vector<double> tmp;
  try { tmp.resize((size_t)h->V * ncomp); } catch (...) {
    return fail(h, MLBM_ERR_ALLOC, "host staging of %zu bytes failed", bytes);
  }
  MLBM_CUDA(h, cudaMemcpyAsync(tmp.data(), dev, bytes, cudaMemcpyDeviceToHost, h->stream));
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  ref_from_dense(h, tmp.data(), host, ncomp);
  return MLBM_OK;
}

static bool valid_layout(int layout) {
  return layout == MLBM_LAYOUT_DENSE || layout == MLBM_LAYOUT_REFERENCE;
}

// ---- API -----------------------------------------------------------------------
extern "C" int mlbm_config_init(mlbm_config* c) {
  if (!c) return MLBM_ERR_INVALID;
  std::memset(c, 0, sizeof *c);
  c->lattice = MLBM_D2Q9;
  c->collision = MLBM_BGK;
  c->forcing_scheme = MLBM_FORCING_NONE;
  c->force = MLBM_FORCE_NONE;
  c->relaxation_time = 0.7;
  for (int d = 0; d < 3; ++d) c->force_wavelength[d] = 32.0;
  c->kolmogorov_axis = 1;
  c->kolmogorov_component = 0;
  c->length[0] = c->length[1] = c->length[2] = 16;
  c->storage = MLBM_STORAGE_F64;
  c->alpha_mode = MLBM_ALPHA_REFERENCE;
  c->alpha_guess = MLBM_GUESS_PREVIOUS;
  c->newton_tolerance = 1e-8;
  c->newton_max_iterations = 50;
  c->deviation_threshold = 1e-3;
  c->device = 0;
  c->force_kmin = 1;  // Input_prod_3d.in:52-58
  c->force_kmax = 2;
  c->removal_kmin = 1;
  c->removal_kmax = 2;
  for (int d = 0; d < 3; ++d) c->removal_amplitude[d] = 1e-6;
  return MLBM_OK;
}

static void release(mlbm_handle* h) {
  if (!h) return;
  void* ptrs[] = {h->f[0], h->f[1], h->rho, h->u, h->force, h->alpha, h->alpha32,
                  h->force_table[0], h->force_table[1], h->force_table[2], h->force_table_f[0],
                  h->force_table_f[1], h->force_table_f[2], h->partials,
                  h->diag_dev, h->counters, h->err_word, h->staging, h->mlp, h->log_table,
                  h->log_table_fine, h->defer_list, h->defer_count, h->sample_nodes,
                  h->sample_feat, h->sample_alpha, h->sample_solved};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  spectral_force_destroy(h->spectral);
  spectral_diag_destroy(h->sdiag);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
}

// Table of the FP64 logarithm (fastlog.cuh): for the centre c_j of each of
// the 128 mantissa intervals, inv_j = RN(1/c_j) and -ln(inv_j) split into a
// double-double, evaluated in the host's extended precision.
// Host copy of a lattice's weights (reference population order) and
// inv_cs2, from the same compile-time tables the kernels use (lattice.cuh).
struct HostLattice {
  double w[kMaxQ];
  double ics;
};
template <int LAT>
static HostLattice host_lattice_of() {
  HostLattice h{};
  for (int q = 0; q < Lattice<LAT>::Q; ++q) h.w[q] = Lattice<LAT>::w(q);
  h.ics = Lattice<LAT>::ics;
  return h;
}
static const HostLattice& host_lattice(int lattice) {
  static const HostLattice t[6] = {host_lattice_of<0>(), host_lattice_of<1>(), host_lattice_of<2>(),
                                   host_lattice_of<3>(), host_lattice_of<4>(), host_lattice_of<5>()};
  return t[lattice];
}
static const double* lattice_weights(int lattice) { return host_lattice(lattice).w; }

// Fine log tables (1024 x {RN(1/c_j), RN(ln(1/inv_j))} and its float
// companion {RN_float(1/c_j), ln(1/inv_j) as a float pair}) with the
// lattice's constants C_q(d) = d ln 2 - ln(m_q), w_q = m_q 2^e_q (FP64) and
// -ln(m_q) as float pairs (fastlog.cuh FineTables).
using FineTable = FineTables;
static void make_log_table_fine(FineTable* ft, int lattice) {
  std::memset(ft, 0, sizeof *ft);
  for (int j = 0; j < LOG_TABLE_FINE; ++j) {
    const double c = 1.0 + (j + 0.5) / (double)LOG_TABLE_FINE;
    const double inv = 1.0 / c;
    ft->t[j].inv = inv;
    ft->t[j].hi = (double)(-std::log((long double)inv));
    const float invf = (float)(1.0L / (long double)c);
    const long double T = -std::log((long double)invf);
    const float hi = (float)T;
    ft->tf[j].inv = invf;
    ft->tf[j].hi = hi;
    ft->tf[j].lo = (float)(T - (long double)hi);
  }
  const double* wl = lattice_weights(lattice);
  const int Q = kQ[lattice];
  for (int q = 0; q < 27; ++q) {
    const double wq = q < Q ? wl[q] : 1.0;
    int ew = 0;
    const long double mw = 2.0L * std::frexp((long double)wq, &ew);  // wq = mw 2^(ew - 1)
    for (int d = -1; d <= 1; ++d)
      ft->lnw[3 * q + d + 1] =
          (double)((long double)d * 0.693147180559945309417232121458176568L - std::log(mw));
    const long double C = -std::log(mw);
    ft->lnwf[q][0] = (float)C;
    ft->lnwf[q][1] = (float)(C - (long double)(float)C);
  }
}

static void make_log_table(LogEntry* t) {
  for (int j = 0; j < LOG_TABLE; ++j) {
    const double c = 1.0 + (j + 0.5) / (double)LOG_TABLE;
    const double inv = 1.0 / c;
    const long double L = -std::log((long double)inv);
    const double hi = (double)L;
    t[j].inv = inv;
    t[j].hi = hi;
    t[j].lo = (double)(L - (long double)hi);
  }
}

static double host_sin_profile(double amplitude, unsigned i, double lambda) {
  // Force.h:213, 266: amplitude * sin(iP * 2 * M_PI / waveLength), with the
  // unsigned coordinate times 2 formed in integer arithmetic.
  return amplitude * std::sin((double)(i * 2u) * kPi / lambda);
}

static int fill_alpha(mlbm_handle* h, double value) {
  h->alpha_cold = true;
  cudaError_t e = fill_alpha_field(h->alpha, h->alpha32, h->V, value, h->stream);
  count_launches(1);
  if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "alpha fill: %s", cudaGetErrorString(e));
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  return MLBM_OK;
}

extern "C" int mlbm_create(const mlbm_config* cfg, mlbm_handle** out) {
  if (!cfg || !out) return fail(nullptr, MLBM_ERR_INVALID, "null argument");
  *out = nullptr;
  const mlbm_config& c = *cfg;
  if (c.lattice < 0 || c.lattice > MLBM_D3Q33) return fail(nullptr, MLBM_ERR_INVALID, "bad lattice %d", c.lattice);
  if (c.collision < MLBM_BGK || c.collision > MLBM_FORCED_NR_ELBM)
    return fail(nullptr, MLBM_ERR_INVALID, "bad collision %d", c.collision);
  if (c.forcing_scheme < 0 || c.forcing_scheme > 3)
    return fail(nullptr, MLBM_ERR_INVALID, "bad forcing scheme %d", c.forcing_scheme);
  if (c.force < 0 || c.force > MLBM_FORCE_TURBULENT_2D)
    return fail(nullptr, MLBM_ERR_INVALID, "bad force %d", c.force);
  if (c.storage < 0 || c.storage > 2) return fail(nullptr, MLBM_ERR_INVALID, "bad storage %d", c.storage);
  if (c.storage != MLBM_STORAGE_F64 && (c.lattice == MLBM_D2Q13 || c.lattice == MLBM_D3Q33))
    return fail(nullptr, MLBM_ERR_INVALID,
                "FP32 / FP16 storage supports D2Q9, D3Q19, D3Q27 and D3Q15; lattice %d runs with "
                "FP64 storage",
                c.lattice);
  if (!(c.relaxation_time > 0.5) || !std::isfinite(c.relaxation_time))
    return fail(nullptr, MLBM_ERR_INVALID, "relaxation time must be > 0.5 (got %g)", c.relaxation_time);
  if (c.alpha_mode < 0 || c.alpha_mode > 1) return fail(nullptr, MLBM_ERR_INVALID, "bad alpha mode");
  if (c.alpha_guess < 0 || c.alpha_guess > MLBM_GUESS_LEARNED_EVERYWHERE)
    return fail(nullptr, MLBM_ERR_INVALID, "bad alpha guess");
  const bool learned = c.alpha_guess == MLBM_GUESS_LEARNED ||
                       c.alpha_guess == MLBM_GUESS_LEARNED_EVERYWHERE;
  if (learned && c.storage == MLBM_STORAGE_F64)
    return fail(nullptr, MLBM_ERR_INVALID, "the learned alpha guess runs with FP32/FP16 storage");
  if (c.fp64_arithmetic != MLBM_F64_REFERENCE_ORDER && c.fp64_arithmetic != MLBM_F64_FIXED_POINT)
    return fail(nullptr, MLBM_ERR_INVALID, "bad fp64_arithmetic %d", c.fp64_arithmetic);
  if (c.newton_max_iterations < 0 || c.bisection_max_iterations < 0 || !(c.newton_tolerance >= 0))
    return fail(nullptr, MLBM_ERR_INVALID, "bad Newton parameters");
  const int D = kD[c.lattice];
  long long L[3] = {c.length[0], c.length[1], D == 2 ? 1 : c.length[2]};
  for (int d = 0; d < 3; ++d)
    if (L[d] < 1 || L[d] > 65536) return fail(nullptr, MLBM_ERR_INVALID, "bad length[%d] = %lld", d, L[d]);
  const long long V = L[0] * L[1] * L[2];
  if (V >= (1ll << 31)) return fail(nullptr, MLBM_ERR_INVALID, "lattice too large (%lld nodes)", V);
  if (c.force == MLBM_FORCE_KOLMOGOROV &&
      (c.kolmogorov_axis < 0 || c.kolmogorov_axis >= D || c.kolmogorov_component < 0 ||
       c.kolmogorov_component >= D))
    return fail(nullptr, MLBM_ERR_INVALID, "bad Kolmogorov axis/component");
  if (c.force == MLBM_FORCE_SINUSOIDAL || c.force == MLBM_FORCE_KOLMOGOROV)
    for (int d = 0; d < D; ++d)
      if (c.force_wavelength[d] == 0.0) return fail(nullptr, MLBM_ERR_INVALID, "zero force wavelength");

  const bool spectral = c.force >= MLBM_FORCE_CONSTANT_SHELL;
  if (spectral) {
    long long lmin = L[0];
    for (int d = 1; d < D; ++d) lmin = std::min(lmin, L[d]);
    // every force takes forceAmplitude / forcekMin / forcekMax (Algorithm.h:90-91);
    // the removal* parameters are the removal part of Turbulent2D (Force.h:585-587)
    const bool rem = c.force == MLBM_FORCE_TURBULENT_2D;
    if ((c.force_kmin < 0 || c.force_kmax < c.force_kmin || 2LL * c.force_kmax >= lmin) ||
        (rem && (c.removal_kmin < 0 || c.removal_kmax < c.removal_kmin ||
                 2LL * c.removal_kmax >= lmin)))
      return fail(nullptr, MLBM_ERR_INVALID,
                  "bad spectral shell: need 0 <= kmin <= kmax and 2 kmax < the shortest length");
  }

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(nullptr, MLBM_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (c.device < 0 || c.device >= ndev) return fail(nullptr, MLBM_ERR_INVALID, "bad device %d", c.device);

  mlbm_handle* h = new (std::nothrow) mlbm_handle();
  if (!h) return fail(nullptr, MLBM_ERR_ALLOC, "host allocation failed");
  h->cfg = c;
  if (h->cfg.collision >= MLBM_FORCED_BNR_ELBM) h->cfg.collision = MLBM_ELBM;
  h->Q = kQ[c.lattice];
  h->D = D;
  h->lx = (uint32_t)L[0];
  h->ly = (uint32_t)L[1];
  h->lz = (uint32_t)L[2];
  h->V = V;
  h->storage = c.storage;
  h->elem = c.storage == MLBM_STORAGE_F64 ? 8 : (c.storage == MLBM_STORAGE_F32 ? 4 : 2);

  auto bail = [&](int code) {
    std::string msg = h->error;
    release(h);
    return fail(nullptr, code, "%s", msg.c_str());
  };
  if (cudaSetDevice(c.device) != cudaSuccess) {
    cudaGetLastError();
    h->error = "cudaSetDevice failed";
    return bail(MLBM_ERR_CUDA);
  }
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    h->error = "cudaStreamCreate failed";
    return bail(MLBM_ERR_CUDA);
  }
  h->stream = h->own_stream;

  const size_t popBytes = h->elem * (size_t)h->Q * (size_t)V;
  int rc;
  if ((rc = device_alloc(h, &h->f[0], popBytes)) || (rc = device_alloc(h, &h->f[1], popBytes)) ||
      (rc = device_alloc(h, (void**)&h->rho, sizeof(double) * V)) ||
      (rc = device_alloc(h, (void**)&h->u, sizeof(double) * V * D)) ||
      (rc = device_alloc(h, (void**)&h->force, sizeof(double) * V * D)) ||
      (rc = device_alloc(h, (void**)&h->staging, sizeof(double) * V)))
    return bail(rc);
  if (c.storage == MLBM_STORAGE_F64) {
    if ((rc = device_alloc(h, (void**)&h->alpha, sizeof(double) * V))) return bail(rc);
  } else {
    if ((rc = device_alloc(h, (void**)&h->alpha32, sizeof(float) * V))) return bail(rc);
  }
  const int bs = 128;  // smallest block size of the step kernels
  h->main_blocks = (int)((V + bs - 1) / bs);
  h->partial_blocks = h->main_blocks;
  const bool two_pass = c.collision != MLBM_BGK && c.storage != MLBM_STORAGE_F64;
  if (two_pass) {
    if (V > 0xffffffffLL) {
      h->error = "entropic FP32/FP16 lattices are limited to 2^32 - 1 nodes";
      return bail(MLBM_ERR_INVALID);
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device) != cudaSuccess ||
        sms <= 0) {
      cudaGetLastError();
      sms = 1;
    }
    h->defer_blocks = 2 * sms;
    h->partial_blocks += h->defer_blocks;
    if ((rc = device_alloc(h, (void**)&h->defer_list, sizeof(unsigned) * (size_t)V)) ||
        (rc = device_alloc(h, (void**)&h->defer_count, 4 * sizeof(unsigned))))
      return bail(rc);
    cudaMemsetAsync(h->defer_count, 0, 4 * sizeof(unsigned), h->stream);
  }
  if ((rc = device_alloc(h, (void**)&h->partials,
                         sizeof(double) * DIAG_FIELDS *
                             (h->partial_blocks + finalize_diag_scratch(h->partial_blocks)))) ||
      (rc = device_alloc(h, (void**)&h->diag_dev, sizeof(double) * DIAG_FIELDS)) ||
      (rc = device_alloc(h, (void**)&h->counters, sizeof(unsigned long long) * CNT_COUNT)) ||
      (rc = device_alloc(h, (void**)&h->err_word, sizeof(unsigned))) ||
      (rc = device_alloc(h, (void**)&h->mlp, sizeof(MlpDev))) ||
      (rc = device_alloc(h, (void**)&h->log_table, sizeof(LogEntry) * LOG_TABLE)) ||
      (rc = device_alloc(h, (void**)&h->log_table_fine, sizeof(FineTable))))
    return bail(rc);
  {
    LogEntry tab[LOG_TABLE];
    make_log_table(tab);
    std::unique_ptr<FineTable> fine(new FineTable);
    make_log_table_fine(fine.get(), c.lattice);
    if (cudaMemcpy(h->log_table, tab, sizeof tab, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->log_table_fine, fine.get(), sizeof(FineTable), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
      h->error = "log table upload failed";
      return bail(MLBM_ERR_CUDA);
    }
  }
  cudaMemsetAsync(h->f[0], 0, popBytes, h->stream);
  cudaMemsetAsync(h->f[1], 0, popBytes, h->stream);
  // the stored fields start at zero (EnergyRemoval reads them before the
  // first store or mlbm_init_equilibrium)
  cudaMemsetAsync(h->rho, 0, sizeof(double) * V, h->stream);
  cudaMemsetAsync(h->u, 0, sizeof(double) * V * D, h->stream);
  cudaMemsetAsync(h->force, 0, sizeof(double) * V * D, h->stream);
  cudaMemsetAsync(h->counters, 0, sizeof(unsigned long long) * CNT_COUNT, h->stream);
  cudaMemsetAsync(h->err_word, 0, sizeof(unsigned), h->stream);
  cudaMemsetAsync(h->mlp, 0, sizeof(MlpDev), h->stream);

  // Spectral forces: the force field on the device (spectral_force.cu).
  if (spectral) {
    char msg[256] = {0};
    // EnergyRemoval alone removes with the force amplitude and shell; in
    // Turbulent2D the force parameters inject and the removal ones remove
    const bool alone = c.force == MLBM_FORCE_ENERGY_REMOVAL;
    if (spectral_force_create(&h->spectral, c.force, D, (int)L[0], (int)L[1], (int)L[2],
                              c.force_amplitude, c.force_kmin, c.force_kmax,
                              alone ? c.force_amplitude : c.removal_amplitude,
                              alone ? c.force_kmin : c.removal_kmin,
                              alone ? c.force_kmax : c.removal_kmax,
                              c.storage != MLBM_STORAGE_F64, h->stream, msg, sizeof msg)) {
      h->error = std::string("spectral force: ") + msg;
      return bail(MLBM_ERR_CUDA);
    }
  }
  // Force profiles tabulated on the host (Force.h:208-215, 262-267).
  if (c.force == MLBM_FORCE_SINUSOIDAL || c.force == MLBM_FORCE_KOLMOGOROV) {
    const int ntab = c.force == MLBM_FORCE_SINUSOIDAL ? D : 1;
    for (int t = 0; t < ntab; ++t) {
      const int axis = c.force == MLBM_FORCE_SINUSOIDAL ? t : c.kolmogorov_axis;
      const int comp = c.force == MLBM_FORCE_SINUSOIDAL ? t : c.kolmogorov_component;
      const long long n = L[axis];
      std::vector<double> tab(n);
      for (long long i = 0; i < n; ++i)
        tab[i] = host_sin_profile(c.force_amplitude[comp], (unsigned)i, c.force_wavelength[comp]);
      std::vector<float> tabf(tab.begin(), tab.end());
      if ((rc = device_alloc(h, (void**)&h->force_table[t], sizeof(double) * n)) ||
          (rc = device_alloc(h, (void**)&h->force_table_f[t], sizeof(float) * n)))
        return bail(rc);
      if (cudaMemcpy(h->force_table[t], tab.data(), sizeof(double) * n, cudaMemcpyHostToDevice) !=
              cudaSuccess ||
          cudaMemcpy(h->force_table_f[t], tabf.data(), sizeof(float) * n, cudaMemcpyHostToDevice) !=
              cudaSuccess) {
        h->error = "force table upload failed";
        return bail(MLBM_ERR_CUDA);
      }
    }
  }

  StepParams& p = h->base;
  p.V = V;
  p.lx = h->lx; p.ly = h->ly; p.lz = h->lz;
  p.div_lz.init(h->lz);
  p.div_ly.init(h->ly);
  p.tau = c.relaxation_time;
  p.beta = (double)1.0 / (2.0 * c.relaxation_time);     // Collision.h:122
  p.bgk_a = 1. - 2. * p.beta;                            // Collision.h:145
  p.bgk_b = 2. * p.beta;                                 // Collision.h:147
  {
    const HostLattice& hl = host_lattice(c.lattice);
    for (int q = 0; q < h->Q; ++q)  // ForcingScheme.h:115-116
      p.guo_k[q] = (1.0 - 1.0 / (2.0 * c.relaxation_time)) * hl.w[q] * hl.ics;
  }
  p.force_type = spectral ? FORCE_FIELD : c.force;
  p.force_field = spectral ? spectral_force_field(h->spectral) : nullptr;
  p.force_field_f = spectral ? spectral_force_field_f(h->spectral) : nullptr;
  p.kol_axis = c.kolmogorov_axis;
  p.kol_comp = c.kolmogorov_component;
  for (int d = 0; d < 3; ++d) p.amp[d] = d < D ? c.force_amplitude[d] : 0.0;
  for (int t = 0; t < 3; ++t) {
    p.force_table[t] = h->force_table[t];
    p.force_table_f[t] = h->force_table_f[t];
    p.amp_f[t] = (float)p.amp[t];
  }
  p.bgk_b_f = (float)p.bgk_b;
  p.guo_kt_f = (float)((1.0 - 1.0 / (2.0 * c.relaxation_time)) * 3.0);
  p.alpha_mode = c.alpha_mode;
  p.guess_mode = c.alpha_guess;
  p.newton_tol = c.newton_tolerance;
  {
    // the fixed-point BGK kernel's omega = 2 beta = a + (omega - a), a the
    // integer nearest omega in {0, 1, 2}, and Guo's factors: values times
    // 2^62 (exact: products of doubles and a power of two) as 31-bit halves
    const double om = p.bgk_b;
    const int a = om < 0.5 ? 0 : (om < 1.5 ? 1 : 2);
    const double r = om - a;
    p.fx_ok = om > 0.0 && om < 2.0 ? 1 : 0;  // |1 - omega| < 1, |omega - a| <= 1/2
    p.fx_omega_a = a;
    auto split31 = [](long long x, int out[2]) {
      out[0] = (int)(x >> 31);
      out[1] = (int)(x & 0x7fffffffLL);
    };
    auto halves = [&](double v, int out[2]) { split31(std::llround(std::ldexp(v, 62)), out); };
    halves(p.fx_ok ? r : 0.0, p.fx_omega_s31);
    // (1 - omega) 2^62 = 2^62 - omega 2^62, exact in integers (omega 2^62 is
    // an integer for omega >= 2^-9; smaller omega rounds once)
    split31(p.fx_ok ? (1LL << 62) - std::llround(std::ldexp(om, 62)) : 0LL, p.fx_1mw_s31);
    for (int q = 0; q < h->Q; ++q) {
      const bool in = std::fabs(p.guo_k[q]) < 1.0;
      if (!in && c.forcing_scheme == MLBM_FORCING_GUO) p.fx_ok = 0;
      halves(in ? p.guo_k[q] : 0.0, p.fx_guo_s31[q]);
    }
  }
  p.newton_maxit = c.newton_max_iterations;
  p.bisect_maxit = c.bisection_max_iterations > 0 ? c.bisection_max_iterations
                                                  : c.newton_max_iterations;
  p.deviation_threshold = c.deviation_threshold;
  p.deviation_threshold_f = (float)c.deviation_threshold;
  p.rho_out = h->rho;
  p.u_out = h->u;
  p.force_out = h->force;
  p.alpha_field = h->alpha;
  p.alpha_field_f32 = h->alpha32;
  p.diag_partials = h->partials;
  p.counters = h->counters;
  p.err_word = h->err_word;
  p.mlp = h->mlp;
  p.log_table = h->log_table;
  p.log_table_fine = h->log_table_fine;
  p.defer_list = h->defer_list;
  p.defer_count = h->defer_count;
  p.cold_flags = h->defer_count ? h->defer_count + 2 : nullptr;
  p.defer_blocks = h->defer_blocks;
  p.defer_slot0 = h->main_blocks;

  if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
    h->error = std::string("device initialisation failed: ") + cudaGetErrorString(cudaGetLastError());
    return bail(MLBM_ERR_CUDA);
  }
  // alpha = 2 from construction on (initAlpha, Initialize.h:82-89), so a
  // handle filled with mlbm_set_populations starts as the reference does
  if ((rc = fill_alpha(h, 2.0))) return bail(rc);
  *out = h;
  return MLBM_OK;
}

extern "C" int mlbm_destroy(mlbm_handle* h) {
  if (!h) return MLBM_ERR_INVALID;
  cudaSetDevice(h->cfg.device);
  cudaStreamSynchronize(h->stream);
  release(h);
  return MLBM_OK;
}

extern "C" int mlbm_init_equilibrium(mlbm_handle* h, const double* rho, const double* u, int layout) {
  if (!h) return MLBM_ERR_INVALID;
  if (!rho || !u || !valid_layout(layout)) return fail(h, MLBM_ERR_INVALID, "bad arguments");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  int rc;
  // rho and u go through the field buffers (overwritten by the next store;
  // a spectral force is formed from them before the first step).
  if ((rc = upload(h, rho, h->rho, 1, layout))) return rc;
  if ((rc = upload(h, u, h->u, h->D, layout))) return rc;
  cudaError_t e = h->storage == MLBM_STORAGE_F64
                      ? init_f64(h->cfg.lattice, h->rho, h->u, (double*)h->f[h->cur], h->V, h->stream)
                      : init_lowp(h->cfg.lattice, h->storage, h->rho, h->u, h->f[h->cur], h->V, h->stream);
  count_launches(1);
  if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "init kernel: %s", cudaGetErrorString(e));
  if ((rc = fill_alpha(h, 2.0))) return rc;  // Initialize.h:82-89
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->fields_valid = false;
  h->force_stale = true;
  return MLBM_OK;
}

extern "C" int mlbm_set_populations(mlbm_handle* h, const double* f, int layout) {
  if (!h) return MLBM_ERR_INVALID;
  if (!f || !valid_layout(layout)) return fail(h, MLBM_ERR_INVALID, "bad arguments");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  const RefLayout r = ref_layout(h);
  const long long stride = layout == MLBM_LAYOUT_DENSE ? h->V : r.volume;
  int rc;
  for (int q = 0; q < h->Q; ++q) {
    double* dst = h->storage == MLBM_STORAGE_F64 ? (double*)h->f[h->cur] + (long long)q * h->V
                                                 : h->staging;
    if ((rc = upload(h, f + (long long)q * stride, dst, 1, layout))) return rc;
    if (h->storage != MLBM_STORAGE_F64) {
      cudaError_t e = f64_to_lowp(h->cfg.lattice, h->storage, h->staging, q, h->f[h->cur], h->V,
                                  h->stream);
      count_launches(1);
      if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "encode: %s", cudaGetErrorString(e));
      MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
    }
  }
  h->fields_valid = false;
  return MLBM_OK;
}

extern "C" int mlbm_get_populations(mlbm_handle* h, double* f, int layout) {
  if (!h) return MLBM_ERR_INVALID;
  if (!f || !valid_layout(layout)) return fail(h, MLBM_ERR_INVALID, "bad arguments");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  const RefLayout r = ref_layout(h);
  const long long stride = layout == MLBM_LAYOUT_DENSE ? h->V : r.volume;
  int rc;
  for (int q = 0; q < h->Q; ++q) {
    const double* src = (const double*)h->f[h->cur] + (long long)q * h->V;
    if (h->storage != MLBM_STORAGE_F64) {
      cudaError_t e = lowp_to_f64(h->cfg.lattice, h->storage, h->f[h->cur], q, h->staging, h->V,
                                  h->stream);
      count_launches(1);
      if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "decode: %s", cudaGetErrorString(e));
      src = h->staging;
    }
    if ((rc = download(h, src, f + (long long)q * stride, 1, layout))) return rc;
  }
  return MLBM_OK;
}

static int enqueue_step(mlbm_handle* h, bool last, unsigned int flags, bool in_place);

// MLBM_GUESS_LEARNED: the network runs where a node has no solved alpha from
// the previous step. Whether any node of the lattice is in that state is
// known on the host after initialisation and set_alpha, and from the
// cold-node flag the previous step's kernels set on the device; a call that
// starts with none runs the kernels without the network (they take the
// previous alpha everywhere, and a node that falls back to alpha = 2 during
// the call takes the constant 2 until the next call). LEARNED_EVERYWHERE
// always runs the network.
static int choose_learned_kernel(mlbm_handle* h) {
  h->learned_now = false;
  if (h->cfg.collision == MLBM_BGK || h->storage == MLBM_STORAGE_F64) return MLBM_OK;
  if (h->cfg.alpha_guess == MLBM_GUESS_LEARNED_EVERYWHERE) {
    h->learned_now = true;
    return MLBM_OK;
  }
  if (h->cfg.alpha_guess != MLBM_GUESS_LEARNED) return MLBM_OK;
  if (!h->alpha_cold && h->steps > 0 && h->defer_count) {
    unsigned flag = 0;
    MLBM_CUDA(h, cudaMemcpy(&flag, h->defer_count + 2 + ((h->steps - 1) & 1), sizeof flag,
                            cudaMemcpyDeviceToHost));
    h->alpha_cold = flag != 0;
  }
  h->learned_now = h->alpha_cold;
  h->alpha_cold = false;  // the flags of this call's steps report what they store
  return MLBM_OK;
}

extern "C" int mlbm_step(mlbm_handle* h, int nsteps, unsigned int flags) {
  int rc0;
  if (!h) return MLBM_ERR_INVALID;
  if (nsteps < 0) return fail(h, MLBM_ERR_INVALID, "negative step count");
  if (nsteps == 0) return MLBM_OK;
  if ((flags & MLBM_STEP_LOG_SAMPLES) && h->n_samples == 0)
    return fail(h, MLBM_ERR_STATE, "LOG_SAMPLES without sample nodes (mlbm_set_sample_nodes)");
  if ((h->cfg.alpha_guess == MLBM_GUESS_LEARNED ||
       h->cfg.alpha_guess == MLBM_GUESS_LEARNED_EVERYWHERE) &&
      h->cfg.collision != MLBM_BGK && !h->have_model)
    return fail(h, MLBM_ERR_STATE, "learned alpha guess without a model (mlbm_set_alpha_model)");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  if ((rc0 = choose_learned_kernel(h))) return rc0;
  MLBM_CUDA(h, cudaMemsetAsync(h->counters, 0, sizeof(unsigned long long) * CNT_COUNT, h->stream));
  for (int s = 0; s < nsteps; ++s) {
    int rc = enqueue_step(h, s == nsteps - 1, flags, false);
    if (rc) return rc;
  }
  return MLBM_OK;
}

// One pull step from the current populations (the body of mlbm_step). With
// in_place the result goes to the spare buffer and the handle keeps the
// current populations (no swap, no step counted; the alpha field and the
// stored fields are updated as by a step).
static int enqueue_step(mlbm_handle* h, bool last, unsigned int flags, bool in_place) {
  const int collision = h->cfg.collision == MLBM_BGK ? 0 : 1;
  {
    StepParams p = h->base;
    p.parity = (int)(h->steps & 1);
    p.learned_kernel = h->learned_now ? 1 : 0;
    p.store = last && (flags & MLBM_STEP_STORE_FIELDS) ? 1 : 0;
    p.diag = last && (flags & MLBM_STEP_DIAGNOSTICS) ? 1 : 0;
    const void* prev = h->f[h->cur];
    void* next = h->f[1 - h->cur];
    if (h->spectral && spectral_force_time_dependent(h->spectral) && h->force_stale) {
      // Collision::update before the sweep (Algorithm.h:338): the force field
      // from the last stored fields. The reference recomputes it every step;
      // between stores its inputs do not change, so neither does the field.
      char msg[256] = {0};
      if (spectral_force_update(h->spectral, h->rho, h->u, h->stream, msg, sizeof msg))
        return fail(h, MLBM_ERR_CUDA, "spectral force: %s", msg);
      h->force_stale = false;
    }
    const bool fixed = h->storage == MLBM_STORAGE_F64 &&
                       h->cfg.fp64_arithmetic == MLBM_F64_FIXED_POINT && p.fx_ok &&
                       f64x_supported(h->cfg.lattice, collision, h->cfg.forcing_scheme);
    cudaError_t e = fixed ? step_f64x(h->cfg.lattice, h->cfg.forcing_scheme, (const double*)prev,
                                      (double*)next, p, h->stream)
                    : h->storage == MLBM_STORAGE_F64
                        ? step_f64(h->cfg.lattice, collision, h->cfg.forcing_scheme,
                                   (const double*)prev, (double*)next, p, h->stream)
                        : step_lowp(h->cfg.lattice, collision, h->cfg.forcing_scheme, h->storage,
                                    prev, next, p, h->stream);
    count_launches(h->defer_blocks > 0 ? 2 : 1);
    if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "step kernel: %s", cudaGetErrorString(e));
    if (p.diag) {
      const int nb = collision ? (int)((h->V + 127) / 128) + h->defer_blocks
                               : (int)bgk_step_blocks(h->cfg.lattice, h->storage, h->V,
                                                      (unsigned)h->base.lz);
      e = finalize_diag_fold(h->partials, nb, h->diag_dev, h->stream);
      count_launches(finalize_diag_launches(nb));
      if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "diagnostics: %s", cudaGetErrorString(e));
    }
    if (last && (flags & MLBM_STEP_LOG_SAMPLES)) {
      e = log_samples(h->cfg.lattice, h->storage, prev, p, h->sample_nodes, h->n_samples,
                      h->sample_feat, h->sample_alpha, h->sample_solved, h->stream);
      count_launches(1);
      if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "samples: %s", cudaGetErrorString(e));
    }
    if (!in_place) {
      h->cur = 1 - h->cur;  // std::swap(prev, next), Algorithm.h:336
      ++h->steps;
    } else if (h->defer_count) {
      // the next step has the same parity: its worklist starts empty again
      MLBM_CUDA(h, cudaMemsetAsync(h->defer_count + (h->steps & 1), 0, sizeof(unsigned), h->stream));
    }
    if (p.store) {
      h->fields_valid = true;
      h->force_stale = true;
    }
    if (p.diag) h->diag_valid = true;
  }
  return MLBM_OK;
}

extern "C" int mlbm_testing_step_in_place(mlbm_handle* h) {
  if (!h) return MLBM_ERR_INVALID;
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  int rc = choose_learned_kernel(h);
  if (rc) return rc;
  rc = enqueue_step(h, true, 0u, true);
  // its cold-node flag sits at the parity the next step reuses and clears:
  // the next call decides from the host state instead
  h->alpha_cold = true;
  return rc;
}

extern "C" int mlbm_sync(mlbm_handle* h, int timeout_ms) {
  if (!h) return MLBM_ERR_INVALID;
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaStreamQuery(h->stream);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) return fail(h, MLBM_ERR_CUDA, "stream error: %s", cudaGetErrorString(e));
    if (timeout_ms >= 0) {
      const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(
                          std::chrono::steady_clock::now() - t0).count();
      if (ms >= timeout_ms) return fail(h, MLBM_ERR_TIMEOUT, "device work not finished after %d ms", timeout_ms);
    }
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  unsigned err = 0;
  MLBM_CUDA(h, cudaMemcpy(&err, h->err_word, sizeof err, cudaMemcpyDeviceToHost));
  if (err) return fail(h, MLBM_ERR_NUMERIC, "device error word 0x%x (non-finite or non-positive density)", err);
  return MLBM_OK;
}

extern "C" int mlbm_get_fields(mlbm_handle* h, double* rho, double* u, double* alpha, double* force,
                               int layout) {
  if (!h) return MLBM_ERR_INVALID;
  if (!valid_layout(layout)) return fail(h, MLBM_ERR_INVALID, "bad layout");
  if (!h->fields_valid) return fail(h, MLBM_ERR_STATE, "no stored fields (use MLBM_STEP_STORE_FIELDS)");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  int rc;
  if (rho && (rc = download(h, h->rho, rho, 1, layout))) return rc;
  if (u && (rc = download(h, h->u, u, h->D, layout))) return rc;
  if (force && (rc = download(h, h->force, force, h->D, layout))) return rc;
  if (alpha) {
    if (h->alpha) {
      if ((rc = download(h, h->alpha, alpha, 1, layout))) return rc;
    } else {
      std::vector<float> a((size_t)h->V);
      std::vector<double> ad((size_t)h->V);
      MLBM_CUDA(h, cudaMemcpy(a.data(), h->alpha32, sizeof(float) * h->V, cudaMemcpyDeviceToHost));
      for (long long i = 0; i < h->V; ++i) ad[i] = 2.0 + (double)a[i];
      if (layout == MLBM_LAYOUT_DENSE) std::memcpy(alpha, ad.data(), sizeof(double) * h->V);
      else ref_from_dense(h, ad.data(), alpha, 1);
    }
  }
  return MLBM_OK;
}

extern "C" int mlbm_spectrum_shells(const mlbm_handle* h, int* nshells) {
  if (!h || !nshells) return MLBM_ERR_INVALID;
  *nshells = spectral_diag_shells(h->D, (int)h->lx, (int)h->ly, (int)h->lz);
  return MLBM_OK;
}

extern "C" int mlbm_get_spectral_diagnostics(mlbm_handle* h, double* vorticity, double* energy,
                                             double* enstrophy, double* spectrum, int layout) {
  if (!h) return MLBM_ERR_INVALID;
  if (!valid_layout(layout)) return fail(h, MLBM_ERR_INVALID, "bad layout");
  if (!h->fields_valid) return fail(h, MLBM_ERR_STATE, "no stored fields (use MLBM_STEP_STORE_FIELDS)");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  char msg[256] = {0};
  if (!h->sdiag && spectral_diag_create(&h->sdiag, h->D, (int)h->lx, (int)h->ly, (int)h->lz,
                                        h->stream, msg, sizeof msg))
    return fail(h, MLBM_ERR_CUDA, "spectral analyses: %s", msg);
  if (spectral_diag_run(h->sdiag, h->rho, h->u, h->stream, msg, sizeof msg))
    return fail(h, MLBM_ERR_CUDA, "spectral analyses: %s", msg);
  const int ncomp = 2 * h->D - 3;  // 1 vorticity component in 2-D, 3 in 3-D
  const long long stride = layout == MLBM_LAYOUT_DENSE ? h->V : ref_layout(h).volume;
  int rc;
  for (int c = 0; c < ncomp; ++c) {
    if (spectral_diag_curl(h->sdiag, c, h->stream, msg, sizeof msg))
      return fail(h, MLBM_ERR_CUDA, "spectral analyses: %s", msg);
    if (vorticity && (rc = download(h, spectral_diag_vorticity(h->sdiag), vorticity + c * stride, 1,
                                    layout)))
      return rc;
  }
  const int ns = spectral_diag_nshells(h->sdiag);
  std::vector<double> res((size_t)(2 + ns));
  MLBM_CUDA(h, cudaMemcpyAsync(res.data(), spectral_diag_results(h->sdiag),
                               sizeof(double) * res.size(), cudaMemcpyDeviceToHost, h->stream));
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  if (energy) *energy = res[0];
  if (enstrophy) *enstrophy = res[1];
  if (spectrum) std::memcpy(spectrum, res.data() + 2, sizeof(double) * ns);
  return MLBM_OK;
}

extern "C" int mlbm_get_diagnostics(mlbm_handle* h, mlbm_diag* out) {
  if (!h || !out) return MLBM_ERR_INVALID;
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  std::memset(out, 0, sizeof *out);
  out->step = h->steps;
  double d[DIAG_FIELDS] = {0, 0, 0, 0, 0};
  if (h->diag_valid) MLBM_CUDA(h, cudaMemcpy(d, h->diag_dev, sizeof d, cudaMemcpyDeviceToHost));
  unsigned long long c[CNT_COUNT];
  MLBM_CUDA(h, cudaMemcpy(c, h->counters, sizeof c, cudaMemcpyDeviceToHost));
  unsigned err = 0;
  MLBM_CUDA(h, cudaMemcpy(&err, h->err_word, sizeof err, cudaMemcpyDeviceToHost));
  out->mass = d[0];
  out->energy = d[1] / (double)h->V;  // AnalysisScalar::normalize, Analysis.h:29
  out->max_mach = d[2];
  out->alpha_min = d[3];
  out->alpha_max = d[4];
  out->solved_nodes = (long long)c[CNT_SOLVED];
  out->newton_iterations = (long long)c[CNT_ITER];
  out->guess_hits = (long long)c[CNT_HITS];
  out->bisection_nodes = (long long)c[CNT_BISECT];
  out->fallback_nodes = (long long)c[CNT_FALLBACK];
  out->limited_nodes = (long long)c[CNT_LIMITED];
  out->shortcut_nodes = (long long)c[CNT_SHORTCUT];
  out->series_nodes = (long long)c[CNT_SERIES];
  out->learned_nodes = (long long)c[CNT_INFER];
  out->error_word = err;
  return MLBM_OK;
}

extern "C" int mlbm_get_alpha(mlbm_handle* h, double* alpha, int layout) {
  if (!h) return MLBM_ERR_INVALID;
  if (!alpha || !valid_layout(layout)) return fail(h, MLBM_ERR_INVALID, "bad arguments");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  if (h->alpha) return download(h, h->alpha, alpha, 1, layout);
  std::vector<float> a((size_t)h->V);
  std::vector<double> ad((size_t)h->V);
  MLBM_CUDA(h, cudaMemcpy(a.data(), h->alpha32, sizeof(float) * h->V, cudaMemcpyDeviceToHost));
  for (long long i = 0; i < h->V; ++i) ad[i] = 2.0 + (double)a[i];
  if (layout == MLBM_LAYOUT_DENSE) std::memcpy(alpha, ad.data(), sizeof(double) * h->V);
  else ref_from_dense(h, ad.data(), alpha, 1);
  return MLBM_OK;
}

extern "C" int mlbm_set_alpha(mlbm_handle* h, const double* alpha, int layout) {
  if (!h) return MLBM_ERR_INVALID;
  if (!alpha || !valid_layout(layout)) return fail(h, MLBM_ERR_INVALID, "bad arguments");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->alpha_cold = true;  // it may hold alpha = 2
  if (h->alpha) return upload(h, alpha, h->alpha, 1, layout);
  std::vector<double> ad((size_t)h->V);
  if (layout == MLBM_LAYOUT_DENSE) std::memcpy(ad.data(), alpha, sizeof(double) * h->V);
  else dense_from_ref(h, alpha, ad.data(), 1);
  std::vector<float> a((size_t)h->V);
  for (long long i = 0; i < h->V; ++i) a[i] = (float)(ad[i] - 2.0);  // the device keeps alpha - 2
  MLBM_CUDA(h, cudaMemcpy(h->alpha32, a.data(), sizeof(float) * h->V, cudaMemcpyHostToDevice));
  return MLBM_OK;
}

extern "C" int mlbm_get_stream(mlbm_handle* h, void** stream) {
  if (!h || !stream) return MLBM_ERR_INVALID;
  *stream = (void*)h->stream;
  return MLBM_OK;
}

extern "C" int mlbm_set_stream(mlbm_handle* h, void* stream) {
  if (!h) return MLBM_ERR_INVALID;
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return MLBM_OK;
}

extern "C" int mlbm_set_sample_nodes(mlbm_handle* h, const long long* nodes, long long n) {
  if (!h) return MLBM_ERR_INVALID;
  if (n < 0 || (n > 0 && !nodes)) return fail(h, MLBM_ERR_INVALID, "bad sample list");
  for (long long i = 0; i < n; ++i)
    if (nodes[i] < 0 || nodes[i] >= h->V) return fail(h, MLBM_ERR_INVALID, "sample node %lld out of range", nodes[i]);
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  void* ptrs[] = {h->sample_nodes, h->sample_feat, h->sample_alpha, h->sample_solved};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  h->sample_nodes = nullptr; h->sample_feat = nullptr; h->sample_alpha = nullptr; h->sample_solved = nullptr;
  h->n_samples = 0;
  if (n == 0) return MLBM_OK;
  int rc;
  if ((rc = device_alloc(h, (void**)&h->sample_nodes, sizeof(long long) * n)) ||
      (rc = device_alloc(h, (void**)&h->sample_feat, sizeof(double) * n * h->Q)) ||
      (rc = device_alloc(h, (void**)&h->sample_alpha, sizeof(double) * n)) ||
      (rc = device_alloc(h, (void**)&h->sample_solved, sizeof(int) * n)))
    return rc;
  MLBM_CUDA(h, cudaMemcpy(h->sample_nodes, nodes, sizeof(long long) * n, cudaMemcpyHostToDevice));
  h->n_samples = n;
  return MLBM_OK;
}

extern "C" int mlbm_get_samples(mlbm_handle* h, double* features, double* alpha, int* solved) {
  if (!h) return MLBM_ERR_INVALID;
  if (h->n_samples == 0) return fail(h, MLBM_ERR_STATE, "no sample nodes");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  if (features)
    MLBM_CUDA(h, cudaMemcpy(features, h->sample_feat, sizeof(double) * h->n_samples * h->Q, cudaMemcpyDeviceToHost));
  if (alpha)
    MLBM_CUDA(h, cudaMemcpy(alpha, h->sample_alpha, sizeof(double) * h->n_samples, cudaMemcpyDeviceToHost));
  if (solved)
    MLBM_CUDA(h, cudaMemcpy(solved, h->sample_solved, sizeof(int) * h->n_samples, cudaMemcpyDeviceToHost));
  return MLBM_OK;
}

// Host model -> device inference layout (BF16 weights, zero-padded inputs).
static int upload_model(mlbm_handle* h, const mlbm_mlp* m, MlpDev* dst, bool any_q = false) {
  const bool q_ok = any_q ? (m->n_in == 9 || m->n_in == 19 || m->n_in == 27) : m->n_in == h->Q;
  if (!q_ok || m->n_hidden != MLBM_MLP_HIDDEN)
    return fail(h, MLBM_ERR_INVALID, "model shape %d->%d does not match Q=%d, hidden=%d", m->n_in,
                m->n_hidden, h->Q, MLBM_MLP_HIDDEN);
  MlpDev d;
  std::memset(&d, 0, sizeof d);
  for (int j = 0; j < MLP_H; ++j) {
    for (int i = 0; i < 32; ++i)
      d.w1[j * 32 + i] = __float2bfloat16(i < m->n_in ? m->w1[j * m->n_in + i] : 0.0f);
    for (int i = 0; i < MLP_H; ++i) d.w2[j * MLP_H + i] = __float2bfloat16(m->w2[j * MLP_H + i]);
    d.b1[j] = m->b1[j];
    d.b2[j] = m->b2[j];
    d.w3[j] = m->w3[j];
  }
  for (int i = 0; i < 32; ++i) d.in_scale[i] = i < m->n_in ? m->input_scale[i] : 0.0f;
  d.b3 = m->b3;
  d.out_scale = m->output_scale;
  d.n_in = m->n_in;
  MLBM_CUDA(h, cudaMemcpy(dst, &d, sizeof d, cudaMemcpyHostToDevice));
  return MLBM_OK;
}

extern "C" int mlbm_set_alpha_model(mlbm_handle* h, const mlbm_mlp* m) {
  if (!h || !m) return MLBM_ERR_INVALID;
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  MLBM_CUDA(h, cudaStreamSynchronize(h->stream));
  int rc = upload_model(h, m, h->mlp);
  if (rc) return rc;
  h->have_model = true;
  return MLBM_OK;
}

extern "C" int mlbm_alpha_model_predict(mlbm_handle* h, const mlbm_mlp* m, const float* X, long long n,
                                        float* alpha) {
  if (!h || !m || !X || !alpha || n <= 0) return MLBM_ERR_INVALID;
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  MlpDev* dm = nullptr;
  float *dX = nullptr, *dA = nullptr;
  int rc;
  if ((rc = device_alloc(h, (void**)&dm, sizeof(MlpDev)))) return rc;
  if ((rc = device_alloc(h, (void**)&dX, sizeof(float) * n * m->n_in)) ||
      (rc = device_alloc(h, (void**)&dA, sizeof(float) * n))) {
    cudaFree(dm); cudaFree(dX);
    return rc;
  }
  rc = upload_model(h, m, dm, true);
  if (!rc) {
    cudaMemcpy(dX, X, sizeof(float) * n * m->n_in, cudaMemcpyHostToDevice);
    cudaError_t e = mlp_predict(dm, m->n_in, dX, n, dA, h->stream);
    count_launches(1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) e = cudaMemcpy(alpha, dA, sizeof(float) * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = fail(h, MLBM_ERR_CUDA, "predict: %s", cudaGetErrorString(e));
  }
  cudaFree(dm); cudaFree(dX); cudaFree(dA);
  return rc;
}

extern "C" int mlbm_alpha_model_gradient(mlbm_handle* h, const mlbm_mlp* m, const float* X,
                                         const float* y, long long n, float* loss, mlbm_mlp* grad) {
  if (!h || !m || !X || !y || !loss || !grad || n <= 0) return MLBM_ERR_INVALID;
  if (m->n_in < 1 || m->n_in > MLBM_MLP_MAX_IN || m->n_hidden != MLBM_MLP_HIDDEN)
    return fail(h, MLBM_ERR_INVALID, "bad model shape");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  MlpTrainer tr;
  cudaError_t e = tr.init(m->n_in, n, h->stream);
  if (e == cudaSuccess) e = tr.set_data(X, y, n);
  if (e == cudaSuccess) e = tr.set_model(*m);
  float l = 0.0f;
  if (e == cudaSuccess) e = tr.gradient(n, &l);
  if (e == cudaSuccess) e = tr.get_gradient(grad);
  count_launches(tr.launches);
  tr.release();
  if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "gradient: %s", cudaGetErrorString(e));
  *loss = l;
  return MLBM_OK;
}

extern "C" int mlbm_train_alpha_model(mlbm_handle* h, const float* X, const float* y, long long n,
                                      mlbm_train_cfg* cfg, mlbm_mlp* m) {
  if (!h || !X || !y || !cfg || !m || n <= 0) return MLBM_ERR_INVALID;
  if (m->n_in < 1 || m->n_in > MLBM_MLP_MAX_IN || m->n_hidden != MLBM_MLP_HIDDEN)
    return fail(h, MLBM_ERR_INVALID, "bad model shape");
  if (cfg->epochs < 1 || cfg->batch < 1) return fail(h, MLBM_ERR_INVALID, "bad training configuration");
  MLBM_CUDA(h, cudaSetDevice(h->cfg.device));
  MlpTrainer tr;
  cudaError_t e = tr.init(m->n_in, cfg->batch, h->stream);
  if (e == cudaSuccess) e = tr.set_data(X, y, n);
  if (e == cudaSuccess) e = tr.set_model(*m);
  float last = 0.0f;
  if (e == cudaSuccess) e = tr.train(*cfg, &last);
  if (e == cudaSuccess) e = tr.get_model(m);
  count_launches(tr.launches);
  tr.release();
  if (e != cudaSuccess) return fail(h, MLBM_ERR_CUDA, "training: %s", cudaGetErrorString(e));
  cfg->final_loss = last;
  return MLBM_OK;
}

extern "C" const char* mlbm_last_error(const mlbm_handle* h) {
  if (h) return h->error.c_str();
  std::lock_guard<std::mutex> lk(g_create_error_mutex);
  static thread_local std::string copy;
  copy = g_create_error;
  return copy.c_str();
}

extern "C" unsigned long long mlbm_kernel_launch_count(void) {
  return g_launches.load(std::memory_order_relaxed);
}

extern "C" int mlbm_testing_fast_log(const double* x, double* out, long long n) {
  if (!x || !out || n <= 0) return MLBM_ERR_INVALID;
  LogEntry tab[LOG_TABLE];
  make_log_table(tab);
  void *dx = nullptr, *dout = nullptr, *dtab = nullptr;
  if (cudaMalloc(&dx, sizeof(double) * n) != cudaSuccess ||
      cudaMalloc(&dout, sizeof(double) * n) != cudaSuccess ||
      cudaMalloc(&dtab, sizeof tab) != cudaSuccess) {
    cudaFree(dx); cudaFree(dout); cudaFree(dtab);
    cudaGetLastError();
    return fail(nullptr, MLBM_ERR_ALLOC, "testing buffers");
  }
  cudaError_t e = cudaMemcpy(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dtab, tab, sizeof tab, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = fast_log_eval((const double*)dx, (double*)dout, n, dtab, 0);
  count_launches(1);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost);
  cudaFree(dx); cudaFree(dout); cudaFree(dtab);
  if (e != cudaSuccess) return fail(nullptr, MLBM_ERR_CUDA, "fast log: %s", cudaGetErrorString(e));
  return MLBM_OK;
}

extern "C" int mlbm_testing_entropy(int lattice, const float* f, const double* fneq,
                                    long long nodes, const double* x, int nx, int mode,
                                    double* F, double* D, int* series) {
  if (lattice < 0 || lattice > 2 || !f || !fneq || !x || !F || !D || !series || nodes <= 0 ||
      nx <= 0 || mode < 0 || mode > 2)
    return MLBM_ERR_INVALID;
  const int Q = lattice == 0 ? 9 : (lattice == 1 ? 19 : 27);
  LogEntry tab[LOG_TABLE];
  make_log_table(tab);
  std::unique_ptr<FineTable> fine(new FineTable);
  make_log_table_fine(fine.get(), lattice);
  const size_t nf = sizeof(float) * Q * nodes, nn = sizeof(double) * Q * nodes,
               nxb = sizeof(double) * nx, no = sizeof(double) * nx * nodes,
               ns = sizeof(int) * nodes;
  void *df = nullptr, *dn = nullptr, *dx = nullptr, *dF = nullptr, *dD = nullptr,
       *dS = nullptr, *dt = nullptr, *dtf = nullptr;
  auto release = [&]() {
    cudaFree(df); cudaFree(dn); cudaFree(dx); cudaFree(dF); cudaFree(dD); cudaFree(dS);
    cudaFree(dt); cudaFree(dtf);
  };
  if (cudaMalloc(&df, nf) != cudaSuccess || cudaMalloc(&dn, nn) != cudaSuccess ||
      cudaMalloc(&dx, nxb) != cudaSuccess || cudaMalloc(&dF, no) != cudaSuccess ||
      cudaMalloc(&dD, no) != cudaSuccess || cudaMalloc(&dS, ns) != cudaSuccess ||
      cudaMalloc(&dt, sizeof tab) != cudaSuccess || cudaMalloc(&dtf, sizeof(FineTable)) != cudaSuccess) {
    release();
    cudaGetLastError();
    return fail(nullptr, MLBM_ERR_ALLOC, "testing buffers");
  }
  cudaError_t e = cudaMemcpy(df, f, nf, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dn, fneq, nn, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, nxb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dt, tab, sizeof tab, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dtf, fine.get(), sizeof(FineTable), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = entropy_test(lattice, (const float*)df, (const double*)dn, nodes, (const double*)dx, nx,
                     mode, dt, dtf, (double*)dF, (double*)dD, (int*)dS, 0);
  count_launches(1);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(F, dF, no, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(D, dD, no, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(series, dS, ns, cudaMemcpyDeviceToHost);
  release();
  if (e != cudaSuccess) return fail(nullptr, MLBM_ERR_CUDA, "entropy test: %s", cudaGetErrorString(e));
  return MLBM_OK;
}

extern "C" int mlbm_testing_alpha_solve(int lattice, double tol, int newton_maxit,
                                        int bisect_maxit, long long n, const double* f,
                                        const double* fneq, const double* guess, double* alpha,
                                        int* flags) {
  if (lattice < 0 || lattice > MLBM_D3Q33 || !f || !fneq || !guess || !alpha || !flags ||
      n <= 0 || newton_maxit < 0 || bisect_maxit < 0 || !(tol >= 0))
    return MLBM_ERR_INVALID;
  const int Q = kQ[lattice];
  LogEntry tab[LOG_TABLE];
  make_log_table(tab);
  const size_t nq = sizeof(double) * Q * n, n8 = sizeof(double) * n, n4 = sizeof(int) * n;
  void *df = nullptr, *dn = nullptr, *dg = nullptr, *da = nullptr, *dfl = nullptr, *dt = nullptr;
  auto release = [&]() {
    cudaFree(df); cudaFree(dn); cudaFree(dg); cudaFree(da); cudaFree(dfl); cudaFree(dt);
  };
  if (cudaMalloc(&df, nq) != cudaSuccess || cudaMalloc(&dn, nq) != cudaSuccess ||
      cudaMalloc(&dg, n8) != cudaSuccess || cudaMalloc(&da, n8) != cudaSuccess ||
      cudaMalloc(&dfl, n4) != cudaSuccess || cudaMalloc(&dt, sizeof tab) != cudaSuccess) {
    release();
    cudaGetLastError();
    return fail(nullptr, MLBM_ERR_ALLOC, "testing buffers");
  }
  StepParams p{};
  p.alpha_mode = ALPHA_RESIDUAL;
  p.guess_mode = GUESS_PREVIOUS;
  p.newton_tol = tol;
  p.newton_maxit = newton_maxit;
  p.bisect_maxit = bisect_maxit;
  p.deviation_threshold = 0.0;
  p.log_table = dt;
  cudaError_t e = cudaMemcpy(df, f, nq, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dn, fneq, nq, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dg, guess, n8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dt, tab, sizeof tab, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = alpha_solve_test(lattice, (const double*)df, (const double*)dn, (const double*)dg, n, p,
                         (double*)da, (int*)dfl, 0);
  count_launches(1);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(alpha, da, n8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(flags, dfl, n4, cudaMemcpyDeviceToHost);
  release();
  if (e != cudaSuccess) return fail(nullptr, MLBM_ERR_CUDA, "alpha solve test: %s", cudaGetErrorString(e));
  return MLBM_OK;
}

extern "C" int mlbm_testing_neq(int lattice, const float* f, long long nodes, int dfloat,
                                double* fneq) {
  if (lattice < 0 || lattice > 2 || !f || !fneq || nodes <= 0) return MLBM_ERR_INVALID;
  const int Q = lattice == 0 ? 9 : (lattice == 1 ? 19 : 27);
  void *df = nullptr, *dn = nullptr;
  if (cudaMalloc(&df, sizeof(float) * Q * nodes) != cudaSuccess ||
      cudaMalloc(&dn, sizeof(double) * Q * nodes) != cudaSuccess) {
    cudaFree(df); cudaFree(dn);
    cudaGetLastError();
    return fail(nullptr, MLBM_ERR_ALLOC, "testing buffers");
  }
  cudaError_t e = cudaMemcpy(df, f, sizeof(float) * Q * nodes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = neq_test(lattice, (const float*)df, nodes, dfloat, (double*)dn, 0);
  count_launches(1);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(fneq, dn, sizeof(double) * Q * nodes, cudaMemcpyDeviceToHost);
  cudaFree(df); cudaFree(dn);
  if (e != cudaSuccess) return fail(nullptr, MLBM_ERR_CUDA, "neq test: %s", cudaGetErrorString(e));
  return MLBM_OK;
}
