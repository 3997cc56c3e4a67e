// Algorithm_gpu.h - C++ drop-in for metaLBM's Algorithm on the mlbm C ABI.
//
// metaLBM's Routine drives its hot path through
//   Algorithm<T, Pull, arch, SoA, OneD, MPI, Off>   (include/metaLBM/Algorithm.h:317-363)
// with  iterate(iteration, streams..., events...)  (Algorithm.h:326-358),
//       pack(stream) / unpack(stream)               (Algorithm.h:132-147),
//       isStored                                    (Algorithm.h:67),
//       getComputationTime / getCommunicationTime   (Algorithm.h:128-130).
// mlbm::AlgorithmGPU keeps that surface; the lattice lives on the GPU behind
// an mlbm_handle, and pack/unpack/storeFields move data between the device
// and the caller's arrays in the reference's padded local layout
// (FieldList / Distribution::getData(numberElements), Field.h:122-125).
//
// Header-only; link with -lmlbm (metalbm_gb300/libmlbm.so). Errors throw
// mlbm::Error (the reference exits the process instead, Commons.h:6-38).
#ifndef MLBM_ALGORITHM_GPU_H
#define MLBM_ALGORITHM_GPU_H

#include <chrono>
#include <stdexcept>
#include <string>

#include "mlbm.h"

namespace mlbm {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, const mlbm_handle* h) {
  if (rc != MLBM_OK) throw Error(rc, mlbm_last_error(h));
}

class AlgorithmGPU {
 public:
  // Replaces the Algorithm constructor (Algorithm.h:317-324) together with the
  // construction of Distribution and FieldList storage.
  explicit AlgorithmGPU(const mlbm_config& cfg) : h_(nullptr), isStored(false), dtComputation_(0.0) {
    check(mlbm_create(&cfg, &h_), nullptr);
  }
  AlgorithmGPU(const AlgorithmGPU&) = delete;
  AlgorithmGPU& operator=(const AlgorithmGPU&) = delete;
  ~AlgorithmGPU() {
    if (h_) mlbm_destroy(h_);
  }

  // initDistribution (Initialize.h:91-116) + unpack: f = f_eq(rho, u).
  // rho: density field data, u: velocity field data (component stride =
  // numberElements), both in the reference's padded layout.
  void initialize(const double* densityPtr, const double* velocityPtr) {
    check(mlbm_init_equilibrium(h_, densityPtr, velocityPtr, MLBM_LAYOUT_REFERENCE), h_);
  }

  // Algorithm::unpack: local distribution array (Q components, stride
  // numberElements) -> device.
  void unpack(const double* distributionPtr) {
    check(mlbm_set_populations(h_, distributionPtr, MLBM_LAYOUT_REFERENCE), h_);
  }

  // Algorithm::pack: device -> local distribution array.
  void pack(double* distributionPtr) {
    check(mlbm_get_populations(h_, distributionPtr, MLBM_LAYOUT_REFERENCE), h_);
  }

  // Algorithm::iterate: one fused pull step; when isStored, the step stores
  // rho, the hydrodynamic velocity, alpha and F (Algorithm.h:150-194). The
  // wait for the device is bounded by syncTimeoutMs: past it, mlbm::Error with
  // code MLBM_ERR_TIMEOUT (the handle stays usable; the step still completes).
  void iterate(unsigned int /*iteration*/) {
    const auto t0 = std::chrono::steady_clock::now();
    check(mlbm_step(h_, 1, isStored ? MLBM_STEP_STORE_FIELDS : 0u), h_);
    check(mlbm_sync(h_, syncTimeoutMs), h_);
    dtComputation_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  // The reference's signature, so that Routine::compute's call site
  // (Routine.h:126) compiles unchanged: iterate(iteration, defaultStream,
  // bulkStream, leftStream, rightStream, leftEvent, rightEvent)
  // (Algorithm.h:326-358). The streams and events order the reference's
  // halo exchange against its bulk sweep; the periodic wrap is inside the
  // kernel here, so they are not used and the step runs on the handle's
  // stream.
  template <class StreamT, class EventT>
  void iterate(unsigned int iteration, StreamT& /*defaultStream*/, StreamT& /*bulkStream*/,
               StreamT& /*leftStream*/, StreamT& /*rightStream*/, EventT& /*leftEvent*/,
               EventT& /*rightEvent*/) {
    iterate(iteration);
  }

  // The stored fields of the last isStored step into FieldList arrays
  // (reference layout; any pointer may be null).
  void storeFields(double* densityPtr, double* velocityPtr, double* alphaPtr, double* forcePtr) {
    check(mlbm_get_fields(h_, densityPtr, velocityPtr, alphaPtr, forcePtr, MLBM_LAYOUT_REFERENCE), h_);
  }

  // The Routine's spectral analyses of the last stored fields
  // (Routine.h:69-72, 126-131; AnalysisList.h:55-73, 135-171): vorticity into
  // the FieldList's vorticity array (reference layout), total energy and
  // enstrophy, and the shell energy spectrum (spectraSize() values); any
  // pointer may be null.
  void analyses(double* vorticityPtr, double* totalEnergy, double* totalEnstrophy,
                double* energySpectra) {
    check(mlbm_get_spectral_diagnostics(h_, vorticityPtr, totalEnergy, totalEnstrophy,
                                        energySpectra, MLBM_LAYOUT_REFERENCE),
          h_);
  }
  int spectraSize() const {
    int n = 0;
    check(mlbm_spectrum_shells(h_, &n), h_);
    return n;
  }

  mlbm_diag diagnostics() {
    mlbm_diag d;
    check(mlbm_get_diagnostics(h_, &d), h_);
    return d;
  }

  double getComputationTime() const { return dtComputation_; }
  double getCommunicationTime() const { return 0.0; }  // periodic wrap is in-kernel

  mlbm_handle* handle() { return h_; }

 private:
  mlbm_handle* h_;

 public:
  bool isStored;
  // Limit of each wait for the device in iterate, milliseconds (< 0: none).
  int syncTimeoutMs = 600000;

 private:
  double dtComputation_;
};

}  // namespace mlbm

#endif  // MLBM_ALGORITHM_GPU_H
