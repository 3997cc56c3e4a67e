// Routine-shaped C++ host loop on mlbm::AlgorithmGPU (include/mlbm/Algorithm_gpu.h).
//
// The same driving sequence as metaLBM's Routine::compute (Routine.h:90-153)
// with the GPU Algorithm dropped in: initial density and velocity in the
// reference's padded FieldList layout, f = f_eq(rho, u), `steps` iterations
// with isStored on the last one, then pack and storeFields.
//
// Usage: routine_gpu <in.bin> <out.bin> <steps> <lattice 0..5> <collision 0..7>
//                    <forcing 0..3> <force 0..3> <tau> <ax> <ay> <az> <lx> <ly> <lz>
//                    <Lx> <Ly> <Lz> [<sync timeout ms> [<alpha solver 0..1>]]
//   in.bin : float64 rho[V], u[D][V] dense (index (x*Ly+y)*Lz+z)
//   out.bin: float64 f[Q][V], rho[V], u[D][V], alpha[V], force[D][V], seconds
//   out.bin.analysis: float64 vorticity[2D-3][V], energy, enstrophy, K, spectrum[K]
//            (the Routine's analyses of the stored fields, Routine.h:126-131)
// Exit status: 0 done, 5 an mlbm error, 6 a wait for the device timed out.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "mlbm/Algorithm_gpu.h"

int main(int argc, char** argv) {
  if (argc < 18 || argc > 20) {
    std::fprintf(stderr, "usage: see the header of routine_gpu.cpp\n");
    return 2;
  }
  mlbm_config cfg;
  mlbm_config_init(&cfg);
  const int steps = std::atoi(argv[3]);
  cfg.lattice = std::atoi(argv[4]);
  cfg.collision = std::atoi(argv[5]);
  cfg.forcing_scheme = std::atoi(argv[6]);
  cfg.force = std::atoi(argv[7]);
  cfg.relaxation_time = std::atof(argv[8]);
  for (int d = 0; d < 3; ++d) {
    cfg.force_amplitude[d] = std::atof(argv[9 + d]);
    cfg.force_wavelength[d] = std::atof(argv[12 + d]);
    cfg.length[d] = std::atoi(argv[15 + d]);
  }
  const int timeout_ms = argc > 18 ? std::atoi(argv[18]) : 600000;
  if (argc > 19) {  // the bracketed residual solver at 1e-12 instead of the reference's
    cfg.alpha_mode = std::atoi(argv[19]);
    if (cfg.alpha_mode == MLBM_ALPHA_RESIDUAL) {
      cfg.newton_tolerance = 1e-12;
      cfg.deviation_threshold = 0.0;
    }
  }
  if (cfg.lattice < MLBM_D2Q9 || cfg.lattice > MLBM_D3Q33) {
    std::fprintf(stderr, "bad lattice %d\n", cfg.lattice);
    return 2;
  }
  static const int kQ[6] = {9, 19, 27, 15, 13, 33};
  const int Q = kQ[cfg.lattice];
  const int D = (cfg.lattice == MLBM_D2Q9 || cfg.lattice == MLBM_D2Q13) ? 2 : 3;
  const long lx = cfg.length[0], ly = cfg.length[1], lz = D == 2 ? 1 : cfg.length[2];
  const long V = lx * ly * lz;
  // reference local layout: last active dimension padded to 2*(N/2+1)
  const long py = D == 2 ? 2 * (ly / 2 + 1) : ly, pz = D == 2 ? 1 : 2 * (lz / 2 + 1);
  const long n = lx * py * pz;  // numberElements
  auto ref = [&](long x, long y, long z) { return (x * py + y) * pz + z; };
  auto dense = [&](long x, long y, long z) { return (x * ly + y) * lz + z; };

  std::vector<double> in((size_t)(1 + D) * V);
  FILE* fi = std::fopen(argv[1], "rb");
  if (!fi || std::fread(in.data(), sizeof(double), in.size(), fi) != in.size()) return 3;
  std::fclose(fi);
  std::vector<double> density(n, 0.0), velocity((size_t)D * n, 0.0);
  for (long x = 0; x < lx; ++x)
    for (long y = 0; y < ly; ++y)
      for (long z = 0; z < lz; ++z) {
        density[ref(x, y, z)] = in[dense(x, y, z)];
        for (int c = 0; c < D; ++c) velocity[c * n + ref(x, y, z)] = in[(1 + c) * V + dense(x, y, z)];
      }

  // Stand-ins for the reference's Stream<arch> / Event<arch> (Routine.h:35-42):
  // the drop-in's iterate takes them and does not use them.
  struct Stream {} defaultStream, bulkStream, leftStream, rightStream;
  struct Event {} leftEvent, rightEvent;
  try {
    mlbm::AlgorithmGPU algorithm(cfg);
    algorithm.syncTimeoutMs = timeout_ms;
    algorithm.initialize(density.data(), velocity.data());
    double seconds = 0.0;
    for (int it = 1; it <= steps; ++it) {
      algorithm.isStored = (it == steps);
      algorithm.iterate(it, defaultStream, bulkStream, leftStream, rightStream, leftEvent,
                        rightEvent);
      seconds += algorithm.getComputationTime();
    }
    std::vector<double> distribution((size_t)Q * n, 0.0), alpha(n), force((size_t)D * n);
    algorithm.pack(distribution.data());
    algorithm.storeFields(density.data(), velocity.data(), alpha.data(), force.data());

    std::vector<double> out((size_t)(Q + 1 + D + 1 + D) * V + 1);
    for (long x = 0; x < lx; ++x)
      for (long y = 0; y < ly; ++y)
        for (long z = 0; z < lz; ++z) {
          const long k = dense(x, y, z), r = ref(x, y, z);
          for (int q = 0; q < Q; ++q) out[q * V + k] = distribution[q * n + r];
          long o = (long)Q * V;
          out[o + k] = density[r];
          o += V;
          for (int c = 0; c < D; ++c) out[o + c * V + k] = velocity[c * n + r];
          o += (long)D * V;
          out[o + k] = alpha[r];
          o += V;
          for (int c = 0; c < D; ++c) out[o + c * V + k] = force[c * n + r];
        }
    out.back() = seconds;
    FILE* fo = std::fopen(argv[2], "wb");
    if (!fo || std::fwrite(out.data(), sizeof(double), out.size(), fo) != out.size()) return 4;
    std::fclose(fo);

    // the Routine's analyses after the stored step: vorticity into the
    // FieldList layout, energy, enstrophy and the shell spectrum
    const int DV = 2 * D - 3, K = algorithm.spectraSize();
    std::vector<double> vorticity((size_t)DV * n, 0.0), spectra((size_t)K);
    double energy = 0.0, enstrophy = 0.0;
    algorithm.analyses(vorticity.data(), &energy, &enstrophy, spectra.data());
    std::vector<double> an((size_t)DV * V + 3 + K);
    for (long x = 0; x < lx; ++x)
      for (long y = 0; y < ly; ++y)
        for (long z = 0; z < lz; ++z)
          for (int c = 0; c < DV; ++c) an[c * V + dense(x, y, z)] = vorticity[c * n + ref(x, y, z)];
    an[(size_t)DV * V] = energy;
    an[(size_t)DV * V + 1] = enstrophy;
    an[(size_t)DV * V + 2] = (double)K;
    for (int k = 0; k < K; ++k) an[(size_t)DV * V + 3 + k] = spectra[k];
    const std::string apath = std::string(argv[2]) + ".analysis";
    FILE* fa = std::fopen(apath.c_str(), "wb");
    if (!fa || std::fwrite(an.data(), sizeof(double), an.size(), fa) != an.size()) return 4;
    std::fclose(fa);
  } catch (const mlbm::Error& e) {
    std::fprintf(stderr, "mlbm error %d: %s\n", e.code, e.what());
    return e.code == MLBM_ERR_TIMEOUT ? 6 : 5;
  }
  return 0;
}
