/* No-op stand-in for FFTW-MPI: plans do nothing (so the reference's
 * spectral curl/spectra are not computed), fftw_malloc is malloc, and
 * fftw_mpi_local_size returns the real FFTW r2c local size
 * prod(n[0..d-2]) * (n[d-1]/2+1), so the reference's padded field layout
 * (2*(N/2+1) in the last dimension) is reproduced exactly. */
#pragma once
#include <cstddef>
#include <cstdlib>
typedef double fftw_complex[2];
typedef void* fftw_plan;
#define FFTW_ESTIMATE 0
template <class... A> inline fftw_plan mlbm_fftw_noop(A...) { return nullptr; }
#define fftw_mpi_plan_dft_r2c mlbm_fftw_noop
#define fftw_mpi_plan_dft_c2r mlbm_fftw_noop
#define fftw_destroy_plan mlbm_fftw_noop
#define fftw_execute mlbm_fftw_noop
#define fftw_init_threads mlbm_fftw_noop
#define fftw_mpi_init mlbm_fftw_noop
#define fftw_plan_with_nthreads mlbm_fftw_noop
#define fftw_mpi_cleanup mlbm_fftw_noop
#define fftw_malloc malloc
#define fftw_free free
inline ptrdiff_t fftw_mpi_local_size(int d, const ptrdiff_t* n, int, ptrdiff_t* local_n0,
                                     ptrdiff_t* local_0_start) {
  ptrdiff_t v = 1;
  for (int i = 0; i < d - 1; ++i) v *= n[i];
  v *= n[d - 1] / 2 + 1;
  *local_n0 = n[0];
  *local_0_start = 0;
  return v;
}
