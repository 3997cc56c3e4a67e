/* Stand-in for FFTW-MPI on one rank, for building the reference as a test
 * oracle (TEST INFRASTRUCTURE ONLY; FFTW is not in the image).
 *
 * The r2c / c2r plans are real discrete Fourier transforms with FFTW's
 * documented conventions for the MPI interface on one process:
 *   - real arrays are row-major with the last dimension padded to
 *     2 (n_last / 2 + 1) doubles; complex arrays are row-major with the last
 *     dimension n_last / 2 + 1 (non-transposed output);
 *   - r2c computes X[k] = sum_x x[x] exp(-2 pi i k.x / n) (unnormalised);
 *   - c2r computes x[x] = sum_k X[k] exp(+2 pi i k.x / n) over the full
 *     spectrum, the missing half being the Hermitian completion, i.e.
 *     Re(sum over the stored half with weight 2 for 0 < k_last < n_last / 2);
 *   - in-place plans (in == out) are allowed.
 * They are evaluated as direct sums (O(N^2), for the small golden grids),
 * with the exponentials taken in long double, so they agree with FFTW's
 * results to rounding. fftw_mpi_local_size returns the real FFTW r2c local
 * size prod(n[0..d-2]) * (n[d-1]/2+1), so the reference's padded field
 * layout is reproduced exactly; the thread and MPI set-up calls do nothing. */
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <vector>

typedef double fftw_complex[2];
#define FFTW_ESTIMATE 0

struct mlbm_fftw_plan_s {
  int rank;
  long n[3];
  bool r2c;
  double* real;
  fftw_complex* cplx;
};
typedef mlbm_fftw_plan_s* fftw_plan;

template <class... A> inline void mlbm_fftw_noop(A...) {}
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

inline fftw_plan mlbm_fftw_make(int rank, const ptrdiff_t* n, bool r2c, double* real,
                                fftw_complex* cplx) {
  fftw_plan p = new mlbm_fftw_plan_s;
  p->rank = rank;
  for (int i = 0; i < 3; ++i) p->n[i] = i < rank ? (long)n[i] : 1;
  p->r2c = r2c;
  p->real = real;
  p->cplx = cplx;
  return p;
}

template <class Comm>
inline fftw_plan fftw_mpi_plan_dft_r2c(int rank, const ptrdiff_t* n, double* in,
                                       fftw_complex* out, Comm, unsigned) {
  return mlbm_fftw_make(rank, n, true, in, out);
}

template <class Comm>
inline fftw_plan fftw_mpi_plan_dft_c2r(int rank, const ptrdiff_t* n, fftw_complex* in,
                                       double* out, Comm, unsigned) {
  return mlbm_fftw_make(rank, n, false, out, in);
}

inline void fftw_destroy_plan(fftw_plan p) { delete p; }

// exp(sign 2 pi i j / n) in long double, j reduced modulo n first
inline void mlbm_fftw_twiddle(long j, long n, int sign, long double& c, long double& s) {
  const long double two_pi = 6.283185307179586476925286766559005768L;
  const long double a = two_pi * (long double)(j % n) / (long double)n;
  c = std::cos(a);
  s = sign * std::sin(a);
}

inline void fftw_execute(const fftw_plan p) {
  // the lattice as n0 x n1 x n2 with the halved axis last (rank 2: n2 = 1 is
  // a dummy leading axis, so map (n0, n1) -> (1, n0, n1))
  long A = p->n[0], B = p->n[1], C = p->n[2];
  if (p->rank == 2) { A = 1; B = p->n[0]; C = p->n[1]; }
  const long H = C / 2 + 1, P = 2 * H;  // complex / padded real last extents
  std::vector<long double> out;
  if (p->r2c) {
    out.assign((size_t)(A * B * H * 2), 0.0L);
    for (long ka = 0; ka < A; ++ka)
      for (long kb = 0; kb < B; ++kb)
        for (long kc = 0; kc < H; ++kc) {
          long double re = 0.0L, im = 0.0L;
          for (long a = 0; a < A; ++a)
            for (long b = 0; b < B; ++b)
              for (long c = 0; c < C; ++c) {
                long double tc, ts;
                mlbm_fftw_twiddle(ka * a * B * C + kb * b * C * A + kc * c * A * B, A * B * C, -1,
                                  tc, ts);
                const long double x = p->real[(a * B + b) * P + c];
                re += x * tc;
                im += x * ts;
              }
          const size_t k = (size_t)((ka * B + kb) * H + kc);
          out[2 * k] = re;
          out[2 * k + 1] = im;
        }
    for (size_t k = 0; k < out.size() / 2; ++k) {
      p->cplx[k][0] = (double)out[2 * k];
      p->cplx[k][1] = (double)out[2 * k + 1];
    }
  } else {
    out.assign((size_t)(A * B * C), 0.0L);
    for (long a = 0; a < A; ++a)
      for (long b = 0; b < B; ++b)
        for (long c = 0; c < C; ++c) {
          long double v = 0.0L;
          for (long ka = 0; ka < A; ++ka)
            for (long kb = 0; kb < B; ++kb)
              for (long kc = 0; kc < H; ++kc) {
                const long double w = (kc == 0 || 2 * kc == C) ? 1.0L : 2.0L;
                long double tc, ts;
                mlbm_fftw_twiddle(ka * a * B * C + kb * b * C * A + kc * c * A * B, A * B * C, +1,
                                  tc, ts);
                const fftw_complex& X = p->cplx[(ka * B + kb) * H + kc];
                v += w * ((long double)X[0] * tc - (long double)X[1] * ts);
              }
          out[(size_t)((a * B + b) * C + c)] = v;
        }
    for (long a = 0; a < A; ++a)
      for (long b = 0; b < B; ++b)
        for (long c = 0; c < C; ++c)
          p->real[(a * B + b) * P + c] = (double)out[(size_t)((a * B + b) * C + c)];
  }
}
