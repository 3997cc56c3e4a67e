/* mlbm_testing.h - test hooks of libmlbm (not part of the drop-in surface).
 *
 * No counterpart in the reference: these expose internal device functions so
 * their accuracy can be checked against the host's math library. */
#ifndef MLBM_TESTING_H
#define MLBM_TESTING_H

#ifdef __cplusplus
extern "C" {
#endif

/* out[i] = the library's FP64 natural logarithm (Tang's table-driven method,
 * used by the entropic kernels) of x[i] > 0, evaluated on the current device.
 * Host arrays; allocates temporary device buffers. */
int mlbm_testing_fast_log(const double* x, double* out, long long n);

/* The entropy-balance function F(x) and its derivative as the FP32-storage
 * entropic kernel evaluates them, for `nodes` nodes given as FP32 populations
 * f[nodes][Q] and FP64 non-equilibrium parts fneq[nodes][Q], at the nx points
 * x[]: F and D are [nodes][nx]; series[node] = 1 where the moment-series form
 * was used. mode 0 chooses the form as the kernel does (series when
 * max_q |f_neq/f| <= 0.0125), 1 forces the direct log1p form, 2 the series.
 * Host arrays; allocates temporary device buffers. */
int mlbm_testing_entropy(int lattice, const float* f, const double* fneq, long long nodes,
                         const double* x, int nx, int mode, double* F, double* D, int* series);

/* f_neq[nodes][Q] of nodes given as FP32 populations f[nodes][Q] (the stored
 * values of FP32 storage), formed as the FP32-storage entropic step forms it:
 * exact fixed-point density and momentum, then the TruncationMa3 equilibrium
 * in double-float arithmetic (dfloat = 1) or FP64 (dfloat = 0). Host arrays. */
int mlbm_testing_neq(int lattice, const float* f, long long nodes, int dfloat, double* fneq);

/* The FP64 entropic step's alpha for n single nodes given as pulled
 * populations f[n][Q] and non-equilibrium parts fneq[n][Q] (FP64): alpha_max
 * and the 0.95 alpha_max limiter (Collision.h:305-326, 362-367), then the
 * RESIDUAL solve from guess[n] (|F| <= tol; Newton capped at newton_maxit,
 * the bisection-Newton of EntropicStep.h:142-220 at bisect_maxit), with the
 * deviation shortcut off. flags[n]: 1 limited, 2 the bracketed solver ran,
 * 4 alpha = 2 fallback. Host arrays; allocates temporary device buffers. */
int mlbm_testing_alpha_solve(int lattice, double tol, int newton_maxit, int bisect_maxit,
                             long long n, const double* f, const double* fneq,
                             const double* guess, double* alpha, int* flags);

/* One step from the handle's current populations that leaves them current:
 * the step's output goes to the spare buffer, the step count does not move,
 * and the per-node alpha field holds the alpha this step solved for. A
 * following mlbm_step with the previous-alpha guess then starts every node
 * from its exact root: the perfect-guess bound of the alpha solve
 * (benchmarks). Enqueued on the handle's stream. */
int mlbm_testing_step_in_place(mlbm_handle* h);

#ifdef __cplusplus
}
#endif
#endif
