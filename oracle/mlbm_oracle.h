/* CPU restatement of metaLBM's fused collide-and-stream pull step.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle the CUDA path is checked
 * against, and the "port" CPU baseline. Nothing in the product library links
 * it, calls it or falls back to it.
 *
 * Parity: pinned against the reference CPU build itself (oracle/_ref, built by
 * oracle/build_ref.py from the reference headers) through the golden vectors
 * in tests/golden/, bit-for-bit for BGK and reference-mode entropic runs.
 *
 * Layout: dense SoA, population q of node (x,y,z) at q*V + (x*ly + y)*lz + z,
 * i.e. the reference's node order (Domain.h:88-91, z fastest) without its
 * halo cells or FFTW padding. Periodic wrap is an index modulo.
 */
#ifndef MLBM_ORACLE_H
#define MLBM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_D2Q9 = 0, ORACLE_D3Q19 = 1, ORACLE_D3Q27 = 2, ORACLE_D3Q15 = 3, ORACLE_D2Q13 = 4,
       ORACLE_D3Q33 = 5 };
enum { ORACLE_BGK = 0, ORACLE_ELBM = 1 };
enum { ORACLE_FS_NONE = 0, ORACLE_FS_GUO = 1, ORACLE_FS_SHANCHEN = 2, ORACLE_FS_EDM = 3 };
/* ORACLE_F_FIELD: the per-node force is read from a D x V array set with
 * oracle_set_force_field (Force<Generic>::setForce, Force.h:36-45), the
 * mechanism of the reference's array forces (ConstantShell, EnergyRemoval,
 * Turbulent2D, Force.h:294-626). */
enum { ORACLE_F_NONE = 0, ORACLE_F_CONSTANT = 1, ORACLE_F_SINUSOIDAL = 2, ORACLE_F_KOLMOGOROV = 3,
       ORACLE_F_FIELD = 4 };
/* Entropic alpha solver.
 * REFERENCE: Collision.h:284-375 + EntropicStep.h:111-140 exactly: alpha = 2
 *   when every |f_neq|/f <= deviation_threshold; 0.95*alpha_max when
 *   alpha_max < 2; otherwise Newton from the guess until |step| <= tolerance,
 *   alpha = 2 when it fails or leaves (1, alpha_max).
 * RESIDUAL: the same shortcut and limiter, then the guess is accepted when the
 *   FP64 entropy residual |F(alpha)| <= tolerance; otherwise Newton from the
 *   guess until |F| <= tolerance; when Newton leaves (1, alpha_max) or runs out
 *   of iterations, the safeguarded bisection-Newton of EntropicStep.h:142-220
 *   on [1, alpha_max] with the same residual test; alpha = 2 if both fail.
 *   F(alpha) = sum f ln(f/w) - sum g ln(g/w), g = f - alpha f_neq
 *   (EntropicStep.h:31-45), evaluated as x B1 - sum f (1+t) log1p(t) with
 *   t = -alpha f_neq/f and B1 = sum f_neq ln(f/w) (the same function, formed
 *   from O(|f_neq|) terms; see mlbm_oracle.c). */
enum { ORACLE_ALPHA_REFERENCE = 0, ORACLE_ALPHA_RESIDUAL = 1 };
/* Starting guess: the node's alpha from the previous step (Algorithm.h:103-106)
 * or the constant 2. */
enum { ORACLE_GUESS_PREVIOUS = 0, ORACLE_GUESS_TWO = 1 };

typedef struct {
  int lattice, collision, forcing, force;
  double tau;
  double amplitude[3];
  double wavelength[3];
  /* Kolmogorov: the node coordinate the force depends on (the reference uses
   * y = 1, Force.h:262-267), and the component it drives (reference: x = 0). */
  int kolmogorov_axis, kolmogorov_component;
  int lx, ly, lz;
  int alpha_mode, guess_mode;
  double newton_tolerance;    /* reference: 1e-8 (Collision.h:336) */
  int newton_max_iterations;  /* reference: 50 (Collision.h:337) */
  double deviation_threshold; /* reference: 1e-3 (Collision.h:357) */
  int threads;                /* host threads sharing the sweep (>=1) */
  int bisection_max_iterations; /* RESIDUAL: cap of the bracketed solver (0: the Newton cap) */
  /* REFERENCE mode, sensitivity tests only: nonzero moves the libm logarithm
   * of the entropy function by one ulp on about half of its arguments. */
  int log_ulp_perturbation;
  /* BGK, sensitivity tests only: nonzero moves each new population by one
   * ulp, up or down, on about half of the stores. */
  int population_ulp_perturbation;
} oracle_config;

typedef struct oracle_state oracle_state;

oracle_state* oracle_create(const oracle_config* cfg);
void oracle_destroy(oracle_state* s);
/* f = f_eq(rho, u) (Initialize.h:91-116); alpha = 2 (Initialize.h:82-89). */
void oracle_init_equilibrium(oracle_state* s, const double* rho, const double* u);
void oracle_set_populations(oracle_state* s, const double* f);
void oracle_get_populations(const oracle_state* s, double* f);
/* Run nsteps pull steps; fields (rho, hydrodynamic u, alpha, force) are stored
 * on the last step when store_last != 0 (Algorithm.h:150-194). */
void oracle_step(oracle_state* s, int nsteps, int store_last);
void oracle_get_fields(const oracle_state* s, double* rho, double* u, double* alpha,
                       double* force);
/* Force field [D][V] (dense node order) read by ORACLE_F_FIELD; copied. */
void oracle_set_force_field(oracle_state* s, const double* force);
/* Sum of Newton iterations and count of alpha=2 fallbacks over the last step. */
void oracle_get_counters(const oracle_state* s, long long* newton_iterations,
                         long long* fallbacks, long long* bisections);

/* The residual mode's FP64 logarithm (Tang's table-driven method). */
double oracle_fast_log(double x);

/* Residual-mode alpha solve of n single nodes (f, f_neq: [n][Q]); see
 * mlbm_oracle.c. */
void oracle_solve_alpha_nodes(int lattice, double tol, int newton_maxit, int bisect_maxit, long n,
                              const double* f, const double* fneq, const double* guess,
                              double* alpha, int* flags);

/* Single-node entry points for unit tests: equilibrium population q. */
double oracle_equilibrium(int lattice, double rho, const double* u, int q);
int oracle_lattice_q(int lattice);
int oracle_lattice_d(int lattice);
void oracle_lattice_tables(int lattice, double* c /* [Q*3] */, double* w /* [Q] */);

#ifdef __cplusplus
}
#endif
#endif
