/* CPU restatement of metaLBM's fused collide-and-stream pull step.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA path is checked against and
 * the "port" CPU baseline. Parity of this file with the reference is pinned
 * bit-for-bit by tests/test_oracle_golden.py against vectors produced by the
 * reference itself (oracle/_ref, tests/golden/make_golden.py).
 *
 * Every floating-point expression below keeps the reference's operation order
 * (left-to-right C++ evaluation of the cited lines) and must be compiled with
 * -ffp-contract=off, so each multiply and add is rounded separately as in the
 * reference build.
 */
#include "mlbm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---- Lattice tables (Lattice.h:146-210, 214-288, 461-533, 536-612,
 * 615-703, 707-802) ----------------------------------------------------------
 * Velocity order: rest, the populations with c_x < 0, those with c_x > 0,
 * then c_x = 0, in the reference's order. Weights written as the reference's
 * (T)a/(T)b, or its decimal literals for D3Q33. */
static const int C_D2Q9[9][3] = {{0, 0, 0},  {-1, 1, 0}, {-1, 0, 0}, {-1, -1, 0}, {1, -1, 0},
                                 {1, 0, 0},  {1, 1, 0},  {0, -1, 0}, {0, 1, 0}};
static const int C_D3Q19[19][3] = {
    {0, 0, 0},  {-1, 0, 0}, {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1}, {-1, 0, 1}, {1, 0, 0},
    {1, 1, 0},  {1, -1, 0}, {1, 0, 1},   {1, 0, -1}, {0, -1, 0},  {0, 0, -1}, {0, -1, -1},
    {0, -1, 1}, {0, 1, 0},  {0, 0, 1},   {0, 1, 1},  {0, 1, -1}};
static const int C_D3Q27[27][3] = {
    {0, 0, 0},   {-1, 0, 0},  {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1}, {-1, 0, 1},  {-1, -1, -1},
    {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1},  {1, 0, 0},  {1, 1, 0},   {1, -1, 0},  {1, 0, 1},
    {1, 0, -1},  {1, 1, 1},   {1, 1, -1},  {1, -1, 1}, {1, -1, -1}, {0, -1, 0},  {0, 0, -1},
    {0, -1, -1}, {0, -1, 1},  {0, 1, 0},   {0, 0, 1},  {0, 1, 1},   {0, 1, -1}};

static const int C_D3Q15[15][3] = {
    {0, 0, 0},  {-1, 0, 0}, {-1, -1, -1}, {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1}, {1, 0, 0}, {1, 1, 1},
    {1, 1, -1}, {1, -1, 1}, {1, -1, -1},  {0, -1, 0},  {0, 0, -1},  {0, 1, 0},  {0, 0, 1}};
static const int C_D2Q13[13][3] = {{0, 0, 0}, {-1, 0, 0}, {-1, -1, 0}, {-1, 1, 0}, {-2, 0, 0},
                                   {1, 0, 0}, {1, -1, 0}, {1, 1, 0},   {2, 0, 0},  {0, -1, 0},
                                   {0, 1, 0}, {0, -2, 0}, {0, 2, 0}};
static const int C_D3Q33[33][3] = {
    {0, 0, 0},   {-1, 0, 0},  {-1, -1, 0}, {-1, 1, 0},  {-1, 0, -1}, {-1, 0, 1}, {-1, -1, -1},
    {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1},  {-2, 0, 0},  {1, 0, 0},   {1, 1, 0},  {1, -1, 0},
    {1, 0, 1},   {1, 0, -1},  {1, 1, 1},   {1, 1, -1},  {1, -1, 1},  {1, -1, -1}, {2, 0, 0},
    {0, -1, 0},  {0, 0, -1},  {0, -1, -1}, {0, -1, 1},  {0, 1, 0},   {0, 0, 1},  {0, 1, 1},
    {0, 1, -1},  {0, 2, 0},   {0, -2, 0},  {0, 0, 2},   {0, 0, -2}};

static void weights(int lattice, double* w) {
  if (lattice == ORACLE_D2Q9) {
    const double a = 4.0 / 9.0, b = 1.0 / 36.0, c = 1.0 / 9.0;
    const double t[9] = {a, b, c, b, b, c, b, c, c};
    memcpy(w, t, sizeof t);
  } else if (lattice == ORACLE_D3Q19) {
    const double a = 1.0 / 3.0, b = 1.0 / 18.0, c = 1.0 / 36.0;
    const double t[19] = {a, b, c, c, c, c, b, c, c, c, c, b, b, c, c, b, b, c, c};
    memcpy(w, t, sizeof t);
  } else if (lattice == ORACLE_D3Q27) {
    const double a = 8.0 / 27.0, b = 2.0 / 27.0, c = 1.0 / 54.0, d = 1.0 / 216.0;
    const double t[27] = {a, b, c, c, c, c, d, d, d, d, b, c, c, c,
                          c, d, d, d, d, b, b, c, c, b, b, c, c};
    memcpy(w, t, sizeof t);
  } else if (lattice == ORACLE_D3Q15) {
    const double a = 2.0 / 9.0, b = 1.0 / 9.0, c = 1.0 / 72.0;
    const double t[15] = {a, b, c, c, c, c, b, c, c, c, c, b, b, b, b};
    memcpy(w, t, sizeof t);
  } else if (lattice == ORACLE_D2Q13) {
    const double w0 = 1.0 / 2.0, w1 = 4.0 / 45.0, w2 = 1.0 / 30.0, w4 = 1.0 / 360.0;
    const double t[13] = {w0, w1, w2, w2, w4, w1, w2, w2, w4, w1, w1, w4, w4};
    memcpy(w, t, sizeof t);
  } else {
    const double w0 = 0.177627658370520295649084, w1 = 0.103315974899246818673111,
                 w2 = 0.000513472406731114352456, w3 = 0.021333928148672240120078,
                 w4 = 0.004273899693974583187026;
    const double t[33] = {w0, w1, w2, w2, w2, w2, w3, w3, w3, w3, w4, w1, w2, w2, w2, w2, w3,
                          w3, w3, w3, w4, w1, w1, w2, w2, w1, w1, w2, w2, w4, w4, w4, w4};
    memcpy(w, t, sizeof t);
  }
}

int oracle_lattice_q(int lattice) {
  static const int q[6] = {9, 19, 27, 15, 13, 33};
  return q[lattice];
}
int oracle_lattice_d(int lattice) {
  return (lattice == ORACLE_D2Q9 || lattice == ORACLE_D2Q13) ? 2 : 3;
}

/* inv_cs2 (Lattice.h): 3, except D3Q33 with cs2 = 0.4156023517935171 */
static double lattice_ics(int lattice) {
  return lattice == ORACLE_D3Q33 ? 1.0 / 0.4156023517935171 : 3.0;
}

static const int (*celerity(int lattice))[3] {
  switch (lattice) {
    case ORACLE_D2Q9: return C_D2Q9;
    case ORACLE_D3Q19: return C_D3Q19;
    case ORACLE_D3Q27: return C_D3Q27;
    case ORACLE_D3Q15: return C_D3Q15;
    case ORACLE_D2Q13: return C_D2Q13;
    default: return C_D3Q33;
  }
}

void oracle_lattice_tables(int lattice, double* c, double* w) {
  const int Q = oracle_lattice_q(lattice);
  const int(*ci)[3] = celerity(lattice);
  for (int q = 0; q < Q; ++q)
    for (int d = 0; d < 3; ++d) c[q * 3 + d] = (double)ci[q][d];
  weights(lattice, w);
}

#define QMAX 33

typedef struct {
  int D, Q;
  double c[QMAX][3];
  double w[QMAX];
  /* inv_cs2 and the Power<T, n>::Do(inv_cs2) of the equilibrium, left-folded
   * products (Helpers.h:93-113) */
  double ics, p2, p3, p4;
} lattice_t;

static void lattice_init(lattice_t* L, int lattice) {
  L->D = oracle_lattice_d(lattice);
  L->Q = oracle_lattice_q(lattice);
  const int(*ci)[3] = celerity(lattice);
  for (int q = 0; q < L->Q; ++q)
    for (int d = 0; d < 3; ++d) L->c[q][d] = (double)ci[q][d];
  weights(lattice, L->w);
  L->ics = lattice_ics(lattice);
  L->p2 = L->ics * L->ics;
  L->p3 = L->ics * L->ics * L->ics;
  L->p4 = L->ics * L->ics * L->ics * L->ics;
}

/* MathVector::dot (MathVector.h:45-53): a0*b0, then += ai*bi. */
static inline double dotD(const double* a, const double* b, int D) {
  double r = a[0] * b[0];
  for (int d = 1; d < D; ++d) r += a[d] * b[d];
  return r;
}

/* Equilibrium<TruncationMa3>::calculate (Equilibrium.h:14-33) with
 * k = inv_cs2 and its powers; Power<T,n> = left-folded products
 * (Helpers.h:93-113). */
static inline double equilibrium(const lattice_t* L, double rho, const double* u, double u2,
                                 int q) {
  const double cu = dotD(L->c[q], u, L->D);
  const double k = L->ics;
  const double fEq = 1.0 + cu * k - 0.5 * u2 * k + 0.5 * L->p2 * cu * cu -
                     0.5 * L->p2 * cu * u2 + (cu * cu * cu) * L->p3 / 6.0 +
                     0.125 * u2 * u2 * L->p2 - 0.25 * cu * cu * u2 * L->p3 +
                     (cu * cu * cu * cu) * L->p4 / 24.0;
  return rho * L->w[q] * fEq;
}

double oracle_equilibrium(int lattice, double rho, const double* u, int q) {
  lattice_t L;
  lattice_init(&L, lattice);
  return equilibrium(&L, rho, u, dotD(u, u, L.D), q);
}

/* Residual-mode alpha solve of single nodes (tests): alpha_max (capped at
 * 2.5, Collision.h:305-326), then the solve from guess[i] with Newton capped
 * at newton_maxit and the bisection-Newton at bisect_maxit. flags[i]: bit 0
 * alpha_max < 2 (alpha = 0.95 alpha_max), bit 1 the bracketed solver ran,
 * bit 2 alpha = 2 fallback. */
static double solve_residual(const double* f, const double* fneq, const double* w, int Q,
                             double tol, int maxit, int bisect_maxit, double guess, double xMax,
                             long long* iters, long long* fallbacks, long long* bisections);
void oracle_solve_alpha_nodes(int lattice, double tol, int newton_maxit, int bisect_maxit, long n,
                              const double* f, const double* fneq, const double* guess,
                              double* alpha, int* flags) {
  lattice_t L;
  lattice_init(&L, lattice);
  for (long i = 0; i < n; ++i) {
    const double* fi = f + i * L.Q;
    const double* ni = fneq + i * L.Q;
    double alphaMax = 2.5;
    for (int q = 0; q < L.Q; ++q)
      if (ni[q] > 0) {
        const double t = fabs(fi[q]) / ni[q];
        if (t < alphaMax) alphaMax = t;
      }
    flags[i] = 0;
    if (alphaMax < 2.) {
      alpha[i] = 0.95 * alphaMax;
      flags[i] = 1;
      continue;
    }
    long long it = 0, fb = 0, bi = 0;
    alpha[i] = solve_residual(fi, ni, L.w, L.Q, tol, newton_maxit, bisect_maxit, guess[i],
                              alphaMax, &it, &fb, &bi);
    flags[i] = (bi ? 2 : 0) | (fb ? 4 : 0);
  }
}

struct oracle_state {
  oracle_config cfg;
  lattice_t L;
  long V;
  double beta;
  double* prev;
  double* next;
  double* alpha; /* per node, persists across steps (Algorithm.h:103-106) */
  double* rho;   /* stored fields (Algorithm.h:150-194) */
  double* u;
  double* force;
  double* force_field; /* [D][V], ORACLE_F_FIELD */
  long long* newton_iterations;
  long long* fallbacks;
  long long* bisections;
};

/* ---- Forces (Force.h:137-292) ------------------------------------------
 * Coordinates are node-local (Collision.h:86: iP - halo). Sinusoidal:
 * F_d = A_d sin(x_d * 2 * pi / lambda_d) per axis (Force.h:208-215);
 * Kolmogorov: F_x = A_x sin(y * 2 * pi / lambda_x), other components 0
 * (Force.h:262-267). The unsigned coordinate times 2 is formed in integers
 * before the double multiply, as in the reference expression. */
static double sin_arg(unsigned coord, double lambda) {
  return (double)(coord * 2u) * M_PI / lambda;
}

static void node_force(const oracle_state* s, const unsigned* pos, double* F) {
  const oracle_config* c = &s->cfg;
  const int D = s->L.D;
  for (int d = 0; d < 3; ++d) F[d] = 0.0;
  switch (c->force) {
    case ORACLE_F_FIELD: { /* Force<Generic>::setForce (Force.h:36-45) */
      const long idx = ((long)pos[0] * c->ly + pos[1]) * c->lz + pos[2];
      for (int d = 0; d < D; ++d) F[d] = s->force_field[(long)d * s->V + idx];
      break;
    }
    case ORACLE_F_CONSTANT:
      for (int d = 0; d < D; ++d) F[d] = c->amplitude[d];
      break;
    case ORACLE_F_SINUSOIDAL:
      for (int d = 0; d < D; ++d) F[d] = c->amplitude[d] * sin(sin_arg(pos[d], c->wavelength[d]));
      break;
    case ORACLE_F_KOLMOGOROV: {
      const int k = c->kolmogorov_component;
      F[k] = c->amplitude[k] * sin(sin_arg(pos[c->kolmogorov_axis], c->wavelength[k]));
      break;
    }
    default:
      break;
  }
}

/* ---- Forcing schemes (ForcingScheme.h:17-198) -------------------------- */
static inline double collision_source(const oracle_state* s, const double* F, double rho,
                                      const double* u, double eq_q, int q) {
  const lattice_t* L = &s->L;
  const int D = L->D;
  switch (s->cfg.forcing) {
    case ORACLE_FS_GUO: { /* ForcingScheme.h:100-117 */
      const double cu = dotD(L->c[q], u, D);
      double v[3] = {0.0, 0.0, 0.0};
      for (int d = 0; d < D; ++d) v[d] = L->c[q][d] - u[d] + (L->ics * cu) * L->c[q][d];
      const double R = dotD(v, F, D);
      return (1.0 - 1.0 / (2.0 * s->cfg.tau)) * L->w[q] * L->ics * R;
    }
    case ORACLE_FS_EDM: { /* ForcingScheme.h:183-197 */
      const double inv = 1.0 / rho;
      double v[3] = {0.0, 0.0, 0.0};
      for (int d = 0; d < D; ++d) v[d] = u[d] + F[d] * inv;
      return equilibrium(L, rho, v, dotD(v, v, D), q) - eq_q;
    }
    default: /* None (ForcingScheme.h:68-78), ShanChen (141-151) */
      return 0.0;
  }
}

/* ---- Entropic step (EntropicStep.h:15-63) ------------------------------ */
typedef struct {
  const double* f;    /* pulled populations */
  const double* fneq; /* f - f_eq */
  const double* w;
  int Q;
  int perturb; /* oracle_config.log_ulp_perturbation */
} hfun_t;

/* The reference's log (libm), or with log_ulp_perturbation the libm result
 * moved by one ulp on about half of the arguments (chosen by a hash of the
 * argument's bits): a stand-in for another correctly working logarithm, to
 * measure how far the reference algorithm's result depends on the last bit
 * of its logarithms. */
static double ref_log(double x, int perturb) {
  const double l = log(x);
  if (!perturb) return l;
  uint64_t b;
  memcpy(&b, &x, sizeof b);
  b ^= b >> 29;
  b *= 0xbf58476d1ce4e5b9ULL;
  b ^= b >> 32;
  if ((b & 3) == 0) return nextafter(l, INFINITY);
  if ((b & 3) == 1) return nextafter(l, -INFINITY);
  return l;
}

/* With population_ulp_perturbation: a BGK result moved by one ulp, up or
 * down, on about half of the stores (chosen by a hash of its bits and its
 * index): a stand-in for another FP64 evaluation of the same update with a
 * different rounding, to measure how far the state over many steps depends on
 * the last bit of each population. */
static double ulp_nudge(double r, uint64_t key) {
  uint64_t b;
  memcpy(&b, &r, sizeof b);
  b ^= key * 0x9e3779b97f4a7c15ULL;
  b ^= b >> 31;
  b *= 0xbf58476d1ce4e5b9ULL;
  b ^= b >> 29;
  if ((b & 3) == 0) return nextafter(r, INFINITY);
  if ((b & 3) == 1) return nextafter(r, -INFINITY);
  return r;
}

static double h_function(const hfun_t* h, double alpha) {
  double r = 0.0;
  for (int q = 0; q < h->Q; ++q) {
    const double f = h->f[q];
    const double g = f - alpha * h->fneq[q];
    r += f * ref_log(f / h->w[q], h->perturb) - g * ref_log(g / h->w[q], h->perturb);
  }
  return r;
}

static double h_derivative(const hfun_t* h, double alpha) {
  double r = 0.0;
  for (int q = 0; q < h->Q; ++q) {
    const double g = h->f[q] - alpha * h->fneq[q];
    r += h->fneq[q] * (1 + ref_log(g / h->w[q], h->perturb));
  }
  return r;
}

/* NewtonRaphsonSolver (EntropicStep.h:111-140). */
static int newton(const hfun_t* h, double tol, int maxit, double* xR, double xMin, double xMax,
                  long long* iters) {
  double xStep = 0.0;
  for (int it = 1; it <= maxit; ++it) {
    *xR = *xR - xStep;
    const double fe = h_function(h, *xR);
    const double de = h_derivative(h, *xR);
    ++*iters;
    xStep = fe / de;
    const double error = fabs(xStep);
    if (error <= tol) return (*xR > xMin && *xR < xMax) ? 1 : 0;
  }
  return 0;
}

/* ---- Residual mode: the FP64 logarithm and log1p series of the kernels ----
 * ln(x) after P. T. P. Tang, ACM TOMS 16(4), 1990: x = 2^e m, j = top 7
 * fraction bits of m, inv_j = RN(1/c_j) for the interval centre c_j,
 * r = fma(m, inv_j, -1), ln x = e ln2 + ln(1/inv_j) + log1p(r) with a
 * degree-7 series; the table is built in the host's extended precision. The
 * kernels use the same function, so the residual-mode step is reproduced
 * operation for operation. */
typedef struct {
  double inv, hi, lo;
} logent_t;

static logent_t g_log_table[128];
static pthread_once_t g_log_once = PTHREAD_ONCE_INIT;

static void build_log_table(void) {
  for (int j = 0; j < 128; ++j) {
    const double c = 1.0 + (j + 0.5) / 128.0;
    const double inv = 1.0 / c;
    const long double L = -logl((long double)inv);
    const double hi = (double)L;
    g_log_table[j].inv = inv;
    g_log_table[j].hi = hi;
    g_log_table[j].lo = (double)(L - (long double)hi);
  }
}

static double series7(double r) {
  double p = 1.0 / 7.0;
  p = fma(p, r, -1.0 / 6.0);
  p = fma(p, r, 1.0 / 5.0);
  p = fma(p, r, -1.0 / 4.0);
  p = fma(p, r, 1.0 / 3.0);
  p = fma(p, r, -0.5);
  return fma(p * r, r, r);
}

static double series9(double t) {
  double p = 1.0 / 9.0;
  p = fma(p, t, -1.0 / 8.0);
  p = fma(p, t, 1.0 / 7.0);
  p = fma(p, t, -1.0 / 6.0);
  p = fma(p, t, 1.0 / 5.0);
  p = fma(p, t, -1.0 / 4.0);
  p = fma(p, t, 1.0 / 3.0);
  p = fma(p, t, -0.5);
  return fma(p * t, t, t);
}

static double series5(double t) {
  double p = 1.0 / 5.0;
  p = fma(p, t, -1.0 / 4.0);
  p = fma(p, t, 1.0 / 3.0);
  p = fma(p, t, -0.5);
  return fma(p * t, t, t);
}

static double tang_log(double x) {
  const double kLn2Hi = 0x1.62e42fefa3800p-1, kLn2Lo = 0x1.ef35793c76730p-45;
  uint64_t bits;
  memcpy(&bits, &x, sizeof bits);
  int e = (int)((bits >> 52) & 0x7ff);
  if (e == 0) {
    const double xs = x * 18014398509481984.0;
    memcpy(&bits, &xs, sizeof bits);
    e = (int)((bits >> 52) & 0x7ff) - 54;
  }
  e -= 1023;
  const int j = (int)((bits >> 45) & 127);
  const uint64_t mb = (bits & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
  double m;
  memcpy(&m, &mb, sizeof m);
  const logent_t t = g_log_table[j];
  const double r = fma(m, t.inv, -1.0);
  const double ed = (double)e;
  const double hi = fma(ed, kLn2Hi, t.hi);
  const double lo = fma(ed, kLn2Lo, t.lo) + series7(r);
  return hi + lo;
}

double oracle_fast_log(double x) {
  pthread_once(&g_log_once, build_log_table);
  return tang_log(x);
}

/* Residual-mode entropy function in log1p form. With r = f_neq/f and
 * t = -x r (g = f (1 + t)), ln(g/w) = L + log1p(t), L = ln(f/w), and
 *   F(x)  = x B1 - sum f (1 + t) log1p(t),  B1 = sum f_neq L,
 *   F'(x) = C0 + sum f r log1p(t),          C0 = sum f_neq + B1,
 * the same function as sum f ln(f/w) - sum g ln(g/w) (EntropicStep.h:31-45)
 * and its derivative (47-62), formed from O(|f_neq|) terms. log1p is a
 * degree-5 series when every |t| <= 2^-10, degree 9 for |t| <= 2^-6, and the
 * logarithm above otherwise. */
typedef struct {
  const double* f;
  const double* r;
  double B1, C0, rmax;
  int Q;
} hlog1p_t;

static void h_log1p(const hlog1p_t* h, double x, double* F, double* dF) {
  double s = 0.0, d = 0.0;
  if (x * h->rmax <= 0.0009765625) {
    for (int q = 0; q < h->Q; ++q) {
      const double t = -x * h->r[q];
      const double lp = series5(t);
      s = fma(fma(h->f[q], t, h->f[q]), lp, s);
      d = fma(h->f[q] * h->r[q], lp, d);
    }
  } else {
    for (int q = 0; q < h->Q; ++q) {
      const double t = -x * h->r[q];
      const double opt = 1.0 + t;
      double lp;
      if (fabs(t) <= 0.015625) lp = series9(t);
      else if (opt > 0.0) lp = tang_log(opt);
      else lp = -745.0; /* g = 0 at alpha_max: g ln g -> 0 */
      if (opt > 0.0) s = fma(h->f[q] * opt, lp, s);
      d = fma(h->f[q] * h->r[q], lp, d);
    }
  }
  *F = fma(x, h->B1, -s);
  *dF = h->C0 + d;
}

/* Safeguarded bisection-Newton on [xMin, xMax], the update rule of
 * Bisection_NewtonRaphsonSolver (EntropicStep.h:142-220) with |F| <= tol as
 * the acceptance test. */
static int bisection_newton_residual(const hlog1p_t* h, double tol, int maxit, double* xR,
                                     double xMin, double xMax, long long* iters) {
  double fLow, fHigh, d;
  h_log1p(h, xMin, &fLow, &d);
  h_log1p(h, xMax, &fHigh, &d);
  if ((fLow > 0.0 && fHigh > 0.0) || (fLow < 0.0 && fHigh < 0.0)) return 0;
  if (fabs(fLow) <= tol) { *xR = xMin; return 1; }
  if (fabs(fHigh) <= tol) { *xR = xMax; return 1; }
  double xLow, xHigh;
  if (fLow < 0.0) { xLow = xMin; xHigh = xMax; } else { xLow = xMax; xHigh = xMin; }
  double x = 0.5 * (xMin + xMax);
  double dxOld = fabs(xMax - xMin), dx = dxOld;
  double fe, de;
  h_log1p(h, x, &fe, &de);
  for (int it = 1; it <= maxit; ++it) {
    if (fabs(fe) <= tol) { *xR = x; return 1; }
    ++*iters;
    if ((((x - xHigh) * de - fe) * ((x - xLow) * de - fe) > 0.0) ||
        (fabs(2.0 * fe) > fabs(dxOld * de))) {
      dxOld = dx;
      dx = 0.5 * (xHigh - xLow);
      x = xLow + dx;
      if (xLow == x) { *xR = x; return 1; }
    } else {
      dxOld = dx;
      dx = fe / de;
      const double xTemp = x;
      x -= dx;
      if (xTemp == x) { *xR = x; return 1; }
    }
    h_log1p(h, x, &fe, &de);
    if (fe < 0.0) xLow = x; else xHigh = x;
  }
  *xR = x;
  return fabs(fe) <= tol;
}

/* Residual-mode solve from a guess (see mlbm_oracle.h). */
static double solve_residual(const double* f, const double* fneq, const double* w, int Q,
                             double tol, int maxit, int bisect_maxit, double guess, double xMax,
                             long long* iters, long long* fallbacks, long long* bisections) {
  pthread_once(&g_log_once, build_log_table);
  double r[QMAX], B1 = 0.0, sfn = 0.0, rmax = 0.0;
  for (int q = 0; q < Q; ++q) {
    B1 = fma(fneq[q], tang_log(f[q] * (1.0 / w[q])), B1);
    sfn += fneq[q];
    r[q] = fneq[q] / f[q];
    rmax = fmax(rmax, fabs(r[q]));
  }
  const hlog1p_t h = {f, r, B1, sfn + B1, rmax, Q};
  double x = guess;
  if (x > 1.0 && x < xMax) {
    double fe, de;
    h_log1p(&h, x, &fe, &de);
    if (fabs(fe) <= tol) return x;
    for (int it = 1; it <= maxit; ++it) {
      ++*iters;
      x -= fe / de;
      if (!(x > 1.0 && x < xMax)) break;
      h_log1p(&h, x, &fe, &de);
      if (fabs(fe) <= tol) return x;
    }
  }
  ++*bisections;
  if (bisection_newton_residual(&h, tol, bisect_maxit, &x, 1.0, xMax, iters)) return x;
  ++*fallbacks;
  return 2.0;
}

/* ELBM::calculateAlpha (Collision.h:351-375) with isDeviationSmall (284-303),
 * calculateAlphaMax (305-326) and solveAlpha (328-349). */
static double entropic_alpha(const oracle_state* s, const double* f, const double* fneq,
                             double guess, long long* iters, long long* fallbacks,
                             long long* bisections) {
  const int Q = s->L.Q;
  const oracle_config* c = &s->cfg;
  int small = 1;
  for (int q = 0; q < Q; ++q)
    if (fabs(fneq[q]) / f[q] > c->deviation_threshold) small = 0;
  if (small) return 2.0;
  double alphaMax = 2.5;
  for (int q = 0; q < Q; ++q) {
    if (fneq[q] > 0) {
      const double t = fabs(f[q]) / fneq[q];
      if (t < alphaMax) alphaMax = t;
    }
  }
  if (alphaMax < 2.) return 0.95 * alphaMax;
  const hfun_t h = {f, fneq, s->L.w, Q, c->log_ulp_perturbation};
  if (c->guess_mode == ORACLE_GUESS_TWO) guess = 2.0;
  if (c->alpha_mode == ORACLE_ALPHA_RESIDUAL)
    return solve_residual(f, fneq, s->L.w, Q, c->newton_tolerance, c->newton_max_iterations,
                          c->bisection_max_iterations > 0 ? c->bisection_max_iterations
                                                          : c->newton_max_iterations,
                          guess, alphaMax, iters, fallbacks, bisections);
  double alpha = guess;
  if (newton(&h, c->newton_tolerance, c->newton_max_iterations, &alpha, 1., alphaMax, iters))
    return alpha;
  ++*fallbacks;
  return 2.0;
}

/* ---- One node of the fused pull step (Algorithm.h:97-126) -------------- */
static void node_update(oracle_state* s, unsigned x, unsigned y, unsigned z, int store,
                        long long* iters, long long* fallbacks, long long* bisections) {
  const lattice_t* L = &s->L;
  const oracle_config* c = &s->cfg;
  const int Q = L->Q, D = L->D;
  const unsigned lx = (unsigned)c->lx, ly = (unsigned)c->ly, lz = (unsigned)c->lz;
  const long V = s->V;
  const long idx = ((long)x * ly + y) * lz + z;

  /* Pulled populations f_q(x - c_q): periodic wrap by modulo replaces the
   * reference's halo planes (Communication.h:134-180, Boundary.h:50-100). */
  double f[QMAX] = {0.0};
  for (int q = 0; q < Q; ++q) {
    const int* cq = celerity(c->lattice)[q];
    const long sx = ((long)x - cq[0] + 2 * (long)lx) % lx;
    const long sy = ((long)y - cq[1] + 2 * (long)ly) % ly;
    const long sz = ((long)z - cq[2] + 2 * (long)lz) % lz;
    f[q] = s->prev[(long)q * V + (sx * ly + sy) * lz + sz];
  }

  /* Moment::calculateDensity / calculateVelocity (Moment.h:13-47). */
  double rho = f[0];
  for (int q = 1; q < Q; ++q) rho += f[q];
  double u[3] = {0.0, 0.0, 0.0};
  for (int d = 0; d < D; ++d) u[d] = L->c[0][d] * f[0];
  for (int q = 1; q < Q; ++q)
    for (int d = 0; d < D; ++d) u[d] += L->c[q][d] * f[q];
  for (int d = 0; d < D; ++d) u[d] /= rho;
  const double u2 = dotD(u, u, D);

  /* Collision::setForce (Collision.h:81-88). */
  const unsigned pos[3] = {x, y, z};
  double F[3];
  node_force(s, pos, F);

  double* nxt = s->next;
  double alpha;
  if (c->collision == ORACLE_BGK) {
    /* Collision<BGK>::collideAndStream (Collision.h:134-151). */
    alpha = 2.0;
    const double a = 1. - 2. * s->beta, b = 2. * s->beta;
    for (int q = 0; q < Q; ++q) {
      const double eq = equilibrium(L, rho, u, u2, q);
      double r = a * f[q] + b * eq + collision_source(s, F, rho, u, eq, q);
      if (c->population_ulp_perturbation) r = ulp_nudge(r, (uint64_t)q * (uint64_t)V + (uint64_t)idx);
      nxt[(long)q * V + idx] = r;
    }
  } else {
    /* Collision<ELBM>::calculateRelaxationTime (Collision.h:227-241) and
     * collideAndStream (243-258). */
    double fneq[QMAX];
    for (int q = 0; q < Q; ++q) fneq[q] = f[q] - equilibrium(L, rho, u, u2, q);
    alpha = entropic_alpha(s, f, fneq, s->alpha[idx], iters, fallbacks, bisections);
    const double tauEff = 1.0 / (alpha * s->beta);
    const double inv = 1.0 / tauEff;
    for (int q = 0; q < Q; ++q) {
      const double eq = f[q] - fneq[q];
      nxt[(long)q * V + idx] = f[q] - inv * fneq[q] + collision_source(s, F, rho, u, eq, q);
    }
  }
  s->alpha[idx] = alpha;

  if (store) { /* Algorithm::storeFields (Algorithm.h:150-194) */
    s->rho[idx] = rho;
    for (int d = 0; d < D; ++d) {
      /* ForcingScheme::calculateHydrodynamicVelocity: u + 0.5/rho F
       * (ForcingScheme.h:27-33), unshifted for None (53-57). */
      const double uh = (c->forcing == ORACLE_FS_NONE) ? u[d] : u[d] + F[d] * (0.5 / rho);
      s->u[(long)d * V + idx] = uh;
      s->force[(long)d * V + idx] = F[d];
    }
  }
}

oracle_state* oracle_create(const oracle_config* cfg) {
  oracle_state* s = (oracle_state*)calloc(1, sizeof(oracle_state));
  if (!s) return NULL;
  s->cfg = *cfg;
  if (s->cfg.threads < 1) s->cfg.threads = 1;
  lattice_init(&s->L, cfg->lattice);
  if (s->L.D == 2) s->cfg.lz = 1;
  s->V = (long)s->cfg.lx * s->cfg.ly * s->cfg.lz;
  s->beta = (double)1.0 / (2.0 * cfg->tau);
  const long V = s->V, Q = s->L.Q, D = s->L.D;
  s->prev = (double*)calloc((size_t)(Q * V), sizeof(double));
  s->next = (double*)calloc((size_t)(Q * V), sizeof(double));
  s->alpha = (double*)malloc(sizeof(double) * (size_t)V);
  s->rho = (double*)calloc((size_t)V, sizeof(double));
  s->u = (double*)calloc((size_t)(D * V), sizeof(double));
  s->force = (double*)calloc((size_t)(D * V), sizeof(double));
  s->force_field = (double*)calloc((size_t)(D * V), sizeof(double));
  s->newton_iterations = (long long*)calloc((size_t)s->cfg.threads, sizeof(long long));
  s->fallbacks = (long long*)calloc((size_t)s->cfg.threads, sizeof(long long));
  s->bisections = (long long*)calloc((size_t)s->cfg.threads, sizeof(long long));
  if (!s->prev || !s->next || !s->alpha || !s->rho || !s->u || !s->force || !s->force_field ||
      !s->newton_iterations || !s->fallbacks || !s->bisections) {
    oracle_destroy(s);
    return NULL;
  }
  for (long i = 0; i < V; ++i) s->alpha[i] = 2.0;
  return s;
}

void oracle_destroy(oracle_state* s) {
  if (!s) return;
  free(s->prev);
  free(s->next);
  free(s->alpha);
  free(s->rho);
  free(s->u);
  free(s->force);
  free(s->force_field);
  free(s->newton_iterations);
  free(s->fallbacks);
  free(s->bisections);
  free(s);
}

void oracle_init_equilibrium(oracle_state* s, const double* rho, const double* u) {
  const long V = s->V;
  const int Q = s->L.Q, D = s->L.D;
  for (long i = 0; i < V; ++i) {
    double v[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) v[d] = u[(long)d * V + i];
    const double u2 = dotD(v, v, D);
    for (int q = 0; q < Q; ++q) s->prev[(long)q * V + i] = equilibrium(&s->L, rho[i], v, u2, q);
    s->alpha[i] = 2.0;
  }
}

void oracle_set_populations(oracle_state* s, const double* f) {
  memcpy(s->prev, f, sizeof(double) * (size_t)(s->L.Q * s->V));
}

void oracle_get_populations(const oracle_state* s, double* f) {
  memcpy(f, s->prev, sizeof(double) * (size_t)(s->L.Q * s->V));
}

typedef struct {
  oracle_state* s;
  int tid, store;
} sweep_arg;

static void* sweep(void* p) {
  sweep_arg* a = (sweep_arg*)p;
  oracle_state* s = a->s;
  const int T = s->cfg.threads;
  const unsigned lx = (unsigned)s->cfg.lx, ly = (unsigned)s->cfg.ly, lz = (unsigned)s->cfg.lz;
  /* X slabs, as the reference's 1-D MPI decomposition (Domain.h:22-24). */
  const unsigned x0 = (unsigned)((long)lx * a->tid / T), x1 = (unsigned)((long)lx * (a->tid + 1) / T);
  long long it = 0, fb = 0, bi = 0;
  for (unsigned x = x0; x < x1; ++x)
    for (unsigned y = 0; y < ly; ++y)
      for (unsigned z = 0; z < lz; ++z) node_update(s, x, y, z, a->store, &it, &fb, &bi);
  s->newton_iterations[a->tid] = it;
  s->fallbacks[a->tid] = fb;
  s->bisections[a->tid] = bi;
  return NULL;
}

void oracle_step(oracle_state* s, int nsteps, int store_last) {
  const int T = s->cfg.threads;
  for (int it = 1; it <= nsteps; ++it) {
    const int store = store_last && it == nsteps;
    if (T == 1) {
      sweep_arg a = {s, 0, store};
      sweep(&a);
    } else {
      pthread_t th[256];
      sweep_arg args[256];
      const int n = T > 256 ? 256 : T;
      for (int t = 0; t < n; ++t) {
        args[t].s = s;
        args[t].tid = t;
        args[t].store = store;
        pthread_create(&th[t], NULL, sweep, &args[t]);
      }
      for (int t = 0; t < n; ++t) pthread_join(th[t], NULL);
    }
    double* tmp = s->prev;
    s->prev = s->next;
    s->next = tmp;
  }
}

void oracle_get_fields(const oracle_state* s, double* rho, double* u, double* alpha,
                       double* force) {
  const long V = s->V, D = s->L.D;
  if (rho) memcpy(rho, s->rho, sizeof(double) * (size_t)V);
  if (u) memcpy(u, s->u, sizeof(double) * (size_t)(D * V));
  if (alpha) memcpy(alpha, s->alpha, sizeof(double) * (size_t)V);
  if (force) memcpy(force, s->force, sizeof(double) * (size_t)(D * V));
}

void oracle_set_force_field(oracle_state* s, const double* force) {
  memcpy(s->force_field, force, sizeof(double) * (size_t)(s->L.D * s->V));
}

void oracle_get_counters(const oracle_state* s, long long* newton_iterations,
                         long long* fallbacks, long long* bisections) {
  long long a = 0, b = 0, c = 0;
  for (int t = 0; t < s->cfg.threads; ++t) {
    a += s->newton_iterations[t];
    b += s->fallbacks[t];
    c += s->bisections[t];
  }
  if (newton_iterations) *newton_iterations = a;
  if (fallbacks) *fallbacks = b;
  if (bisections) *bisections = c;
}
