/* mlbm.h - C ABI of the GB300-native fused collide-and-stream pull step.
 *
 * Drop-in for metaLBM's hot path: Algorithm<T, Pull, ..., OneD, MPI, Off>
 * (include/metaLBM/Algorithm.h:23-29, 326-358) with its Collision / ForcingScheme
 * / Force / Lattice template choices (Collision.h:913-914, ForcingScheme.h:200,
 * Force.h:628-629, Lattice.h:804-806) and the Input.in parameters
 * (src/Input_prod.in:16-53) turned into a runtime configuration. One handle owns
 * one periodic lattice on one GPU; the periodic wrap is done inside the kernel,
 * so there are no halo cells and no halo exchange (Communication.h:134-180,
 * Boundary.h:50-100 become an index modulo).
 *
 * Every function returns MLBM_OK (0) or an error code; mlbm_last_error(h)
 * gives the message. Host arrays are caller-owned and copied; device buffers
 * are owned by the handle. A handle is used by one host thread at a time; there
 * is no global state shared between handles. No call aborts the process (the
 * reference prints and calls exit(-1), Commons.h:6-38).
 */
#ifndef MLBM_H
#define MLBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MLBM_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum {
  MLBM_OK = 0,
  MLBM_ERR_INVALID = 1,   /* bad argument or configuration */
  MLBM_ERR_CUDA = 2,      /* a CUDA runtime call failed */
  MLBM_ERR_ALLOC = 3,     /* device or host allocation failed */
  MLBM_ERR_TIMEOUT = 4,   /* mlbm_sync gave up waiting */
  MLBM_ERR_NUMERIC = 5,   /* the device error word is set (see mlbm_diag) */
  MLBM_ERR_STATE = 6,     /* call not valid in the handle's state */
  MLBM_ERR_NO_DEVICE = 7  /* no usable CUDA device */
};

/* ---- template axes of the reference, as runtime enums -------------------
 * Names and order follow include/metaLBM/Options.h:12-43. */
/* LatticeType (Options.h:12-13). D2Q13 and D3Q33 reach two nodes (the
 * reference's halo 2) and run with FP64 storage only; D3Q15 also runs with
 * FP32 / FP16-shifted storage. */
enum {
  MLBM_D2Q9 = 0,
  MLBM_D3Q19 = 1,
  MLBM_D3Q27 = 2,
  MLBM_D3Q15 = 3,
  MLBM_D2Q13 = 4,
  MLBM_D3Q33 = 5
};
/* CollisionType (Options.h:33-36). Every entropic type from 2 on runs as
 * MLBM_ELBM: in the reference they only redefine the non-virtual
 * calculateAlpha, which ELBM::calculateRelaxationTime never reaches
 * (Collision.h:227-241), so their populations equal ELBM's bit for bit.
 * ForcedNR_ELBM_Forcing (subtracts f_eq from the pulled source in place) and
 * GenericSRT / GenericMRT (abstract) have no value. */
enum {
  MLBM_BGK = 0,
  MLBM_ELBM = 1,
  MLBM_FORCED_BNR_ELBM = 2,
  MLBM_APPROACHED_ELBM = 3,
  MLBM_MALASPINAS_ELBM = 4,
  MLBM_ESSENTIALLY1_ELBM = 5,
  MLBM_ESSENTIALLY2_ELBM = 6,
  MLBM_FORCED_NR_ELBM = 7
};
enum { MLBM_FORCING_NONE = 0, MLBM_FORCING_GUO = 1, MLBM_FORCING_SHAN_CHEN = 2,
       MLBM_FORCING_EXACT_DIFFERENCE = 3 };                         /* ForcingSchemeType */
/* ForceType (Options.h:39-41). The spectral forces (Force.h:294-626) are a
 * per-node force field computed on the device (FP64; a float copy for FP32 /
 * FP16 storage). Every force takes force_amplitude and the shell
 * force_kmin <= |k| <= force_kmax (Algorithm.h:90-91); removal_amplitude /
 * removal_kmin / removal_kmax are the removal part of TURBULENT_2D only
 * (Force.h:585-587):
 *   CONSTANT_SHELL  time-independent solenoidal forcing on the shell (curl of
 *                   a constant-amplitude spectrum)
 *   ENERGY_REMOVAL  F = -A P_shell(rho u) from the last stored fields
 *   TURBULENT_2D    CONSTANT_SHELL(force_*) + ENERGY_REMOVAL(removal_*), any
 *                   dimension */
enum {
  MLBM_FORCE_NONE = 0,
  MLBM_FORCE_CONSTANT = 1,
  MLBM_FORCE_SINUSOIDAL = 2,
  MLBM_FORCE_KOLMOGOROV = 3,
  MLBM_FORCE_CONSTANT_SHELL = 4,
  MLBM_FORCE_ENERGY_REMOVAL = 5,
  MLBM_FORCE_TURBULENT_2D = 6
};

/* Population storage in HBM. F64 is the reference's dataT = double;
 * F32 stores f in float; F16_SHIFTED stores (f_q - w_q) * 2^k_q in binary16
 * with a per-population power of two k_q (k_q = round(log2(1024 / w_q))).
 * F32 and F16_SHIFTED collide in float, in deviation variables f_q - w_q. */
enum { MLBM_STORAGE_F64 = 0, MLBM_STORAGE_F32 = 1, MLBM_STORAGE_F16_SHIFTED = 2 };
/* mlbm_config.fp64_arithmetic */
enum { MLBM_F64_REFERENCE_ORDER = 0, MLBM_F64_FIXED_POINT = 1 };

/* Entropic alpha solver.
 * REFERENCE: Collision.h:284-375 with NewtonRaphsonSolver (EntropicStep.h:111-140):
 *   alpha = 2 if every |f_neq|/f <= deviation_threshold, 0.95*alpha_max if
 *   alpha_max < 2, else Newton until |step| <= newton_tolerance; alpha = 2 when
 *   Newton fails. The reference's ForcedBNR_ELBM resolves to this same solver
 *   (its bisection override is never called, Collision.h:227-241).
 * RESIDUAL: accept alpha when the FP64 entropy residual
 *   |F(alpha)| = |sum f ln(f/w) - sum g ln(g/w)|, g = f - alpha f_neq, is
 *   <= newton_tolerance; Newton from the guess, then the safeguarded
 *   bisection-Newton of EntropicStep.h:142-220 on [1, alpha_max]; alpha = 2
 *   only when both fail. */
enum { MLBM_ALPHA_REFERENCE = 0, MLBM_ALPHA_RESIDUAL = 1 };
/* Starting guess of the alpha solve: the node's alpha from the previous step
 * (the reference, Algorithm.h:103-106), the constant 2, or the learned model
 * installed with mlbm_set_alpha_model. LEARNED runs the model where a node has
 * no solved alpha from the previous step (its stored alpha is exactly 2:
 * after mlbm_init_equilibrium, mlbm_set_alpha, or an alpha = 2 fallback) and
 * takes the previous alpha elsewhere; an mlbm_step call that starts with no
 * such node runs kernels without the network (a node that falls back to
 * alpha = 2 during that call takes the constant 2 until the next call).
 * LEARNED_EVERYWHERE runs the model at every solved node. Both need FP32 /
 * FP16 storage. */
enum { MLBM_GUESS_PREVIOUS = 0, MLBM_GUESS_TWO = 1, MLBM_GUESS_LEARNED = 2,
       MLBM_GUESS_LEARNED_EVERYWHERE = 3 };

/* Host array layouts.
 * DENSE: component-major, node index (x*Ly + y)*Lz + z (z fastest, the
 *   reference's node order, Domain.h:88-91), no padding. Populations are
 *   [Q][V], vectors [D][V].
 * REFERENCE: the reference's FieldList/Distribution local arrays: the same
 *   order with the last dimension padded to 2*(N/2+1) (FFTW real-to-complex
 *   padding, Domain.h:53-57, FFTWInitializer.h:24-27), component stride
 *   numberElements = padded volume (Field.h:122-125). Padding entries are
 *   left untouched on output and ignored on input. */
enum { MLBM_LAYOUT_DENSE = 0, MLBM_LAYOUT_REFERENCE = 1 };

/* mlbm_step flags */
#define MLBM_STEP_STORE_FIELDS 0x1u /* isStored on the last step (Algorithm.h:67, 150-194) */
#define MLBM_STEP_DIAGNOSTICS 0x2u  /* fused energy / mass / max-Mach reduction, last step */
#define MLBM_STEP_LOG_SAMPLES 0x4u  /* log (f_neq/rho, alpha*) at the sample nodes, last step */

typedef struct {
  int lattice;            /* latticeT */
  int collision;          /* collisionT */
  int forcing_scheme;     /* forcingSchemeT */
  int force;              /* forceT */
  double relaxation_time; /* relaxationTime (tau); beta = 1/(2 tau) */
  double force_amplitude[3];  /* forceAmplitude */
  double force_wavelength[3]; /* forceWaveLength */
  /* Kolmogorov force: F[component] = A[component] sin(2 pi x[axis] / lambda[component]).
   * The reference is axis = 1 (y), component = 0 (x) (Force.h:262-267). */
  int kolmogorov_axis;
  int kolmogorov_component;
  int length[3];          /* globalLengthX/Y/Z; length[2] is ignored for D2Q9 */
  int storage;            /* MLBM_STORAGE_* */
  int alpha_mode;         /* MLBM_ALPHA_* */
  int alpha_guess;        /* MLBM_GUESS_* */
  double newton_tolerance;    /* reference 1e-8 (Collision.h:336) */
  int newton_max_iterations;  /* reference 50 (Collision.h:337) */
  double deviation_threshold; /* reference 1e-3 (Collision.h:357); 0 disables */
  int device;             /* CUDA device ordinal */
  /* spectral forces (Input_prod_3d.in:50-58): integer wavenumber shells */
  int force_kmin;             /* forcekMin, reference 1 */
  int force_kmax;             /* forcekMax, reference 2 */
  int removal_kmin;           /* removalForcekMin, reference 1 */
  int removal_kmax;           /* removalForcekMax, reference 2 */
  double removal_amplitude[3]; /* removalForceAmplitude, reference 1e-6 */
  /* RESIDUAL alpha solver: iteration cap of the safeguarded bisection-Newton
   * (0: newton_max_iterations, as the reference passes one iterationMax to
   * both solvers, Collision.h:336-341, 892-897). With newton_max_iterations = 0
   * every node whose guess fails goes straight to the bracketed solver. */
  int bisection_max_iterations;
  /* FP64 storage, BGK: MLBM_F64_REFERENCE_ORDER (the reference's operations
   * in its order, bit-identical results) or MLBM_F64_FIXED_POINT (the same
   * update with exact fixed-point moments and equilibrium on the integer
   * pipe, within a few FP64 ulp a step; D2Q9, D3Q19, D3Q27, D3Q15 with
   * forcing None, Guo or Shan-Chen, otherwise the reference order). */
  int fp64_arithmetic;
  int reserved[2];
} mlbm_config;

typedef struct {
  long long step;         /* steps taken since creation */
  double mass;            /* sum rho over the lattice (last diagnostics step) */
  double energy;          /* (1/V) sum 1/2 rho |u|^2, u = hydrodynamic velocity
                             (Analysis.h:33-66) */
  double max_mach;        /* max |u| / c_s */
  double alpha_min, alpha_max;
  long long solved_nodes;      /* entropic nodes that went through the alpha solve */
  long long newton_iterations; /* Newton/bisection updates over the last mlbm_step call */
  long long guess_hits;        /* solved nodes whose guess passed the residual test */
  long long bisection_nodes;   /* nodes that needed the bracketed solver */
  long long fallback_nodes;    /* nodes that fell back to alpha = 2 */
  long long limited_nodes;     /* nodes with alpha = 0.95 alpha_max */
  long long shortcut_nodes;    /* nodes with every |f_neq|/f below the threshold */
  unsigned int error_word;     /* bit 0: non-finite population; bit 1: negative density */
  unsigned int reserved0;
  long long series_nodes;      /* solved nodes of the FP32/FP16-storage kernels whose
                                  entropy function took the moment-series form */
  long long learned_nodes;     /* solved nodes whose guess came from the learned model */
  double reserved[4];
} mlbm_diag;

/* Learned alpha guess: an MLP in -> 32 -> 32 -> 1 with tanh hidden layers.
 * Input x_q = (f_neq_q / rho) * input_scale[q]; guess = 2 + output_scale * y.
 * Weights are row-major [out][in], float; inference runs in BF16 with FP32
 * accumulation. */
#define MLBM_MLP_HIDDEN 32
#define MLBM_MLP_MAX_IN 27
typedef struct {
  int n_in; /* = Q of the lattice */
  int n_hidden; /* = MLBM_MLP_HIDDEN */
  float input_scale[MLBM_MLP_MAX_IN];
  float w1[MLBM_MLP_HIDDEN * MLBM_MLP_MAX_IN];
  float b1[MLBM_MLP_HIDDEN];
  float w2[MLBM_MLP_HIDDEN * MLBM_MLP_HIDDEN];
  float b2[MLBM_MLP_HIDDEN];
  float w3[MLBM_MLP_HIDDEN];
  float b3;
  float output_scale;
} mlbm_mlp;

typedef struct {
  int epochs;
  int batch;
  float learning_rate;
  float beta1, beta2, eps; /* Adam */
  unsigned long long seed;
  float final_loss;        /* out: mean squared error of the last epoch */
} mlbm_train_cfg;

typedef struct mlbm_handle mlbm_handle;

/* Fill *cfg with the reference defaults (D2Q9 BGK, no forcing, tau 0.7,
 * reference alpha solver: tolerance 1e-8, 50 iterations, threshold 1e-3). */
int mlbm_config_init(mlbm_config* cfg);

/* Replaces the construction of Distribution + FieldList + Algorithm
 * (Distribution.h:25-30, FieldList.h:44-63, Algorithm.h:69-95). Populations are
 * zero until mlbm_init_equilibrium or mlbm_set_populations. */
int mlbm_create(const mlbm_config* cfg, mlbm_handle** out);
int mlbm_destroy(mlbm_handle* h);

/* f = f_eq(rho, u) and alpha = 2 (Initialize.h:82-116, then Algorithm::unpack,
 * Algorithm.h:141-147). rho: [V], u: [D][V] in the given layout, FP64 host
 * arrays.
 * Every host array of this interface in the DENSE layout that kernels can
 * address (page-locked memory, or any host memory on a device that accesses
 * pageable memory through the host's page tables, as NVLink-C2C systems do)
 * moves by a copy kernel over the host link; other arrays by the copy
 * engines. */
int mlbm_init_equilibrium(mlbm_handle* h, const double* rho, const double* u, int layout);

/* Populations in and out, FP64, [Q][V] in the given layout (Algorithm::pack /
 * unpack, Algorithm.h:132-147, plus the storage conversion). */
int mlbm_set_populations(mlbm_handle* h, const double* f, int layout);
int mlbm_get_populations(mlbm_handle* h, double* f, int layout);

/* nsteps fused pull steps (Algorithm::iterate, Algorithm.h:326-358), enqueued
 * on the handle's stream; flags apply to the last step. Returns once the work
 * is enqueued; mlbm_sync waits for it. */
int mlbm_step(mlbm_handle* h, int nsteps, unsigned int flags);

/* Fields stored by the last MLBM_STEP_STORE_FIELDS step (Algorithm.h:150-194):
 * rho [V], hydrodynamic velocity [D][V] (u + F/(2 rho), ForcingScheme.h:27-33),
 * alpha [V], force [D][V]. Any pointer may be NULL. Synchronizes. */
int mlbm_get_fields(mlbm_handle* h, double* rho, double* u, double* alpha, double* force,
                    int layout);

/* The per-node alpha field [V] (FP64 on the host; FP32 on the device for
 * FP32/FP16 storage): the guess the next entropic step starts from
 * (Algorithm.h:103-106). For checkpoint / restart; the reference's restart
 * re-initialises alpha to 2 (Initialize.h:82-89, 118-145). Synchronize. */
int mlbm_get_alpha(mlbm_handle* h, double* alpha, int layout);
int mlbm_set_alpha(mlbm_handle* h, const double* alpha, int layout);

/* Number of shells of the energy spectrum: the reference's maxWaveNumber()
 * (FourierDomain.h:77-79), arrayMax(globalLength) / 2, whose recursion takes
 * the minimum of the remaining lengths (Helpers.h:37-39), so
 * max(L_x, min(L_y, L_z)) / 2 with L_z = 1 on 2-D lattices. */
int mlbm_spectrum_shells(const mlbm_handle* h, int* nshells);

/* The spectral analyses the reference's Routine runs on the fields stored by
 * the last MLBM_STEP_STORE_FIELDS step (Routine.h:69-72, 126-131;
 * AnalysisList.h:55-73, 135-171), on the device (cuFFT): the vorticity
 * [2D-3][V] by the spectral curl omega_hat = i k x u_hat with integer
 * wavenumbers (Curl, Transformer.h:118-295, including its extra 1/V of
 * Curl::normalize and, in 2-D, its real part of i k x u_hat only), the total
 * energy (1/V) sum 1/2 rho |u|^2 and enstrophy (1/V) sum 1/2 |omega|^2
 * (TotalEnergy / TotalEnstrophy, Analysis.h:33-98) and the shell energy
 * spectrum [mlbm_spectrum_shells] (PowerSpectra, Analysis.h:122-177). The
 * transform buffers (about 2.5 V doubles a component) are allocated on the
 * first call. Any output may be NULL. Synchronizes. */
int mlbm_get_spectral_diagnostics(mlbm_handle* h, double* vorticity, double* energy,
                                  double* enstrophy, double* spectrum, int layout);

/* Diagnostics and solver counters of the last mlbm_step call. Synchronizes. */
int mlbm_get_diagnostics(mlbm_handle* h, mlbm_diag* out);

/* Waits for the handle's stream, polling; MLBM_ERR_TIMEOUT after timeout_ms
 * (<0: wait without limit). Then checks the device error word. */
int mlbm_sync(mlbm_handle* h, int timeout_ms);

/* The cudaStream_t the handle enqueues on (as void*), for event timing. */
int mlbm_get_stream(mlbm_handle* h, void** stream);
/* Make the handle enqueue on a caller's cudaStream_t (NULL: the handle's own). */
int mlbm_set_stream(mlbm_handle* h, void* stream);

/* Sample nodes for MLBM_STEP_LOG_SAMPLES: node indices (dense order). The log
 * of the last step is read with mlbm_get_samples: features [n][Q] = f_neq/rho
 * (FP64), alpha* [n], and solved[n] (1 when the node went through the alpha
 * solve). */
int mlbm_set_sample_nodes(mlbm_handle* h, const long long* nodes, long long n);
int mlbm_get_samples(mlbm_handle* h, double* features, double* alpha, int* solved);

/* Learned alpha guess (MLBM_GUESS_LEARNED). */
int mlbm_set_alpha_model(mlbm_handle* h, const mlbm_mlp* model);

/* Train an alpha model on the GPU with the library's own forward, backward and
 * Adam kernels. X: [n][n_in] features (f_neq/rho), y: [n] alpha*. model is
 * both the initial weights (input_scale and output_scale are kept) and the
 * result. Uses the handle's device and stream. */
int mlbm_train_alpha_model(mlbm_handle* h, const float* X, const float* y, long long n,
                           mlbm_train_cfg* cfg, mlbm_mlp* model);

/* One forward + backward pass of the model on a batch (for gradient checks):
 * loss = mean((2 + output_scale*net(x) - y)^2); gradients in mlbm_mlp layout
 * (input_scale and output_scale entries of grad are zero). */
int mlbm_alpha_model_gradient(mlbm_handle* h, const mlbm_mlp* model, const float* X,
                              const float* y, long long n, float* loss, mlbm_mlp* grad);

/* Forward pass only: guesses [n] = 2 + output_scale*net(x), with the same
 * BF16/FP32 arithmetic the fused kernel uses. */
int mlbm_alpha_model_predict(mlbm_handle* h, const mlbm_mlp* model, const float* X,
                             long long n, float* alpha);

/* Last error message of the handle (or of the last failed mlbm_create when h
 * is NULL). Never NULL. */
const char* mlbm_last_error(const mlbm_handle* h);

/* Number of CUDA kernels this library has launched in this process. */
unsigned long long mlbm_kernel_launch_count(void);

/* Allocation-free FP64 BGK step with fused diagnostics. No counterpart in the
 * reference: it exists for callers that cannot allocate device memory (a host
 * framework that owns every device allocation through its own pool, a step
 * replayed where cudaMalloc is not allowed, an embedded fixed memory budget).
 * It allocates nothing: f_in and f_out ([Q][V], dense, distinct) and
 * force_profile are the caller's device buffers; the diagnostics scratch (one
 * slot per 256-node block) is a static device array of 65,536 slots (2.5 MiB)
 * that every GPU loading the library holds until the process exits, so
 * lattices are limited to 16,777,216 nodes (256^3); larger ones return
 * MLBM_ERR_INVALID. cfg must be BGK with FP64 storage. force_profile: the
 * Kolmogorov profile A sin(2 pi i / lambda) over length[kolmogorov_axis]
 * nodes, or for Sinusoidal the three per-axis profiles concatenated (x, y, z);
 * NULL for None / Constant. Writes device diag_out[5] = {sum rho,
 * sum 1/2 rho |u|^2 (divide by V for mlbm_diag.energy), max Mach, 2, 2} and,
 * if non-NULL, the device error word to *error_word_out. Enqueued on
 * `stream` (a cudaStream_t; NULL = legacy default stream) on the current
 * device; returns before the work completes. Every call looks up the
 * scratch's device address (cudaGetSymbolAddress, no allocation); the first
 * call on a device also loads the library's device code there, so make that
 * first call before any stream capture. Every call shares the scratch: calls
 * that overlap on the GPU race. Errors: mlbm_last_error(NULL). */
int mlbm_step_f64_noalloc(const mlbm_config* cfg, const double* f_in, double* f_out,
                          const double* force_profile, double* diag_out,
                          unsigned int* error_word_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MLBM_H */
