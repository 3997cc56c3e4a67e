// Host-callable launchers of the mlbm kernels (plain C++ signatures).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace mlbm {

// FP64 storage, BGK collision in fixed point (step_f64x.cu): lattices 0-3,
// forcing None / Guo / Shan-Chen.
cudaError_t step_f64x(int lattice, int forcing, const double* prev, double* next,
                      const StepParams& p, cudaStream_t s);
inline bool f64x_supported(int lattice, int collision, int forcing) {
  return collision == 0 && lattice >= 0 && lattice <= 3 && forcing != FS_EDM;
}
cudaError_t step_f64x_L0(int forcing, const double* prev, double* next, const StepParams& p, cudaStream_t s);
cudaError_t step_f64x_L1(int forcing, const double* prev, double* next, const StepParams& p, cudaStream_t s);
cudaError_t step_f64x_L2(int forcing, const double* prev, double* next, const StepParams& p, cudaStream_t s);
cudaError_t step_f64x_L3(int forcing, const double* prev, double* next, const StepParams& p, cudaStream_t s);

// FP64 storage, reference arithmetic (step_f64.cu).
cudaError_t step_f64(int lattice, int collision, int forcing, const double* prev, double* next,
                     const StepParams& p, cudaStream_t s);
cudaError_t init_f64(int lattice, const double* rho, const double* u, double* f, long long V,
                     cudaStream_t s);

// BGK with FP16-shifted storage on 3-D lattices runs two z-adjacent nodes a
// thread when Lz is even (bgk_f16_pair_kernel); the number of 256-thread
// blocks of the BGK step kernel, whose partials finalize_diag sums.
inline bool bgk_pairs(int lattice, int storage, unsigned lz) {
  return storage == 2 && lattice != 0 && lz % 2 == 0;
}
inline long long bgk_step_blocks(int lattice, int storage, long long V, unsigned lz) {
  return bgk_pairs(lattice, storage, lz) ? (V / 2 + 255) / 256 : (V + 255) / 256;
}

// FP32 / FP16-shifted storage, FP32 collision (step_lowp.cu).
cudaError_t step_lowp(int lattice, int collision, int forcing, int storage, const void* prev,
                      void* next, const StepParams& p, cudaStream_t s);
cudaError_t init_lowp(int lattice, int storage, const double* rho, const double* u, void* f,
                      long long V, cudaStream_t s);
// Population q between storage and FP64 (staging buffers of V doubles).
cudaError_t lowp_to_f64(int lattice, int storage, const void* f, int q, double* out, long long V,
                        cudaStream_t s);
cudaError_t f64_to_lowp(int lattice, int storage, const double* in, int q, void* f, long long V,
                        cudaStream_t s);

// The FP64 logarithm of fastlog.cuh applied to x[0..n) (accuracy tests).
cudaError_t fast_log_eval(const double* x, double* out, long long n, const void* table,
                          cudaStream_t s);

// The entropic FP32-storage kernel's entropy function F(x), F'(x) at nodes
// given as FP32 populations and FP64 f_neq [nodes][Q] (tests); mode 0: the
// kernel's choice of form, 1: direct, 2: moment series.
cudaError_t entropy_test(int lattice, const float* f, const double* fneq, long long nodes,
                         const double* x, int nx, int mode, const void* table, const void* table_fine,
                         double* F, double* D, int* series, cudaStream_t s);
cudaError_t entropy_test_L0(const float* f, const double* fneq, long long nodes, const double* x,
                            int nx, int mode, const void* table, const void* table_fine, double* F, double* D,
                            int* series, cudaStream_t s);
cudaError_t entropy_test_L1(const float* f, const double* fneq, long long nodes, const double* x,
                            int nx, int mode, const void* table, const void* table_fine, double* F, double* D,
                            int* series, cudaStream_t s);
cudaError_t entropy_test_L2(const float* f, const double* fneq, long long nodes, const double* x,
                            int nx, int mode, const void* table, const void* table_fine, double* F, double* D,
                            int* series, cudaStream_t s);

// The FP64 kernel's entropic alpha (shortcut, limiter, solve) on single nodes
// [n][Q] (tests); p supplies the solver mode, tolerance, caps and log table.
cudaError_t alpha_solve_test(int lattice, const double* f, const double* fneq,
                             const double* guess, long long n, const StepParams& p, double* alpha,
                             int* flags, cudaStream_t s);
#define MLBM_DECL_ALPHA_TEST(N)                                                              \
  cudaError_t alpha_solve_test_L##N(const double* f, const double* fneq, const double* guess, \
                                    long long n, const StepParams& p, double* alpha,          \
                                    int* flags, cudaStream_t s);
MLBM_DECL_ALPHA_TEST(0) MLBM_DECL_ALPHA_TEST(1) MLBM_DECL_ALPHA_TEST(2)
MLBM_DECL_ALPHA_TEST(3) MLBM_DECL_ALPHA_TEST(4) MLBM_DECL_ALPHA_TEST(5)
#undef MLBM_DECL_ALPHA_TEST

// f_neq as the FP32-storage entropic main pass forms it (tests).
cudaError_t neq_test(int lattice, const float* f, long long nodes, int dfloat, double* out,
                     cudaStream_t s);
cudaError_t neq_test_L0(const float* f, long long nodes, int dfloat, double* out, cudaStream_t s);
cudaError_t neq_test_L1(const float* f, long long nodes, int dfloat, double* out, cudaStream_t s);
cudaError_t neq_test_L2(const float* f, long long nodes, int dfloat, double* out, cudaStream_t s);

// Diagnostics: sum the per-block partials in a fixed order (deterministic).
// The per-block diagnostics partials folded in a fixed order into out[5] by
// one block (finalize_diag); finalize_diag_fold does the same for long lists
// with a first level of blocks that writes finalize_diag_scratch(nblocks)
// partials behind the list (the buffer must hold them) and one block folding
// those. finalize_diag_launches: the kernels finalize_diag_fold launches.
cudaError_t finalize_diag(const double* partials, int nblocks, double* out, cudaStream_t s);
cudaError_t finalize_diag_fold(double* partials, int nblocks, double* out, cudaStream_t s);
int finalize_diag_scratch(int nblocks);
int finalize_diag_launches(int nblocks);
// n doubles from src to dst, both addresses kernels can access.
cudaError_t copy_doubles(const double* src, double* dst, long long n, cudaStream_t s);
// The alpha field filled with `value` (FP64 field a64, or alpha - 2 in the
// float field a32 when a64 is null).
cudaError_t fill_alpha_field(double* a64, float* a32, long long n, double value, cudaStream_t s);

// Sample logger: (f_neq/rho [Q], alpha) at the given nodes, from the
// pre-collision populations `prev` and the alpha field of the step just run.
cudaError_t log_samples_f64(int lattice, const double* prev, const StepParams& p,
                            const long long* nodes, long long n, double* features, double* alpha,
                            int* solved, cudaStream_t s);
cudaError_t log_samples_lowp(int lattice, int storage, const void* prev, const StepParams& p,
                             const long long* nodes, long long n, double* features, double* alpha,
                             int* solved, cudaStream_t s);
cudaError_t log_samples(int lattice, int storage, const void* prev, const StepParams& p,
                        const long long* nodes, long long n, double* features, double* alpha,
                        int* solved, cudaStream_t s);

// Spectral forces (spectral_force.cu): a force field [D][V] on the device,
// computed once (ConstantShell) or before every step from the stored fields
// (EnergyRemoval, Turbulent2D). Functions return 0 on success, else write a
// message to err.
void count_launches(unsigned n);
struct SpectralForce;
// want_float: also keep a float copy of the field (FP32/FP16 storage).
int spectral_force_create(SpectralForce** out, int force, int D, int lx, int ly, int lz,
                          const double amp[3], int kmin, int kmax, const double ramp[3],
                          int rkmin, int rkmax, int want_float, cudaStream_t s, char* err,
                          size_t errlen);
int spectral_force_update(SpectralForce* sf, const double* rho, const double* u, cudaStream_t s,
                          char* err, size_t errlen);
const double* spectral_force_field(const SpectralForce* sf);
const float* spectral_force_field_f(const SpectralForce* sf);
bool spectral_force_time_dependent(const SpectralForce* sf);
void spectral_force_destroy(SpectralForce* sf);

// Spectral analyses of the stored fields (spectral_diag.cu): vorticity,
// energy, enstrophy, shell spectrum. Functions return 0 on success, else
// write a message to err.
struct SpectralDiag;
int spectral_diag_shells(int D, int lx, int ly, int lz);
int spectral_diag_create(SpectralDiag** out, int D, int lx, int ly, int lz, cudaStream_t s,
                         char* err, size_t errlen);
void spectral_diag_destroy(SpectralDiag* sd);
int spectral_diag_nshells(const SpectralDiag* sd);
long long spectral_diag_volume(const SpectralDiag* sd);
// device [energy, enstrophy, spectrum[nshells]]
const double* spectral_diag_results(const SpectralDiag* sd);
const double* spectral_diag_vorticity(const SpectralDiag* sd);
int spectral_diag_run(SpectralDiag* sd, const double* rho, const double* u, cudaStream_t s,
                      char* err, size_t errlen);
int spectral_diag_curl(SpectralDiag* sd, int c, cudaStream_t s, char* err, size_t errlen);

// Per-lattice (and per-storage) entry points, one translation unit each.
cudaError_t step_f64_L0(int collision, int forcing, const double* prev, double* next, const StepParams& p, cudaStream_t s);
cudaError_t init_f64_L0(const double* rho, const double* u, double* f, long long V, cudaStream_t s);
cudaError_t log_samples_f64_L0(const double* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_lowp_L0_S1(int collision, int fs, const void* prev, void* next, const StepParams& p, cudaStream_t s);
cudaError_t init_lowp_L0_S1(const double* rho, const double* u, void* f, long long V, cudaStream_t s);
cudaError_t lowp_to_f64_L0_S1(const void* f, int q, double* out, long long V, cudaStream_t s);
cudaError_t f64_to_lowp_L0_S1(const double* in, int q, void* f, long long V, cudaStream_t s);
cudaError_t log_samples_lowp_L0_S1(const void* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_lowp_L0_S2(int collision, int fs, const void* prev, void* next, const StepParams& p, cudaStream_t s);
cudaError_t init_lowp_L0_S2(const double* rho, const double* u, void* f, long long V, cudaStream_t s);
cudaError_t lowp_to_f64_L0_S2(const void* f, int q, double* out, long long V, cudaStream_t s);
cudaError_t f64_to_lowp_L0_S2(const double* in, int q, void* f, long long V, cudaStream_t s);
cudaError_t log_samples_lowp_L0_S2(const void* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_f64_L1(int collision, int forcing, const double* prev, double* next, const StepParams& p, cudaStream_t s);
cudaError_t init_f64_L1(const double* rho, const double* u, double* f, long long V, cudaStream_t s);
cudaError_t log_samples_f64_L1(const double* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_lowp_L1_S1(int collision, int fs, const void* prev, void* next, const StepParams& p, cudaStream_t s);
cudaError_t init_lowp_L1_S1(const double* rho, const double* u, void* f, long long V, cudaStream_t s);
cudaError_t lowp_to_f64_L1_S1(const void* f, int q, double* out, long long V, cudaStream_t s);
cudaError_t f64_to_lowp_L1_S1(const double* in, int q, void* f, long long V, cudaStream_t s);
cudaError_t log_samples_lowp_L1_S1(const void* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_lowp_L1_S2(int collision, int fs, const void* prev, void* next, const StepParams& p, cudaStream_t s);
cudaError_t init_lowp_L1_S2(const double* rho, const double* u, void* f, long long V, cudaStream_t s);
cudaError_t lowp_to_f64_L1_S2(const void* f, int q, double* out, long long V, cudaStream_t s);
cudaError_t f64_to_lowp_L1_S2(const double* in, int q, void* f, long long V, cudaStream_t s);
cudaError_t log_samples_lowp_L1_S2(const void* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_f64_L2(int collision, int forcing, const double* prev, double* next, const StepParams& p, cudaStream_t s);
cudaError_t init_f64_L2(const double* rho, const double* u, double* f, long long V, cudaStream_t s);
cudaError_t log_samples_f64_L2(const double* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
// D3Q15 with FP32 / FP16-shifted storage
cudaError_t step_lowp_L3_S1(int collision, int fs, const void* prev, void* next, const StepParams& p, cudaStream_t s);
cudaError_t init_lowp_L3_S1(const double* rho, const double* u, void* f, long long V, cudaStream_t s);
cudaError_t lowp_to_f64_L3_S1(const void* f, int q, double* out, long long V, cudaStream_t s);
cudaError_t f64_to_lowp_L3_S1(const double* in, int q, void* f, long long V, cudaStream_t s);
cudaError_t log_samples_lowp_L3_S1(const void* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_lowp_L3_S2(int collision, int fs, const void* prev, void* next, const StepParams& p, cudaStream_t s);
cudaError_t init_lowp_L3_S2(const double* rho, const double* u, void* f, long long V, cudaStream_t s);
cudaError_t lowp_to_f64_L3_S2(const void* f, int q, double* out, long long V, cudaStream_t s);
cudaError_t f64_to_lowp_L3_S2(const double* in, int q, void* f, long long V, cudaStream_t s);
cudaError_t log_samples_lowp_L3_S2(const void* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
// D3Q15, D2Q13, D3Q33 with FP64 storage
cudaError_t step_f64_L3(int collision, int forcing, const double* prev, double* next, const StepParams& p, cudaStream_t s);
cudaError_t init_f64_L3(const double* rho, const double* u, double* f, long long V, cudaStream_t s);
cudaError_t log_samples_f64_L3(const double* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_f64_L4(int collision, int forcing, const double* prev, double* next, const StepParams& p, cudaStream_t s);
cudaError_t init_f64_L4(const double* rho, const double* u, double* f, long long V, cudaStream_t s);
cudaError_t log_samples_f64_L4(const double* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_f64_L5(int collision, int forcing, const double* prev, double* next, const StepParams& p, cudaStream_t s);
cudaError_t init_f64_L5(const double* rho, const double* u, double* f, long long V, cudaStream_t s);
cudaError_t log_samples_f64_L5(const double* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_lowp_L2_S1(int collision, int fs, const void* prev, void* next, const StepParams& p, cudaStream_t s);
cudaError_t init_lowp_L2_S1(const double* rho, const double* u, void* f, long long V, cudaStream_t s);
cudaError_t lowp_to_f64_L2_S1(const void* f, int q, double* out, long long V, cudaStream_t s);
cudaError_t f64_to_lowp_L2_S1(const double* in, int q, void* f, long long V, cudaStream_t s);
cudaError_t log_samples_lowp_L2_S1(const void* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);
cudaError_t step_lowp_L2_S2(int collision, int fs, const void* prev, void* next, const StepParams& p, cudaStream_t s);
cudaError_t init_lowp_L2_S2(const double* rho, const double* u, void* f, long long V, cudaStream_t s);
cudaError_t lowp_to_f64_L2_S2(const void* f, int q, double* out, long long V, cudaStream_t s);
cudaError_t f64_to_lowp_L2_S2(const double* in, int q, void* f, long long V, cudaStream_t s);
cudaError_t log_samples_lowp_L2_S2(const void* prev, const StepParams& p, const long long* nodes, long long n, double* features, double* alpha, int* solved, cudaStream_t s);

}  // namespace mlbm
