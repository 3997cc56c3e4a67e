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

#ifdef __cplusplus
}
#endif
#endif
