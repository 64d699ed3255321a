/* libjcg measurement tooling (not part of the angular_cl interface).
 *
 * Calibration kernels exported by libjcg.so for the benchmark: the FP64 FMA
 * and MUFU (ex2) issue peaks of the current GPU, the denominators of the
 * FP64-bound (table stages) and SFU-bound (fp32c Limber integrand) rooflines.
 * They have no counterpart in jax_cosmo and compute nothing of the path.
 * blocks x 256 threads x iters x 128 operations; out_dev holds blocks * 256
 * results.  Same conventions as jcg.h: 0 on success, asynchronous on stream.
 */
#ifndef JCG_CALIB_H
#define JCG_CALIB_H

#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

int jcg_calib_peak_fp64(double* out_dev, int blocks, int iters, cudaStream_t stream);
int jcg_calib_peak_mufu(float* out_dev, int blocks, int iters, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* JCG_CALIB_H */
