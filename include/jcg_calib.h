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
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

int jcg_calib_peak_fp64(double* out_dev, int blocks, int iters, cudaStream_t stream);
int jcg_calib_peak_mufu(float* out_dev, int blocks, int iters, cudaStream_t stream);

/* Stage timing of the fp32c vector-Jacobian product (jcg_angular_cl_vjp with
 * precision JCG_FP32C, gamma_dir -1): runs only the stages in stage_mask on a
 * workspace that a full call with the same arguments filled, so that each
 * stage can be timed alone.  Bits: 1 tables (scalars, node evaluations,
 * tables, moments), 2 rows, 4 radial kernels, 8 product kernel (with the
 * partial C_ell when cl is given), 16 reverse lensing and the gradient sum. */
struct jcg_geometry;
int jcg_calib_vjp_stages(const struct jcg_geometry* g, const void* geo_dev, const double* params_dev, int n_cosmo,
                         const double* cl_bar_dev, double* cl_dev, double* grad_dev, void* ws, size_t ws_bytes,
                         unsigned stage_mask, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* JCG_CALIB_H */
