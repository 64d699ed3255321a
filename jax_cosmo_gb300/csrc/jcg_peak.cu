// Calibration kernels: the FP64 FMA and MUFU (ex2) issue peaks of this GPU,
// measured by the benchmark as the denominators of the FP64-bound (tables,
// halofit rows) and SFU-bound (fp32c Limber integrand) rooflines.  Each thread
// runs 8 independent dependency chains, enough to fill the pipe; the results
// are stored so that no chain is dead code.
#include "jcg_internal.cuh"
#include "../../include/jcg_calib.h"

namespace jcg {

__global__ void __launch_bounds__(256) peak_fp64_kernel(double* out, int iters, double b, double cst) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-3, a2 = a0 + 2e-3, a3 = a0 + 3e-3;
  double a4 = a0 + 4e-3, a5 = a0 + 5e-3, a6 = a0 + 6e-3, a7 = a0 + 7e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fma(a0, b, cst); a1 = fma(a1, b, cst); a2 = fma(a2, b, cst); a3 = fma(a3, b, cst);
      a4 = fma(a4, b, cst); a5 = fma(a5, b, cst); a6 = fma(a6, b, cst); a7 = fma(a7, b, cst);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void __launch_bounds__(256) peak_mufu_kernel(float* out, int iters) {
  float a0 = -threadIdx.x * 1e-6f, a1 = a0 - 0.1f, a2 = a0 - 0.2f, a3 = a0 - 0.3f;
  float a4 = a0 - 0.4f, a5 = a0 - 0.5f, a6 = a0 - 0.6f, a7 = a0 - 0.7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      // x -> -2^x stays in [-1, -0.5]
      a0 = -ex2_approx(a0); a1 = -ex2_approx(a1); a2 = -ex2_approx(a2); a3 = -ex2_approx(a3);
      a4 = -ex2_approx(a4); a5 = -ex2_approx(a5); a6 = -ex2_approx(a6); a7 = -ex2_approx(a7);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

}  // namespace jcg

using namespace jcg;

// blocks x 256 threads x iters x 16 x 8 operations (DFMA or MUFU ex2)
extern "C" int jcg_calib_peak_fp64(double* out_dev, int blocks, int iters, cudaStream_t stream) {
  if (!out_dev || blocks < 1 || iters < 1) return JCG_ERR_ARG;
  peak_fp64_kernel<<<blocks, 256, 0, stream>>>(out_dev, iters, 0.999999999, 1e-12);
  return cudaGetLastError() == cudaSuccess ? JCG_OK : JCG_ERR_CUDA;
}

extern "C" int jcg_calib_peak_mufu(float* out_dev, int blocks, int iters, cudaStream_t stream) {
  if (!out_dev || blocks < 1 || iters < 1) return JCG_ERR_ARG;
  peak_mufu_kernel<<<blocks, 256, 0, stream>>>(out_dev, iters);
  return cudaGetLastError() == cudaSuccess ? JCG_OK : JCG_ERR_CUDA;
}
