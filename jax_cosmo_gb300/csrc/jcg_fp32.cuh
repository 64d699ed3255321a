// FP32 building blocks of the compensated ("fp32c") integrands: MUFU forms of
// exp2 / log2 / reciprocal / sine and cosine (PTX approx instructions) and
// the constants they use.
#pragma once

namespace jcg {

__device__ __forceinline__ float ex2f(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2f(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcpf(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sinf_approx(float x) {
  float y;
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// sin(x) for x >= 0: reduce by 2 pi in two parts (Cody & Waite), then the
// hardware approximation on [-pi, pi].
__device__ __forceinline__ float sin_reduced(float x) {
  const float n = rintf(x * 0.15915494309189535f);
  float r = fmaf(-n, 6.28125f, x);                // 6.28125 = 201/32, exact products
  r = fmaf(-n, 1.9353071795864769e-3f, r);        // 2 pi - 6.28125
  return sinf_approx(r);
}

constexpr float LOG2E_F = 1.4426950408889634f;
constexpr float LN2_F = 0.6931471805599453f;
constexpr float E_F = 2.718281828459045f;
constexpr float TWO_PI2_F = 19.739208802178716f;

__device__ __forceinline__ float cosf_approx(float x) {
  float y;
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// sin and cos of x >= 0 with the same reduction as sin_reduced
__device__ __forceinline__ void sincos_reduced(float x, float* s, float* c) {
  const float n = rintf(x * 0.15915494309189535f);
  float r = fmaf(-n, 6.28125f, x);
  r = fmaf(-n, 1.9353071795864769e-3f, r);
  *s = sinf_approx(r);
  *c = cosf_approx(r);
}

}  // namespace jcg
