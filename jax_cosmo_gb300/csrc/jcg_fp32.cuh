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

// 2^f for |f| <= 0.5 + 2^-20: Taylor series of exp(f ln 2) to degree 7
// (truncation < 6e-9 relative), Horner in FP32.
__device__ __forceinline__ float exp2_frac(float f) {
  float p = 1.5252733804059840e-05f;
  p = fmaf(p, f, 1.5403530393381609e-04f);
  p = fmaf(p, f, 1.3333558146428443e-03f);
  p = fmaf(p, f, 9.6181291076284772e-03f);
  p = fmaf(p, f, 5.5504108664821580e-02f);
  p = fmaf(p, f, 2.4022650695910071e-01f);
  p = fmaf(p, f, 6.9314718055994531e-01f);
  return fmaf(p, f, 1.0f);
}

// exp(-x) for x = xh + xl (a float pair, 0 <= x <= 87): m = -x log2(e) in
// two parts (the product's rounding error recovered by an FMA), 2^m =
// 2^rint(m) * 2^frac.  Relative error a few 1e-8, independent of x's size.
__device__ __forceinline__ float exp_neg_pair(float xh, float xl) {
  constexpr float L_HI = 1.44269502162933349609375f;        // float(log2 e)
  constexpr float L_LO = 1.92596298909109e-08f;             // log2 e - L_HI
  const float mh = -xh * L_HI;
  float ml = fmaf(-xh, L_HI, -mh);
  ml = fmaf(-xh, L_LO, ml);
  ml = fmaf(-xl, L_HI, ml);
  const float nf = rintf(mh);
  const float f = (mh - nf) + ml;
  return exp2_frac(f) * __int_as_float(((int)nf + 127) << 23);
}

// ------------------------------------------------------------ float pairs --
// A value as hi + lo floats (about 48 significant bits), with the error-free
// transforms of Knuth (two-sum) and Dekker (product by FMA).
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {  // |a| >= |b|
  FF r;
  r.hi = a + b;
  r.lo = b - (r.hi - a);
  return r;
}
__device__ __forceinline__ FF ff_add(FF x, FF y) {
  const float s = x.hi + y.hi;
  const float bb = s - x.hi;
  const float e = (x.hi - (s - bb)) + (y.hi - bb);
  return ff_fast_two_sum(s, e + (x.lo + y.lo));
}
__device__ __forceinline__ FF ff_mul(FF x, FF y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ FF ff_of(double v) {
  FF r;
  r.hi = (float)v;
  r.lo = (float)(v - (double)r.hi);
  return r;
}
__device__ __forceinline__ double ff_to_double(FF x) { return (double)x.hi + (double)x.lo; }

// (ah, al) += a b with a, b float pairs: Dekker's product by FMA and Knuth's
// two-sum of the high parts; the product's low part and the two-sum's error
// gather in al (about 2^-46 relative per term; the caller forms ah + al)
__device__ __forceinline__ void ff_acc_prod(float& ah, float& al, float2 a, float2 b) {
  const float p = a.x * b.x;
  float pe = fmaf(a.x, b.x, -p);
  pe = fmaf(a.x, b.y, pe);
  pe = fmaf(a.y, b.x, pe);
  const float s = ah + p;
  const float bb = s - ah;
  al += ((ah - (s - bb)) + (p - bb)) + pe;
  ah = s;
}

}  // namespace jcg
