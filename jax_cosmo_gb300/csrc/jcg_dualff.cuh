// Forward-mode tangents with a float-pair value: DualFF<N> carries the value
// as a float pair (about 48 bits, FP32 pipe; jcg_ff.cuh) and N tangents in
// FP32.  It replaces DualF<N> (value in FP64) in the fp32c Jacobian's table
// stages, where the value arithmetic of the per-node evaluations (ODE
// right-hand sides, Eisenstein-Hu at the Romberg and P(k) nodes) bound the
// stage on the 1/64-rate FP64 pipe.  The interface is DualF's, so the
// templated physics of jcg_dual.cuh instantiates with it unchanged; double
// operands (grid abscissae, constants) become pairs (constants at compile
// time).  Tangent factors are formed in FP32 from the value's high part, as
// DualF forms them from the rounded FP64 value.
#pragma once

#include "jcg_dual.cuh"
#include "jcg_ff.cuh"

namespace jcg {

template <int N>
struct DualFF {
  FF v;
  float d[N];
};

template <int N>
__device__ __forceinline__ DualFF<N> ffd_const(double v) {
  DualFF<N> r;
  r.v = ff_of(v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.f;
  return r;
}
template <int N>
__device__ __forceinline__ double val(const DualFF<N>& x) {
  return ffd(x.v);
}
template <int N>
__device__ __forceinline__ DualFF<N> operator+(const DualFF<N>& a, const DualFF<N>& b) {
  DualFF<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator-(const DualFF<N>& a, const DualFF<N>& b) {
  DualFF<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator*(const DualFF<N>& a, const DualFF<N>& b) {
  DualFF<N> r;
  r.v = a.v * b.v;
  const float av = a.v.hi, bv = b.v.hi;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fmaf(a.d[i], bv, av * b.d[i]);
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator/(const DualFF<N>& a, const DualFF<N>& b) {
  DualFF<N> r;
  r.v = a.v / b.v;
  const float ib = rcpf(b.v.hi), rv = r.v.hi;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - rv * b.d[i]) * ib;
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator-(const DualFF<N>& a) {
  DualFF<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator+(const DualFF<N>& a, double b) {
  DualFF<N> r = a;
  r.v = a.v + ff_of(b);
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator+(double a, const DualFF<N>& b) {
  return b + a;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator-(const DualFF<N>& a, double b) {
  DualFF<N> r = a;
  r.v = a.v - ff_of(b);
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator-(double a, const DualFF<N>& b) {
  DualFF<N> r;
  r.v = ff_of(a) - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator*(const DualFF<N>& a, double b) {
  DualFF<N> r;
  const FF bf = ff_of(b);
  r.v = a.v * bf;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bf.hi;
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator*(double a, const DualFF<N>& b) {
  return b * a;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator/(const DualFF<N>& a, double b) {
  DualFF<N> r;
  const FF bf = ff_of(b);
  r.v = a.v / bf;
  const float ib = rcpf(bf.hi);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * ib;
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator/(double a, const DualFF<N>& b) {
  DualFF<N> r;
  r.v = ff_of(a) / b.v;
  const float s = -r.v.hi * rcpf(b.v.hi);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * b.d[i];
  return r;
}
// value v, tangents s * a.d
template <int N>
__device__ __forceinline__ DualFF<N> ffd_scale(FF v, float s, const DualFF<N>& a) {
  DualFF<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> xexp(const DualFF<N>& a) {
  const FF e = ff_exp(a.v);
  return ffd_scale(e, e.hi, a);
}
template <int N>
__device__ __forceinline__ DualFF<N> xlog(const DualFF<N>& a) {
  return ffd_scale(ff_log(a.v), rcpf(a.v.hi), a);
}
template <int N>
__device__ __forceinline__ DualFF<N> xsqrt(const DualFF<N>& a) {
  const FF s = ff_sqrt(a.v);
  return ffd_scale(s, 0.5f * rcpf(s.hi), a);
}
template <int N>
__device__ __forceinline__ DualFF<N> xcbrt(const DualFF<N>& a) {
  const FF rc = ff_rcbrt(a.v);
  const FF c = a.v * ff_sqr(rc);  // x^(1/3) = x (x^(-1/3))^2
  return ffd_scale(c, c.hi * rcpf(3.f * a.v.hi), a);
}
template <int N>
__device__ __forceinline__ DualFF<N> xsin(const DualFF<N>& a) {
  FF cs;
  const FF sn = ff_sincos(a.v, &cs);
  return ffd_scale(sn, cs.hi, a);
}
template <int N>
__device__ __forceinline__ DualFF<N> xcos(const DualFF<N>& a) {
  FF cs;
  const FF sn = ff_sincos(a.v, &cs);
  return ffd_scale(cs, -sn.hi, a);
}
template <int N>
__device__ __forceinline__ DualFF<N> xfabs(const DualFF<N>& a) {
  return a.v.hi < 0.f ? -a : a;
}
template <int N>
__device__ __forceinline__ DualFF<N> xpow(const DualFF<N>& a, double e) {
  const FF p = ff_exp(ff_of(e) * ff_log(a.v));
  return ffd_scale(p, (float)e * p.hi * rcpf(a.v.hi), a);
}
template <int N>
__device__ __forceinline__ DualFF<N> xpow(const DualFF<N>& a, const DualFF<N>& e) {
  return xexp(e * xlog(a));
}
// max / min against a constant: the selected branch's tangent (JAX's rule)
template <int N>
__device__ __forceinline__ bool ff_ge(FF a, double c) {
  const FF d = a - ff_of(c);
  return d.hi > 0.f || (d.hi == 0.f && d.lo >= 0.f);
}
template <int N>
__device__ __forceinline__ DualFF<N> xfmax(const DualFF<N>& a, double c) {
  return ff_ge<N>(a.v, c) ? a : ffd_const<N>(c);
}
template <int N>
__device__ __forceinline__ DualFF<N> xfmin(const DualFF<N>& a, double c) {
  const FF d = ff_of(c) - a.v;
  return (d.hi > 0.f || (d.hi == 0.f && d.lo >= 0.f)) ? a : ffd_const<N>(c);
}

// a float pair stored as float2 (hi, lo)
__device__ __forceinline__ FF f2ff(float2 v) { return FF{v.x, v.y}; }

// float-pair scalars (grid abscissae held as pairs: no FP64 conversions)
template <int N>
__device__ __forceinline__ DualFF<N> operator+(const DualFF<N>& a, FF b) {
  DualFF<N> r = a;
  r.v = a.v + b;
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator+(FF a, const DualFF<N>& b) {
  return b + a;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator-(const DualFF<N>& a, FF b) {
  DualFF<N> r = a;
  r.v = a.v - b;
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator-(FF a, const DualFF<N>& b) {
  DualFF<N> r;
  r.v = a - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator*(const DualFF<N>& a, FF b) {
  DualFF<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.hi;
  return r;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator*(FF a, const DualFF<N>& b) {
  return b * a;
}
template <int N>
__device__ __forceinline__ DualFF<N> operator/(FF a, const DualFF<N>& b) {
  DualFF<N> r;
  r.v = a / b.v;
  const float s = -r.v.hi * rcpf(b.v.hi);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * b.d[i];
  return r;
}
// DualFF<8> from a float-pair value (float2 hi, lo) and 8 float tangents
__device__ __forceinline__ DualFF<NDIR> ff8_of(float2 v, const float* d) {
  DualFF<NDIR> r;
  r.v = FF{v.x, v.y};
#pragma unroll
  for (int i = 0; i < NDIR; ++i) r.d[i] = d[i];
  return r;
}

// DualFF<8> from a value and 8 double tangents at stride `stride`
__device__ __forceinline__ DualFF<NDIR> ff8_of(double v, const double* d, int stride) {
  DualFF<NDIR> r;
  r.v = ff_of(v);
#pragma unroll
  for (int i = 0; i < NDIR; ++i) r.d[i] = (float)d[i * stride];
  return r;
}

}  // namespace jcg
