// Forward-mode (tangent) arithmetic for the derivative kernels, and the FP64
// physics of the tables written once for a number type T (double or Dual<N>).
//
// Dual<N> carries a value and N tangents.  The derivative kernels use it two
// ways: Dual<1> with one tangent direction per lane (8 lanes = the 8 Cosmology
// leaves of core.py:98-108; register use stays that of plain FP64), and
// Dual<8> for short per-term loops (spectral moments, lensing integrand) where
// the value part is shared by the 8 directions.
//
// Derivative conventions follow JAX's for the reference's operations:
// max(x, c) / min(x, c) pass the tangent of x where x is the selected branch;
// the interpolation segment (argmin) is locally constant.
#pragma once

#include "jcg_internal.cuh"

namespace jcg {

constexpr int NDIR = 8;  // d/d(Omega_c, Omega_b, h, n_s, sigma8, Omega_k, w0, wa)

template <int N>
struct Dual {
  double v;
  double d[N];
};

template <int N>
__device__ __forceinline__ Dual<N> dconst(double v) {
  Dual<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}

__device__ __forceinline__ double val(double x) { return x; }
template <int N>
__device__ __forceinline__ double val(const Dual<N>& x) {
  return x.v;
}

#define JCG_DUAL_BIN(OP, VEXPR, DEXPR)                                                       \
  template <int N>                                                                           \
  __device__ __forceinline__ Dual<N> operator OP(const Dual<N>& a, const Dual<N>& b) {       \
    Dual<N> r;                                                                               \
    r.v = VEXPR;                                                                             \
    _Pragma("unroll") for (int i = 0; i < N; ++i) r.d[i] = DEXPR;                            \
    return r;                                                                                \
  }

JCG_DUAL_BIN(+, a.v + b.v, a.d[i] + b.d[i])
JCG_DUAL_BIN(-, a.v - b.v, a.d[i] - b.d[i])
JCG_DUAL_BIN(*, a.v * b.v, a.d[i] * b.v + a.v * b.d[i])
#undef JCG_DUAL_BIN

template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, double b) {
  Dual<N> r = a;
  r.v = a.v + b;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(double a, const Dual<N>& b) {
  return b + a;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, double b) {
  Dual<N> r = a;
  r.v = a.v - b;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(double a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(double a, const Dual<N>& b) {
  return b * a;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v / b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(double a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a / b.v;
  const double s = -r.v / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * b.d[i];
  return r;
}

// elementary functions: xf(double) = CUDA libm, xf(Dual) = chain rule
__device__ __forceinline__ double xexp(double x) { return exp(x); }
__device__ __forceinline__ double xlog(double x) { return log(x); }
__device__ __forceinline__ double xsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ double xcbrt(double x) { return cbrt(x); }
__device__ __forceinline__ double xsin(double x) { return sin(x); }
__device__ __forceinline__ double xcos(double x) { return cos(x); }
__device__ __forceinline__ double xfabs(double x) { return fabs(x); }
__device__ __forceinline__ double xpow(double x, double e) { return pow(x, e); }
__device__ __forceinline__ double xfmax(double x, double c) { return fmax(x, c); }
__device__ __forceinline__ double xfmin(double x, double c) { return fmin(x, c); }

template <int N>
__device__ __forceinline__ Dual<N> scale_d(double v, double s, const Dual<N>& a) {
  Dual<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> xexp(const Dual<N>& a) {
  const double e = exp(a.v);
  return scale_d(e, e, a);
}
template <int N>
__device__ __forceinline__ Dual<N> xlog(const Dual<N>& a) {
  return scale_d(log(a.v), 1.0 / a.v, a);
}
template <int N>
__device__ __forceinline__ Dual<N> xsqrt(const Dual<N>& a) {
  const double s = sqrt(a.v);
  return scale_d(s, 0.5 / s, a);
}
template <int N>
__device__ __forceinline__ Dual<N> xcbrt(const Dual<N>& a) {
  const double c = cbrt(a.v);
  return scale_d(c, c / (3.0 * a.v), a);
}
template <int N>
__device__ __forceinline__ Dual<N> xsin(const Dual<N>& a) {
  return scale_d(sin(a.v), cos(a.v), a);
}
template <int N>
__device__ __forceinline__ Dual<N> xcos(const Dual<N>& a) {
  return scale_d(cos(a.v), -sin(a.v), a);
}
template <int N>
__device__ __forceinline__ Dual<N> xfabs(const Dual<N>& a) {
  return a.v < 0.0 ? -a : a;
}
template <int N>
__device__ __forceinline__ Dual<N> xpow(const Dual<N>& a, double e) {
  const double p = pow(a.v, e);
  return scale_d(p, e * p / a.v, a);
}
template <int N>
__device__ __forceinline__ Dual<N> xpow(const Dual<N>& a, const Dual<N>& e) {
  return xexp(e * xlog(a));
}
template <int N>
__device__ __forceinline__ Dual<N> xfmax(const Dual<N>& a, double c) {
  return a.v >= c ? a : dconst<N>(c);
}
template <int N>
__device__ __forceinline__ Dual<N> xfmin(const Dual<N>& a, double c) {
  return a.v <= c ? a : dconst<N>(c);
}

// ---------------------------------------------------------------- DualF ----
// Value in FP64, N tangents in FP32 (the fp32c Jacobian's table and row
// stages): the value arithmetic is exactly that of double, each tangent
// update is one FP32 operation with a factor rounded from FP64.
template <int N>
struct DualF {
  double v;
  float d[N];
};

template <int N>
__device__ __forceinline__ DualF<N> fconst(double v) {
  DualF<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.f;
  return r;
}
template <int N>
__device__ __forceinline__ double val(const DualF<N>& x) {
  return x.v;
}
template <int N>
__device__ __forceinline__ DualF<N> operator+(const DualF<N>& a, const DualF<N>& b) {
  DualF<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> operator-(const DualF<N>& a, const DualF<N>& b) {
  DualF<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> operator*(const DualF<N>& a, const DualF<N>& b) {
  DualF<N> r;
  r.v = a.v * b.v;
  const float av = (float)a.v, bv = (float)b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fmaf(a.d[i], bv, av * b.d[i]);
  return r;
}
// The tangent factors of division and the elementary functions are formed
// in FP32 from the rounded value (one float64 division per operation, not
// two): the tangents are FP32 anyway.
template <int N>
__device__ __forceinline__ DualF<N> operator/(const DualF<N>& a, const DualF<N>& b) {
  DualF<N> r;
  r.v = a.v / b.v;
  const float ib = 1.f / (float)b.v, rv = (float)r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - rv * b.d[i]) * ib;
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> operator-(const DualF<N>& a) {
  DualF<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> operator+(const DualF<N>& a, double b) {
  DualF<N> r = a;
  r.v = a.v + b;
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> operator+(double a, const DualF<N>& b) {
  return b + a;
}
template <int N>
__device__ __forceinline__ DualF<N> operator-(const DualF<N>& a, double b) {
  DualF<N> r = a;
  r.v = a.v - b;
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> operator-(double a, const DualF<N>& b) {
  DualF<N> r;
  r.v = a - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> operator*(const DualF<N>& a, double b) {
  DualF<N> r;
  r.v = a.v * b;
  const float bf = (float)b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bf;
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> operator*(double a, const DualF<N>& b) {
  return b * a;
}
template <int N>
__device__ __forceinline__ DualF<N> operator/(const DualF<N>& a, double b) {
  DualF<N> r;
  r.v = a.v / b;
  const float ib = (float)(1.0 / b);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * ib;
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> operator/(double a, const DualF<N>& b) {
  DualF<N> r;
  r.v = a / b.v;
  const float s = -(float)r.v / (float)b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> scale_f(double v, double s, const DualF<N>& a) {
  DualF<N> r;
  r.v = v;
  const float sf = (float)s;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = sf * a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> xexp(const DualF<N>& a) {
  const double e = exp(a.v);
  return scale_f(e, e, a);
}
template <int N>
__device__ __forceinline__ DualF<N> scale_ff(double v, float s, const DualF<N>& a) {
  DualF<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualF<N> xlog(const DualF<N>& a) {
  return scale_ff(log(a.v), 1.f / (float)a.v, a);
}
template <int N>
__device__ __forceinline__ DualF<N> xsqrt(const DualF<N>& a) {
  const double s = sqrt(a.v);
  return scale_ff(s, 0.5f / (float)s, a);
}
template <int N>
__device__ __forceinline__ DualF<N> xcbrt(const DualF<N>& a) {
  const double c = cbrt(a.v);
  return scale_ff(c, (float)c / (3.f * (float)a.v), a);
}
template <int N>
__device__ __forceinline__ DualF<N> xsin(const DualF<N>& a) {
  double sn, cs;
  sincos(a.v, &sn, &cs);
  return scale_f(sn, cs, a);
}
template <int N>
__device__ __forceinline__ DualF<N> xcos(const DualF<N>& a) {
  double sn, cs;
  sincos(a.v, &sn, &cs);
  return scale_f(cs, -sn, a);
}
template <int N>
__device__ __forceinline__ DualF<N> xfabs(const DualF<N>& a) {
  return a.v < 0.0 ? -a : a;
}
template <int N>
__device__ __forceinline__ DualF<N> xpow(const DualF<N>& a, double e) {
  const double p = pow(a.v, e);
  return scale_f(p, e * p / a.v, a);
}
template <int N>
__device__ __forceinline__ DualF<N> xpow(const DualF<N>& a, const DualF<N>& e) {
  return xexp(e * xlog(a));
}
template <int N>
__device__ __forceinline__ DualF<N> xfmax(const DualF<N>& a, double c) {
  return a.v >= c ? a : fconst<N>(c);
}
template <int N>
__device__ __forceinline__ DualF<N> xfmin(const DualF<N>& a, double c) {
  return a.v <= c ? a : fconst<N>(c);
}

// value of lane `src` of a warp for a Dual<1> (the tangent of direction src)
__device__ __forceinline__ Dual<1> shfl_d1(const Dual<1>& x, int src) {
  Dual<1> r;
  r.v = __shfl_sync(0xffffffffu, x.v, src);
  r.d[0] = __shfl_sync(0xffffffffu, x.d[0], src);
  return r;
}

// Gather the 8 directions held by lanes 0..7 (one Dual<1> each) into a Dual<8>.
__device__ __forceinline__ Dual<NDIR> gather8(const Dual<1>& x) {
  Dual<NDIR> r;
  r.v = __shfl_sync(0xffffffffu, x.v, 0);
#pragma unroll
  for (int i = 0; i < NDIR; ++i) r.d[i] = __shfl_sync(0xffffffffu, x.d[0], i);
  return r;
}

// ------------------------------------------------------- templated physics --
// The float64 formulas of jcg_internal.cuh / jcg_tables.cu / jcg_halofit.cu
// written for a number type T; grid abscissae (a, k) stay double.

template <class T>
struct BgT {
  T Om, Ok, Ode, w0, wa;
};

template <class T>
__device__ __forceinline__ BgT<T> make_bgT(const T* s) {
  BgT<T> b;
  b.Om = s[S_OMEGA_M];
  b.Ok = s[S_OMEGA_K];
  b.Ode = s[S_OMEGA_DE];
  b.w0 = s[S_W0];
  b.wa = s[S_WA];
  return b;
}

// background.py:90, 122-126
template <class T>
__device__ __forceinline__ T esqrT(const BgT<T>& c, double a, double lna, T* efde) {
  const T f = -3.0 * (1.0 + c.w0 + c.wa) * lna + 3.0 * c.wa * (a - 1.0);
  const T ef = xexp(f);
  if (efde) *efde = ef;
  const double ia = 1.0 / a, ia2 = ia * ia;
  return c.Om * (ia2 * ia) + c.Ok * ia2 + c.Ode * ef;
}
// background.py:168, 196
template <class T>
__device__ __forceinline__ void omT(const BgT<T>& c, double a, double lna, T& omm, T& omde) {
  T ef;
  const T e2 = esqrT(c, a, lna, &ef);
  const double ia = 1.0 / a;
  omm = c.Om * (ia * ia * ia) / e2;
  omde = c.Ode * ef / e2;
}
// background.py:294
template <class T>
__device__ __forceinline__ T dchioverdaT(const BgT<T>& c, double a, double lna) {
  return RH / ((a * a) * xsqrt(esqrT(c, a, lna, (T*)nullptr)));
}
// background.py:53
template <class T>
__device__ __forceinline__ T wT(const BgT<T>& c, double a) {
  return c.w0 + (1.0 - a) * c.wa;
}
// dchi/dln a = R_H / (a sqrt(E^2(a))) with ln a and 1 / a given (background.py:227-229, 294)
template <class T>
__device__ __forceinline__ T dchi_dlna_cT(const BgT<T>& c, double a, double lna, double ia) {
  const T f = -3.0 * (1.0 + c.w0 + c.wa) * lna + 3.0 * c.wa * (a - 1.0);
  const T ef = xexp(f);
  const double ia2 = ia * ia;
  const T e2 = c.Om * (ia2 * ia) + c.Ok * ia2 + c.Ode * ef;
  return (RH * ia) / xsqrt(e2);
}
// growth ODE coefficients with ln x and 1 / x given (background.py:96-106)
template <class T>
__device__ __forceinline__ void growth_qr_cT(const BgT<T>& b, double x, double lnx, double ix, T& q, T& r) {
  const T f = -3.0 * (1.0 + b.w0 + b.wa) * lnx + 3.0 * b.wa * (x - 1.0);
  const T ef = xexp(f);
  const double ix2 = ix * ix, ix3 = ix2 * ix;
  const T ie2 = 1.0 / (b.Om * ix3 + b.Ok * ix2 + b.Ode * ef);
  const T omm = b.Om * ix3 * ie2, omde = b.Ode * ef * ie2;
  q = (2.0 - 0.5 * (omm + (1.0 + 3.0 * wT(b, x)) * omde)) * ix;
  r = 1.5 * omm * ix2;
}
// background.py:227-229
template <class T>
__device__ __forceinline__ T dchi_dlnaT(const BgT<T>& c, double x) {
  const double xa = exp(x);
  return dchioverdaT(c, xa, x) * xa;
}
// background.py:96-106
template <class T>
__device__ __forceinline__ void growth_qrT(const BgT<T>& b, double x, T& q, T& r) {
  T omm, omde;
  omT(b, x, log(x), omm, omde);
  q = (2.0 - 0.5 * (omm + (1.0 + 3.0 * wT(b, x)) * omde)) / x;
  r = 1.5 * omm / x / x;
}

// transfer.py:47-142, core.py:145-162 (cosmo_scalars of jcg_tables.cu)
template <class T>
__device__ void cosmo_scalarsT(const T* p, T* s, bool nowiggle) {
  for (int i = 0; i < NSCAL; ++i) s[i] = T(p[0] * 0.0);
  const T Oc = p[0], Ob = p[1], h = p[2];
  s[S_OMEGA_C] = Oc;
  s[S_OMEGA_B] = Ob;
  s[S_H] = h;
  s[S_NS] = p[3];
  s[S_SIGMA8] = p[4];
  s[S_OMEGA_K] = p[5];
  s[S_W0] = p[6];
  s[S_WA] = p[7];
  const T Om = Ob + Oc;
  s[S_OMEGA_M] = Om;
  s[S_OMEGA_DE] = (1.0 - p[5]) - Om;
  const double T27 = (TCMB / 2.7) * (TCMB / 2.7);
  const T h2 = h * h;
  const T w_m = Om * h2;
  const T w_b = Ob * h2;
  const T fb = Ob / Om;
  const T fc = (Om - Ob) / Om;
  const T k_eq = 7.46e-2 * w_m / T27 / h;
  const T z_eq = 2.50e4 * w_m / (T27 * T27);
  T b1 = 0.313 * xpow(w_m, -0.419) * (1.0 + 0.607 * xpow(w_m, 0.674));
  T b2 = 0.238 * xpow(w_m, 0.223);
  const T z_d = 1291.0 * xpow(w_m, 0.251) / (1.0 + 0.659 * xpow(w_m, 0.828)) *
                (1.0 + b1 * xpow(w_b, b2));
  const T R_d = 31.5 * w_b / (T27 * T27) * (1.0e3 / z_d);
  const T R_eq = 31.5 * w_b / (T27 * T27) * (1.0e3 / z_eq);
  const T sh_d = 2.0 / (3.0 * k_eq) * xsqrt(6.0 / R_eq) *
                 xlog((xsqrt(1.0 + R_d) + xsqrt(R_eq + R_d)) / (1.0 + xsqrt(R_eq)));
  const T k_silk = 1.6 * xpow(w_b, 0.52) * xpow(w_m, 0.73) * (1.0 + xpow(10.4 * w_m, -0.95)) / h;
  const T a1 = xpow(46.9 * w_m, 0.670) * (1.0 + xpow(32.1 * w_m, -0.532));
  const T a2 = xpow(12.0 * w_m, 0.424) * (1.0 + xpow(45.0 * w_m, -0.582));
  const T alpha_c = xpow(a1, -fb) * xpow(a2, -(fb * fb * fb));
  b1 = 0.944 / (1.0 + xpow(458.0 * w_m, -0.708));
  b2 = xpow(0.395 * w_m, -0.0266);
  T beta_c = 1.0 + b1 * (xpow(fc, b2) - 1.0);
  beta_c = 1.0 / beta_c;
  const T y = (1.0 + z_eq) / (1.0 + z_d);
  const T x = xsqrt(1.0 + y);
  const T G = y * (-6.0 * x + (2.0 + 3.0 * y) * xlog((x + 1.0) / (x - 1.0)));
  const T alpha_b = 2.07 * k_eq * sh_d * xpow(1.0 + R_d, -0.75) * G;
  const T beta_node = 8.41 * xpow(w_m, 0.435);
  const T beta_b = 0.5 + fb + (3.0 - 2.0 * fb) * xsqrt((17.2 * w_m) * (17.2 * w_m) + 1.0);
  s[S_K_EQ] = k_eq;
  s[S_Z_EQ] = z_eq;
  s[S_Z_D] = z_d;
  s[S_R_D] = R_d;
  s[S_R_EQ] = R_eq;
  s[S_SH_D] = sh_d;
  s[S_K_SILK] = k_silk;
  s[S_ALPHA_C] = alpha_c;
  s[S_BETA_C] = beta_c;
  s[S_ALPHA_B] = alpha_b;
  s[S_BETA_B] = beta_b;
  s[S_BETA_NODE] = beta_node;
  s[S_FB] = fb;
  s[S_FC] = fc;
  s[S_LGQ] = xlog(13.41 * k_eq);
  s[S_LGKSILK] = xlog(k_silk);
  // transfer.py:88-100
  s[S_AGAM] = 1.0 - 0.328 * xlog(431.0 * w_m) * w_b / w_m + 0.38 * xlog(22.3 * w_m) * ((Ob / Om) * (Ob / Om));
  s[S_NWQ] = T27 / (Om * h);
  s[S_TFNW] = T(p[0] * 0.0 + (nowiggle ? 1.0 : 0.0));
}

// Shuffles of a double or a Dual<1> within a 16-lane half warp (every lane
// of the warp executes them).
__device__ __forceinline__ double shfl_t(double x, int src) { return __shfl_sync(0xffffffffu, x, src, 16); }
__device__ __forceinline__ Dual<1> shfl_t(const Dual<1>& x, int src) {
  Dual<1> r;
  r.v = __shfl_sync(0xffffffffu, x.v, src, 16);
  r.d[0] = __shfl_sync(0xffffffffu, x.d[0], src, 16);
  return r;
}

// The scalars of transfer.py:47-142 and core.py:145-162 for a 16-lane half
// warp (lane in [0, 16); both halves of the warp execute it, converged): the
// formulas and calls of the reference's order (cosmo_scalarsT), but the
// independent pow / sqrt / log calls of each level run on different lanes at
// once (one call site per function and level, lane-selected arguments,
// results broadcast by shuffles).  The chain's latency is that of 5 levels
// instead of about 25 calls.  s is written by every lane.
template <class T>
__device__ void cosmo_scalars_warpT(const T* p, T* s, int lane, bool nowiggle) {
  const T one = T(p[0] * 0.0 + 1.0);
  for (int i = 0; i < NSCAL; ++i) s[i] = T(p[0] * 0.0);
  const T Oc = p[0], Ob = p[1], h = p[2];
  s[S_OMEGA_C] = Oc;
  s[S_OMEGA_B] = Ob;
  s[S_H] = h;
  s[S_NS] = p[3];
  s[S_SIGMA8] = p[4];
  s[S_OMEGA_K] = p[5];
  s[S_W0] = p[6];
  s[S_WA] = p[7];
  const T Om = Ob + Oc;
  s[S_OMEGA_M] = Om;
  s[S_OMEGA_DE] = (1.0 - p[5]) - Om;
  const double T27 = (TCMB / 2.7) * (TCMB / 2.7);
  const T h2 = h * h;
  const T w_m = Om * h2;
  const T w_b = Ob * h2;
  const T fb = Ob / Om;
  const T fc = (Om - Ob) / Om;
  const T k_eq = 7.46e-2 * w_m / T27 / h;
  const T z_eq = 2.50e4 * w_m / (T27 * T27);
  const T R_eq = 31.5 * w_b / (T27 * T27) * (1.0e3 / z_eq);
  // level 1: pow(w, e), sqrt, log of the parameters
  T pb = one, sq = one, lg = one;
  double pe = 1.0;
  switch (lane) {
    case 0: pb = w_m, pe = -0.419; break;
    case 1: pb = w_m, pe = 0.674; break;
    case 2: pb = w_m, pe = 0.223; break;
    case 3: pb = w_m, pe = 0.251; break;
    case 4: pb = w_m, pe = 0.828; break;
    case 5: pb = w_b, pe = 0.52; break;
    case 6: pb = w_m, pe = 0.73; break;
    case 7: pb = 10.4 * w_m, pe = -0.95; break;
    case 8: pb = 46.9 * w_m, pe = 0.670; break;
    case 9: pb = 32.1 * w_m, pe = -0.532; break;
    case 10: pb = 12.0 * w_m, pe = 0.424; break;
    case 11: pb = 45.0 * w_m, pe = -0.582; break;
    case 12: pb = 458.0 * w_m, pe = -0.708; break;
    case 13: pb = 0.395 * w_m, pe = -0.0266; break;
    case 14: pb = w_m, pe = 0.435; break;
    case 15: pb = fb, pe = 3.0; break;
    default: break;
  }
  switch (lane) {
    case 0: sq = 6.0 / R_eq; break;
    case 1: sq = R_eq; break;
    case 2: sq = (17.2 * w_m) * (17.2 * w_m) + 1.0; break;
    default: break;
  }
  if (lane == 0) lg = 13.41 * k_eq;
  if (lane == 1) lg = 431.0 * w_m;
  if (lane == 2) lg = 22.3 * w_m;
  const T P1 = xpow(pb, pe), S1 = xsqrt(sq), L1 = xlog(lg);
  const T A0 = shfl_t(P1, 0), A1 = shfl_t(P1, 1), A2 = shfl_t(P1, 2), A3 = shfl_t(P1, 3);
  const T A4 = shfl_t(P1, 4), A5 = shfl_t(P1, 5), A6 = shfl_t(P1, 6), A7 = shfl_t(P1, 7);
  const T A8 = shfl_t(P1, 8), A9 = shfl_t(P1, 9), A10 = shfl_t(P1, 10), A11 = shfl_t(P1, 11);
  const T A12 = shfl_t(P1, 12), A13 = shfl_t(P1, 13), A14 = shfl_t(P1, 14), FB3 = shfl_t(P1, 15);
  const T sq6 = shfl_t(S1, 0), sqeq = shfl_t(S1, 1), sqbb = shfl_t(S1, 2);
  const T lgq = shfl_t(L1, 0), lg431 = shfl_t(L1, 1), lg223 = shfl_t(L1, 2);
  // level 2: pows with parameter-dependent exponents, log(k_silk)
  const T b1 = 0.313 * A0 * (1.0 + 0.607 * A1);
  const T b2 = 0.238 * A2;
  const T k_silk = 1.6 * A5 * A6 * (1.0 + A7) / h;
  const T a1 = A8 * (1.0 + A9);
  const T a2 = A10 * (1.0 + A11);
  const T b1c = 0.944 / (1.0 + A12);
  const T b2c = A13;
  T qb = one, qe = one;
  switch (lane) {
    case 0: qb = w_b, qe = b2; break;
    case 1: qb = a1, qe = -fb; break;
    case 2: qb = a2, qe = -FB3; break;
    case 3: qb = fc, qe = b2c; break;
    default: break;
  }
  const T P2 = xpow(qb, qe), L2 = xlog(lane == 0 ? k_silk : one);
  const T B0 = shfl_t(P2, 0), B1 = shfl_t(P2, 1), B2 = shfl_t(P2, 2), B3 = shfl_t(P2, 3);
  const T lgks = shfl_t(L2, 0);
  // level 3
  const T z_d = 1291.0 * A3 / (1.0 + 0.659 * A4) * (1.0 + b1 * B0);
  const T R_d = 31.5 * w_b / (T27 * T27) * (1.0e3 / z_d);
  const T alpha_c = B1 * B2;
  T beta_c = 1.0 + b1c * (B3 - 1.0);
  beta_c = 1.0 / beta_c;
  const T y = (1.0 + z_eq) / (1.0 + z_d);
  T sq3 = one;
  switch (lane) {
    case 0: sq3 = 1.0 + R_d; break;
    case 1: sq3 = R_eq + R_d; break;
    case 2: sq3 = 1.0 + y; break;
    default: break;
  }
  const T S3 = xsqrt(sq3), P3 = xpow(lane == 0 ? 1.0 + R_d : one, lane == 0 ? -0.75 : 1.0);
  const T C0 = shfl_t(S3, 0), C1 = shfl_t(S3, 1), x = shfl_t(S3, 2), C3 = shfl_t(P3, 0);
  // level 4
  T lg4 = one;
  if (lane == 0) lg4 = (C0 + C1) / (1.0 + sqeq);
  if (lane == 1) lg4 = (x + 1.0) / (x - 1.0);
  const T L4 = xlog(lg4);
  const T D0 = shfl_t(L4, 0), D1v = shfl_t(L4, 1);
  // level 5
  const T sh_d = 2.0 / (3.0 * k_eq) * sq6 * D0;
  const T G = y * (-6.0 * x + (2.0 + 3.0 * y) * D1v);
  const T alpha_b = 2.07 * k_eq * sh_d * C3 * G;
  const T beta_node = 8.41 * A14;
  const T beta_b = 0.5 + fb + (3.0 - 2.0 * fb) * sqbb;
  s[S_K_EQ] = k_eq;
  s[S_Z_EQ] = z_eq;
  s[S_Z_D] = z_d;
  s[S_R_D] = R_d;
  s[S_R_EQ] = R_eq;
  s[S_SH_D] = sh_d;
  s[S_K_SILK] = k_silk;
  s[S_ALPHA_C] = alpha_c;
  s[S_BETA_C] = beta_c;
  s[S_ALPHA_B] = alpha_b;
  s[S_BETA_B] = beta_b;
  s[S_BETA_NODE] = beta_node;
  s[S_FB] = fb;
  s[S_FC] = fc;
  s[S_LGQ] = lgq;
  s[S_LGKSILK] = lgks;
  s[S_QINV] = 1.0 / (13.41 * k_eq);
  s[S_ISH] = 1.0 / sh_d;
  s[S_C142AC] = 14.2 / alpha_c;
  // transfer.py:88-100
  s[S_AGAM] = 1.0 - 0.328 * lg431 * w_b / w_m + 0.38 * lg223 * ((Ob / Om) * (Ob / Om));
  s[S_NWQ] = T27 / (Om * h);
  s[S_TFNW] = T(p[0] * 0.0 + (nowiggle ? 1.0 : 0.0));
}

// transfer.py:88-105, type "eisenhu", at a fixed wavenumber k; not inlined,
// so that the oscillating fit's callers keep their registers
template <class T>
__device__ __noinline__ T eh_nowiggleT(T sh_d, T ag, T nwq, double k) {
  const T x = 0.43 * k * sh_d, x2 = x * x;
  const T q = k * nwq / (ag + (1.0 - ag) / (1.0 + x2 * x2));
  const T L = xlog(2.0 * EULER_E + 1.8 * q);
  const T C = 14.2 + 731.0 / (1.0 + 62.5 * q);
  return L / (L + C * q * q);
}

// transfer.py:107-153 at a fixed wavenumber k (lk = log k); type "eisenhu"
// (S_TFNW set) by eh_nowiggleT unless NW = false (scalars known to be of type
// "eisenhu_osc")
template <bool NW = true, class T>
__device__ __forceinline__ T eh_transferT(const T* s, double k, double lk) {
  const T k_eq = s[S_K_EQ], sh_d = s[S_SH_D];
  if (NW && val(s[S_TFNW]) != 0.0) return eh_nowiggleT(sh_d, s[S_AGAM], s[S_NWQ], k);
  const T q = k / (13.41 * k_eq);
  const T q108 = xexp(1.08 * (lk - s[S_LGQ]));
  const T Cb = 386.0 / (1.0 + 69.9 * q108);
  const T qq = q * q;
  const T L1 = xlog(EULER_E + 1.8 * s[S_BETA_C] * q);
  const T L2 = xlog(EULER_E + 1.8 * q);
  const T Ta = L1 / (L1 + (14.2 + Cb) * qq);
  const T Tb = L1 / (L1 + (14.2 / s[S_ALPHA_C] + Cb) * qq);
  const T Tn = L2 / (L2 + (14.2 + Cb) * qq);
  const T ksh = k * sh_d;
  const T x54 = ksh / 5.4, x54s = x54 * x54;
  const T f = 1.0 / (1.0 + x54s * x54s);
  const T Tc = f * Ta + (1.0 - f) * Tb;
  const T bn = s[S_BETA_NODE] / ksh;
  const T tilde_s = sh_d / xcbrt(1.0 + bn * bn * bn);
  const T x52 = ksh / 5.2;
  const T bb = s[S_BETA_B] / ksh;
  const T silk = xexp(-xexp(1.4 * (lk - s[S_LGKSILK])));
  const T arg = k * tilde_s;
  const T sinc = xsin(arg) / arg;
  const T Tbar = (Tn / (1.0 + x52 * x52) + s[S_ALPHA_B] / (1.0 + bb * bb * bb) * silk) * sinc;
  return s[S_FB] * Tbar + s[S_FC] * Tc;
}

// power.py:42-53 at a fixed wavenumber
template <bool NW = true, class T>
__device__ __forceinline__ T pk_linearT(const T* s, double k, double lk, const T& g) {
  const T t = eh_transferT<NW>(s, k, lk);
  const T pk = xexp(s[S_NS] * lk) * (t * t) * (g * g);
  return pk * s[S_PKNORM];
}

// Halofit coefficients at one scale factor from n_eff, C, Omega_m(a),
// Omega_de(a) and w(a): takahashi2012 (power.py:199-224, 235-238) or smith2003
// (power.py:182-198, 239-242, with frac = Omega_de / (1 - Omega_m) of
// power.py:180).  lcf3 = log(c_n f3); mu = 0 for takahashi2012.
template <class T>
struct HfCoef {
  T an, bn, cn, gam, alpha, beta, mu, nu, f1, f2, f3, lcf3;
};
template <class T>
__device__ __forceinline__ HfCoef<T> hf_coefs(int model, const T& n, const T& C, const T& om_m,
                                              const T& om_de, const T& w) {
  constexpr double L10 = 2.302585092994046;
  HfCoef<T> r;
  const T n2 = n * n, n3 = n2 * n, n4 = n2 * n2;
  const T lom = xlog(om_m);
  if (model == JCG_PK_SMITH2003) {
    const T e_cn = -0.2807 + 0.6669 * n + 0.3214 * n2 - 0.0793 * C;
    r.an = xexp(L10 * (1.4861 + 1.8369 * n + 1.6762 * n2 + 0.7940 * n3 + 0.1670 * n4 - 0.6206 * C));
    r.bn = xexp(L10 * (0.9463 + 0.9466 * n + 0.3084 * n2 - 0.9400 * C));
    r.cn = xexp(L10 * e_cn);
    r.gam = 0.8649 + 0.2989 * n + 0.1631 * C;
    r.alpha = 1.3884 + 0.3700 * n - 0.1452 * n2;
    r.beta = 0.8291 + 0.9854 * n + 0.3401 * n2;
    r.mu = xexp(L10 * (-3.5442 + 0.1908 * n));
    r.nu = xexp(L10 * (0.9585 + 1.2857 * n));
    const T frac = om_de / (1.0 - om_m);
    const T ofr = 1.0 - frac;
    r.f1 = frac * xexp(-0.0307 * lom) + ofr * xexp(-0.0732 * lom);
    r.f2 = frac * xexp(-0.0585 * lom) + ofr * xexp(-0.1423 * lom);
    r.f3 = frac * xexp(0.0743 * lom) + ofr * xexp(0.0725 * lom);
    r.lcf3 = L10 * e_cn + xlog(r.f3);
  } else {
    const T e_an = 1.5222 + 2.8553 * n + 2.3706 * n2 + 0.9903 * n3 + 0.2250 * n4 - 0.6038 * C +
                   0.1749 * om_de * (1.0 + w);
    const T e_bn = -0.5642 + 0.5864 * n + 0.5716 * n2 - 1.5474 * C + 0.2279 * om_de * (1.0 + w);
    const T e_cn = 0.3698 + 2.0404 * n + 0.8161 * n2 + 0.5869 * C;
    r.an = xexp(L10 * e_an);
    r.bn = xexp(L10 * e_bn);
    r.cn = xexp(L10 * e_cn);
    r.gam = 0.1971 - 0.0843 * n + 0.8460 * C;
    r.alpha = xfabs(6.0835 + 1.3373 * n - 0.1959 * n2 - 5.5274 * C);
    r.beta = 2.0379 - 0.7354 * n + 0.3157 * n2 + 1.2490 * n3 + 0.3980 * n4 - 0.1682 * C;
    r.mu = 0.0 * n;
    r.nu = xexp(L10 * (5.2105 + 3.6902 * n));
    r.f1 = xexp(-0.0307 * lom);
    r.f2 = xexp(-0.0585 * lom);
    r.f3 = xexp(0.0743 * lom);
    r.lcf3 = L10 * e_cn + 0.0743 * lom;
  }
  return r;
}

}  // namespace jcg
