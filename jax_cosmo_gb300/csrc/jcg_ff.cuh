// Float-pair ("double-float") arithmetic and elementary functions for the
// fp32c table stages.
//
// A value is hi + lo with |lo| <= ulp(hi) / 2: about 48 significant bits,
// computed on the FP32 pipe.  GB300 issues FP32 at 64 times its FP64 rate,
// so the float64-class tables that the halofit root find depends on (its
// nearest-node decisions are taken on sigma^2(R), built from P(k)) are
// formed here in float pairs: the decisions agree with float64 except within
// ~1e-14 of a boundary.
//
// Methods (each function names the one it follows):
//   sums / products      Knuth's two-sum, Dekker's two-product by FMA
//   quotient, roots      a float estimate refined by Newton steps in pairs
//   exp                  P. T. P. Tang, "Table-driven implementation of the
//                        exponential function in IEEE floating-point
//                        arithmetic", ACM TOMS 15 (1989): x = (64 m + j) ln2/64
//                        + r, 2^(j/64) from a table, e^r by its Taylor series
//                        (the leading terms in pairs, the rest in float);
//                        ln2/64 split in three parts (W. J. Cody and W. Waite,
//                        "Software Manual for the Elementary Functions", 1980)
//   log                  one Newton step on e^y = x from the float logarithm
//   sin                  Cody-Waite reduction by 2 pi (four parts) and by pi/64, then
//                        sin(a + r) = sin a cos r + cos a sin r with sin and
//                        cos of the 128 points a = j pi/64 from a table and
//                        Taylor series of sin r, cos r (|r| <= pi/128)
//   cube root            Newton steps on y^-3 = x from the float estimate
#pragma once

#include "jcg_fp32.cuh"
#include "jcg_internal.cuh"

namespace jcg {

__host__ __device__ constexpr FF ffc(double v) { return FF{(float)v, (float)(v - (double)(float)v)}; }

__device__ __forceinline__ FF ff(float v) { return FF{v, 0.f}; }
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  FF r;
  r.hi = a + b;
  const float bb = r.hi - a;
  r.lo = (a - (r.hi - bb)) + (b - bb);
  return r;
}
__device__ __forceinline__ FF operator+(FF a, FF b) { return ff_add(a, b); }
__device__ __forceinline__ FF operator-(FF a) { return FF{-a.hi, -a.lo}; }
__device__ __forceinline__ FF operator-(FF a, FF b) { return ff_add(a, -b); }
__device__ __forceinline__ FF operator*(FF a, FF b) { return ff_mul(a, b); }
__device__ __forceinline__ FF operator+(FF a, float b) {
  const FF s = ff_two_sum(a.hi, b);
  return ff_fast_two_sum(s.hi, s.lo + a.lo);
}
__device__ __forceinline__ FF operator+(float a, FF b) { return b + a; }
__device__ __forceinline__ FF operator-(FF a, float b) { return a + (-b); }
__device__ __forceinline__ FF operator-(float a, FF b) { return (-b) + a; }
__device__ __forceinline__ FF operator*(FF a, float b) {
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ FF operator*(float a, FF b) { return b * a; }
// a / b: quotient estimate q from the reciprocal, two corrections by the
// remainder a - b q formed exactly in pairs
__device__ __forceinline__ FF operator/(FF a, FF b) {
  const float rb = rcpf(b.hi);
  const float q1 = a.hi * rb;
  FF r = a - b * q1;
  const float q2 = r.hi * rb;
  r = r - b * q2;
  const float q3 = r.hi * rb;
  const FF q = ff_fast_two_sum(q1, q2);
  return q + q3;
}
__device__ __forceinline__ FF operator/(float a, FF b) { return ff(a) / b; }
__device__ __forceinline__ FF operator/(FF a, float b) { return a / ff(b); }
__device__ __forceinline__ FF ff_rcp(FF b) { return ff(1.f) / b; }
__device__ __forceinline__ FF ff_scale2(FF a, float p2) { return FF{a.hi * p2, a.lo * p2}; }  // exact
__device__ __forceinline__ FF ff_sqr(FF a) { return a * a; }
__device__ __forceinline__ double ffd(FF a) { return (double)a.hi + (double)a.lo; }

// 1 / sqrt(x), x > 0: float estimate, then y (3 - x y^2) / 2 in pairs
__device__ __forceinline__ FF ff_rsqrt(FF x) {
  const float y0 = rsqrtf(x.hi);
  const FF d = 1.f - x * ff_sqr(ff(y0));           // |d| ~ 1e-7
  return ff(y0) + ff(y0) * (d.hi * (0.5f + 0.375f * d.hi));
}
__device__ __forceinline__ FF ff_sqrt(FF x) { return x * ff_rsqrt(x); }

// x^(-1/3), x > 0: y (1 + d/3 + 2 d^2/9) with d = 1 - x y^3
__device__ __forceinline__ FF ff_rcbrt(FF x) {
  const float y0 = ex2f(-0.33333334f * lg2f(x.hi));
  const FF y3 = ff_sqr(ff(y0)) * y0;
  const FF d = 1.f - x * y3;
  const float c = d.hi * (0.33333334f + 0.22222222f * d.hi);
  return ff(y0) + ff(y0) * c;
}

// exp(x), -87 < x < 88 (Tang's table-driven method, see above).  `tab`:
// 2^(j/64), j = 0..63, as float pairs.
__device__ __forceinline__ FF ff_exp(FF x, const float2* __restrict__ tab) {
  constexpr float INV_LN2_64 = 92.33248f;                 // 64 / ln 2 (any rounding: only picks k)
  constexpr float L1 = 0x1.63p-7f;                        // ln2/64 = L1 + L2 + L3, L1 with 9 bits
  constexpr float L2 = -0x1.bd0106p-19f;
  constexpr float L3 = 0x1.cf79acp-46f;
  if (x.hi < -87.f) return ff(0.f);  // below the float range (FP64 would give < 1.6e-38)
  const float kf = rintf(x.hi * INV_LN2_64);
  const int k = (int)kf;
  // r = x - k ln2/64: k L1 exact (k < 2^13), k L2 by two-product
  FF r = x - kf * L1;
  const float p = kf * L2;
  const FF kl2 = FF{p, fmaf(kf, L2, -p)};
  r = r - kl2;
  r = r - kf * L3;
  // e^r = 1 + r + r^2/2 + r^3/6 + r^4 (1/24 + r/120), |r| <= ln2/128: the
  // quartic and higher terms (< 4e-11) in float
  const float rh = r.hi;
  const float tail = (rh * rh) * (rh * rh) * (0.041666668f + rh * 0.008333334f);
  const FF r2 = ff_sqr(r);
  const FF e = (1.f + r) + ((ff_scale2(r2, 0.5f) + (r2 * r) * ffc(1.0 / 6.0)) + tail);
  const float2 t = tab[k & 63];
  const FF m = e * FF{t.x, t.y};
  const float two_m = __int_as_float(((k >> 6) + 127) << 23);
  return ff_scale2(m, two_m);
}

// log(x), x > 0: y0 the float logarithm, t = x e^-y0 - 1, log x = y0 + t - t^2/2
__device__ __forceinline__ FF ff_log(FF x, const float2* __restrict__ tab) {
  const float y0 = LN2_F * lg2f(x.hi);
  const FF t = x * ff_exp(ff(-y0), tab) - 1.f;
  return (ff(y0) + t) - 0.5f * t.hi * t.hi;
}

// sin(x), |x| < 2^18 pi (see above), and cos(x) into *cos_out if given.
// `sc`: sin and cos of j pi/64, j = 0..127, as float pairs (sin in .x/.y of
// sc[2j], cos in sc[2j + 1]).
__device__ __forceinline__ FF ff_sin(FF x, const float2* __restrict__ sc, FF* cos_out = nullptr) {
  // by 2 pi: 2 pi = 6.25 + P2 + P3 + P4 (m 6.25 exact for m < 2^18; m P2
  // and m P3 by two-products, so that the reduced argument keeps ~1e-16
  // absolute accuracy up to the largest m)
  constexpr float P2 = 0x1.0fdaa2p-5f, P3 = 0x1.0b4612p-32f, P4 = -0x1.676734p-58f;
  const float mf = rintf(x.hi * 0.15915494f);
  FF r = x - mf * 6.25f;
  const float p = mf * P2;
  r = r - FF{p, fmaf(mf, P2, -p)};
  const float p3 = mf * P3;
  r = r - FF{p3, fmaf(mf, P3, -p3)};
  r = r - mf * P4;
  // by pi/64 = Q1 + Q2 + Q3 (n Q1 exact for |n| <= 128)
  constexpr float Q1 = 0x1.922p-5f, Q2 = -0x1.2aeef4p-23f, Q3 = -0x1.73dcb4p-48f;
  const float nf = rintf(r.hi * 20.371832f);
  r = r - nf * Q1;
  const float q = nf * Q2;
  r = r - FF{q, fmaf(nf, Q2, -q)};
  r = r - nf * Q3;
  const int j = ((int)nf) & 127;
  // |r| <= pi/128: sin r = r - r^3/6 + r^5/120, cos r = 1 - r^2/2 + r^4/24 - r^6/720
  const float rh = r.hi, r2f = rh * rh;
  const FF r2 = ff_sqr(r);
  const FF r3 = r2 * r;
  const FF sr = (r - r3 * ffc(1.0 / 6.0)) + r3.hi * r2f * 0.008333334f;
  const FF cr = (1.f - ff_scale2(r2, 0.5f)) + r2f * r2f * (0.041666668f - r2f * 0.0013888889f);
  const float2 s = sc[2 * j], c = sc[2 * j + 1];
  if (cos_out) *cos_out = FF{c.x, c.y} * cr - FF{s.x, s.y} * sr;
  return FF{s.x, s.y} * cr + FF{c.x, c.y} * sr;
}

}  // namespace jcg

// ------------------------------------------- tables as literal constants ---
// The same tables in global memory (read through L1), for code without a
// staged copy: the forward-mode tangent types below.
namespace jcg {
// 2^(j/64), j = 0..63, as float pairs (hi, lo)
__device__ const float2 kExp2FF[64] = {
    {0x1.0000000000000p+0f, 0.0f}, {0x1.02c9a40000000p+0f, -0x1.887fa00000000p-28f},
    {0x1.059b0e0000000p+0f, -0x1.9d4f520000000p-25f}, {0x1.0874520000000p+0f, -0x1.e2990e0000000p-26f},
    {0x1.0b55860000000p+0f, 0x1.9f31220000000p-25f}, {0x1.0e3ec40000000p+0f, -0x1.a585cc0000000p-25f},
    {0x1.11301e0000000p+0f, -0x1.fdb4960000000p-25f}, {0x1.1429aa0000000p+0f, 0x1.d525bc0000000p-25f},
    {0x1.172b840000000p+0f, -0x1.c157420000000p-27f}, {0x1.1a35be0000000p+0f, 0x1.6df96e0000000p-25f},
    {0x1.1d48740000000p+0f, -0x1.d2e8ca0000000p-25f}, {0x1.2063b80000000p+0f, 0x1.0c519a0000000p-25f},
    {0x1.2387a60000000p+0f, 0x1.ceac480000000p-25f}, {0x1.26b4560000000p+0f, 0x1.789f380000000p-26f},
    {0x1.29e9e00000000p+0f, -0x1.5c04240000000p-25f}, {0x1.2d285a0000000p+0f, 0x1.b900c20000000p-26f},
    {0x1.306fe00000000p+0f, 0x1.4636e20000000p-25f}, {0x1.33c08c0000000p+0f, -0x1.b37d200000000p-25f},
    {0x1.371a740000000p+0f, -0x1.18aac60000000p-25f}, {0x1.3a7db40000000p+0f, -0x1.634c020000000p-25f},
    {0x1.3dea640000000p+0f, 0x1.8246840000000p-25f}, {0x1.4160a20000000p+0f, 0x1.f72e2a0000000p-28f},
    {0x1.44e0860000000p+0f, 0x1.8624b40000000p-30f}, {0x1.486a2c0000000p+0f, -0x1.47d8660000000p-25f},
    {0x1.4bfdae0000000p+0f, -0x1.593abc0000000p-25f}, {0x1.4f9b280000000p+0f, -0x1.2c5a6c0000000p-25f},
    {0x1.5342b60000000p+0f, -0x1.2c56100000000p-25f}, {0x1.56f4740000000p+0f, -0x1.295b040000000p-25f},
    {0x1.5ab07e0000000p+0f, -0x1.5bd5ec0000000p-27f}, {0x1.5e76f20000000p+0f, -0x1.4a5bd60000000p-25f},
    {0x1.6247ec0000000p+0f, -0x1.f8b5500000000p-25f}, {0x1.6623880000000p+0f, 0x1.2a91120000000p-27f},
    {0x1.6a09e60000000p+0f, 0x1.9fcef40000000p-26f}, {0x1.6dfb240000000p+0f, -0x1.cd72e80000000p-27f},
    {0x1.71f75e0000000p+0f, 0x1.1d8bee0000000p-25f}, {0x1.75feb60000000p+0f, -0x1.37b3060000000p-25f},
    {0x1.7a11480000000p+0f, -0x1.829fd00000000p-25f}, {0x1.7e2f340000000p+0f, -0x1.2616340000000p-25f},
    {0x1.82589a0000000p+0f, -0x1.accc7c0000000p-26f}, {0x1.868d9a0000000p+0f, -0x1.2edb440000000p-26f},
    {0x1.8ace540000000p+0f, 0x1.15506e0000000p-27f}, {0x1.8f1aea0000000p+0f, -0x1.baa2320000000p-26f},
    {0x1.93737c0000000p+0f, -0x1.e647440000000p-25f}, {0x1.97d82a0000000p+0f, -0x1.0d8d840000000p-31f},
    {0x1.9c49180000000p+0f, 0x1.51f8480000000p-27f}, {0x1.a0c6680000000p+0f, -0x1.2886a60000000p-26f},
    {0x1.a5503c0000000p+0f, -0x1.b83b540000000p-25f}, {0x1.a9e6b60000000p+0f, -0x1.50c0480000000p-25f},
    {0x1.ae89fa0000000p+0f, -0x1.a94b140000000p-26f}, {0x1.b33a2c0000000p+0f, -0x1.ec3a820000000p-26f},
    {0x1.b7f7700000000p+0f, -0x1.a094380000000p-25f}, {0x1.bcc1ea0000000p+0f, -0x1.f687c60000000p-25f},
    {0x1.c199be0000000p+0f, -0x1.3d56b20000000p-27f}, {0x1.c67f120000000p+0f, 0x1.cafa2a0000000p-25f},
    {0x1.cb720e0000000p+0f, -0x1.8837cc0000000p-27f}, {0x1.d072d40000000p+0f, 0x1.40f1300000000p-25f},
    {0x1.d5818e0000000p+0f, -0x1.822dbc0000000p-27f}, {0x1.da9e600000000p+0f, 0x1.ed99420000000p-27f},
    {0x1.dfc9740000000p+0f, -0x1.908c940000000p-25f}, {0x1.e502ee0000000p+0f, 0x1.e2cffe0000000p-26f},
    {0x1.ea4afa0000000p+0f, 0x1.52486c0000000p-27f}, {0x1.efa1be0000000p+0f, 0x1.cc2b440000000p-25f},
    {0x1.f507660000000p+0f, -0x1.246eb00000000p-26f}, {0x1.fa7c180000000p+0f, 0x1.9e90d80000000p-28f},
};
// sin and cos of j pi/64, j = 0..127, interleaved, as float pairs (hi, lo)
__device__ const float2 kSinCosFF[256] = {
    {0.0f, 0.0f}, {0x1.0000000000000p+0f, 0.0f},
    {0x1.91f6600000000p-5f, -0x1.de44fe0000000p-30f}, {0x1.ff621e0000000p-1f, 0x1.bcb6be0000000p-28f},
    {0x1.917a6c0000000p-4f, -0x1.eb25ea0000000p-31f}, {0x1.fd88da0000000p-1f, 0x1.e892920000000p-28f},
    {0x1.2c81060000000p-3f, 0x1.d1cc280000000p-28f}, {0x1.fa75580000000p-1f, -0x1.eeb5d20000000p-30f},
    {0x1.8f8b840000000p-3f, -0x1.cb2cfa0000000p-30f}, {0x1.f6297c0000000p-1f, 0x1.feeb960000000p-26f},
    {0x1.f19f980000000p-3f, -0x1.37a83a0000000p-29f}, {0x1.f0a7f00000000p-1f, -0x1.1b73ca0000000p-27f},
    {0x1.2940620000000p-2f, 0x1.dab3e00000000p-27f}, {0x1.e9f4160000000p-1f, -0x1.273a440000000p-26f},
    {0x1.58f9a80000000p-2f, -0x1.4a9c040000000p-27f}, {0x1.e212100000000p-1f, 0x1.3da1ba0000000p-27f},
    {0x1.87de2a0000000p-2f, 0x1.abaa580000000p-28f}, {0x1.d906bc0000000p-1f, 0x1.e651a80000000p-26f},
    {0x1.b5d1000000000p-2f, 0x1.3c2b980000000p-27f}, {0x1.ced7b00000000p-1f, -0x1.7867120000000p-26f},
    {0x1.e2b5d40000000p-2f, -0x1.fe42720000000p-28f}, {0x1.c38b300000000p-1f, -0x1.cfe84a0000000p-26f},
    {0x1.07387a0000000p-1f, -0x1.b740040000000p-27f}, {0x1.b728340000000p-1f, 0x1.465b900000000p-27f},
    {0x1.1c73b40000000p-1f, -0x1.9465ce0000000p-27f}, {0x1.a9b6620000000p-1f, 0x1.21d4340000000p-26f},
    {0x1.30ff800000000p-1f, -0x1.8f47e60000000p-28f}, {0x1.9b3e040000000p-1f, 0x1.fce1d00000000p-27f},
    {0x1.44cf320000000p-1f, 0x1.4247760000000p-27f}, {0x1.8bc8060000000p-1f, 0x1.62a2e80000000p-26f},
    {0x1.57d6940000000p-1f, -0x1.6e626c0000000p-26f}, {0x1.7b5df20000000p-1f, 0x1.3557d80000000p-28f},
    {0x1.6a09e60000000p-1f, 0x1.9fcef40000000p-27f}, {0x1.6a09e60000000p-1f, 0x1.9fcef40000000p-27f},
    {0x1.7b5df20000000p-1f, 0x1.3557d80000000p-28f}, {0x1.57d6940000000p-1f, -0x1.6e626c0000000p-26f},
    {0x1.8bc8060000000p-1f, 0x1.62a2e80000000p-26f}, {0x1.44cf320000000p-1f, 0x1.4247760000000p-27f},
    {0x1.9b3e040000000p-1f, 0x1.fce1d00000000p-27f}, {0x1.30ff800000000p-1f, -0x1.8f47e60000000p-28f},
    {0x1.a9b6620000000p-1f, 0x1.21d4340000000p-26f}, {0x1.1c73b40000000p-1f, -0x1.9465ce0000000p-27f},
    {0x1.b728340000000p-1f, 0x1.465b900000000p-27f}, {0x1.07387a0000000p-1f, -0x1.b740040000000p-27f},
    {0x1.c38b300000000p-1f, -0x1.cfe84a0000000p-26f}, {0x1.e2b5d40000000p-2f, -0x1.fe42720000000p-28f},
    {0x1.ced7b00000000p-1f, -0x1.7867120000000p-26f}, {0x1.b5d1000000000p-2f, 0x1.3c2b980000000p-27f},
    {0x1.d906bc0000000p-1f, 0x1.e651a80000000p-26f}, {0x1.87de2a0000000p-2f, 0x1.abaa580000000p-28f},
    {0x1.e212100000000p-1f, 0x1.3da1ba0000000p-27f}, {0x1.58f9a80000000p-2f, -0x1.4a9c040000000p-27f},
    {0x1.e9f4160000000p-1f, -0x1.273a440000000p-26f}, {0x1.2940620000000p-2f, 0x1.dab3e00000000p-27f},
    {0x1.f0a7f00000000p-1f, -0x1.1b73ca0000000p-27f}, {0x1.f19f980000000p-3f, -0x1.37a83a0000000p-29f},
    {0x1.f6297c0000000p-1f, 0x1.feeb960000000p-26f}, {0x1.8f8b840000000p-3f, -0x1.cb2cfa0000000p-30f},
    {0x1.fa75580000000p-1f, -0x1.eeb5d20000000p-30f}, {0x1.2c81060000000p-3f, 0x1.d1cc280000000p-28f},
    {0x1.fd88da0000000p-1f, 0x1.e892920000000p-28f}, {0x1.917a6c0000000p-4f, -0x1.eb25ea0000000p-31f},
    {0x1.ff621e0000000p-1f, 0x1.bcb6be0000000p-28f}, {0x1.91f6600000000p-5f, -0x1.de44fe0000000p-30f},
    {0x1.0000000000000p+0f, 0.0f}, {0.0f, 0.0f},
    {0x1.ff621e0000000p-1f, 0x1.bcb6be0000000p-28f}, {-0x1.91f6600000000p-5f, 0x1.de44fe0000000p-30f},
    {0x1.fd88da0000000p-1f, 0x1.e892920000000p-28f}, {-0x1.917a6c0000000p-4f, 0x1.eb25ea0000000p-31f},
    {0x1.fa75580000000p-1f, -0x1.eeb5d20000000p-30f}, {-0x1.2c81060000000p-3f, -0x1.d1cc280000000p-28f},
    {0x1.f6297c0000000p-1f, 0x1.feeb960000000p-26f}, {-0x1.8f8b840000000p-3f, 0x1.cb2cfa0000000p-30f},
    {0x1.f0a7f00000000p-1f, -0x1.1b73ca0000000p-27f}, {-0x1.f19f980000000p-3f, 0x1.37a83a0000000p-29f},
    {0x1.e9f4160000000p-1f, -0x1.273a440000000p-26f}, {-0x1.2940620000000p-2f, -0x1.dab3e00000000p-27f},
    {0x1.e212100000000p-1f, 0x1.3da1ba0000000p-27f}, {-0x1.58f9a80000000p-2f, 0x1.4a9c040000000p-27f},
    {0x1.d906bc0000000p-1f, 0x1.e651a80000000p-26f}, {-0x1.87de2a0000000p-2f, -0x1.abaa580000000p-28f},
    {0x1.ced7b00000000p-1f, -0x1.7867120000000p-26f}, {-0x1.b5d1000000000p-2f, -0x1.3c2b980000000p-27f},
    {0x1.c38b300000000p-1f, -0x1.cfe84a0000000p-26f}, {-0x1.e2b5d40000000p-2f, 0x1.fe42720000000p-28f},
    {0x1.b728340000000p-1f, 0x1.465b900000000p-27f}, {-0x1.07387a0000000p-1f, 0x1.b740040000000p-27f},
    {0x1.a9b6620000000p-1f, 0x1.21d4340000000p-26f}, {-0x1.1c73b40000000p-1f, 0x1.9465ce0000000p-27f},
    {0x1.9b3e040000000p-1f, 0x1.fce1d00000000p-27f}, {-0x1.30ff800000000p-1f, 0x1.8f47e60000000p-28f},
    {0x1.8bc8060000000p-1f, 0x1.62a2e80000000p-26f}, {-0x1.44cf320000000p-1f, -0x1.4247760000000p-27f},
    {0x1.7b5df20000000p-1f, 0x1.3557d80000000p-28f}, {-0x1.57d6940000000p-1f, 0x1.6e626c0000000p-26f},
    {0x1.6a09e60000000p-1f, 0x1.9fcef40000000p-27f}, {-0x1.6a09e60000000p-1f, -0x1.9fcef40000000p-27f},
    {0x1.57d6940000000p-1f, -0x1.6e626c0000000p-26f}, {-0x1.7b5df20000000p-1f, -0x1.3557d80000000p-28f},
    {0x1.44cf320000000p-1f, 0x1.4247760000000p-27f}, {-0x1.8bc8060000000p-1f, -0x1.62a2e80000000p-26f},
    {0x1.30ff800000000p-1f, -0x1.8f47e60000000p-28f}, {-0x1.9b3e040000000p-1f, -0x1.fce1d00000000p-27f},
    {0x1.1c73b40000000p-1f, -0x1.9465ce0000000p-27f}, {-0x1.a9b6620000000p-1f, -0x1.21d4340000000p-26f},
    {0x1.07387a0000000p-1f, -0x1.b740040000000p-27f}, {-0x1.b728340000000p-1f, -0x1.465b900000000p-27f},
    {0x1.e2b5d40000000p-2f, -0x1.fe42720000000p-28f}, {-0x1.c38b300000000p-1f, 0x1.cfe84a0000000p-26f},
    {0x1.b5d1000000000p-2f, 0x1.3c2b980000000p-27f}, {-0x1.ced7b00000000p-1f, 0x1.7867120000000p-26f},
    {0x1.87de2a0000000p-2f, 0x1.abaa580000000p-28f}, {-0x1.d906bc0000000p-1f, -0x1.e651a80000000p-26f},
    {0x1.58f9a80000000p-2f, -0x1.4a9c040000000p-27f}, {-0x1.e212100000000p-1f, -0x1.3da1ba0000000p-27f},
    {0x1.2940620000000p-2f, 0x1.dab3e00000000p-27f}, {-0x1.e9f4160000000p-1f, 0x1.273a440000000p-26f},
    {0x1.f19f980000000p-3f, -0x1.37a83a0000000p-29f}, {-0x1.f0a7f00000000p-1f, 0x1.1b73ca0000000p-27f},
    {0x1.8f8b840000000p-3f, -0x1.cb2cfa0000000p-30f}, {-0x1.f6297c0000000p-1f, -0x1.feeb960000000p-26f},
    {0x1.2c81060000000p-3f, 0x1.d1cc280000000p-28f}, {-0x1.fa75580000000p-1f, 0x1.eeb5d20000000p-30f},
    {0x1.917a6c0000000p-4f, -0x1.eb25ea0000000p-31f}, {-0x1.fd88da0000000p-1f, -0x1.e892920000000p-28f},
    {0x1.91f6600000000p-5f, -0x1.de44fe0000000p-30f}, {-0x1.ff621e0000000p-1f, -0x1.bcb6be0000000p-28f},
    {0.0f, 0.0f}, {-0x1.0000000000000p+0f, 0.0f},
    {-0x1.91f6600000000p-5f, 0x1.de44fe0000000p-30f}, {-0x1.ff621e0000000p-1f, -0x1.bcb6be0000000p-28f},
    {-0x1.917a6c0000000p-4f, 0x1.eb25ea0000000p-31f}, {-0x1.fd88da0000000p-1f, -0x1.e892920000000p-28f},
    {-0x1.2c81060000000p-3f, -0x1.d1cc280000000p-28f}, {-0x1.fa75580000000p-1f, 0x1.eeb5d20000000p-30f},
    {-0x1.8f8b840000000p-3f, 0x1.cb2cfa0000000p-30f}, {-0x1.f6297c0000000p-1f, -0x1.feeb960000000p-26f},
    {-0x1.f19f980000000p-3f, 0x1.37a83a0000000p-29f}, {-0x1.f0a7f00000000p-1f, 0x1.1b73ca0000000p-27f},
    {-0x1.2940620000000p-2f, -0x1.dab3e00000000p-27f}, {-0x1.e9f4160000000p-1f, 0x1.273a440000000p-26f},
    {-0x1.58f9a80000000p-2f, 0x1.4a9c040000000p-27f}, {-0x1.e212100000000p-1f, -0x1.3da1ba0000000p-27f},
    {-0x1.87de2a0000000p-2f, -0x1.abaa580000000p-28f}, {-0x1.d906bc0000000p-1f, -0x1.e651a80000000p-26f},
    {-0x1.b5d1000000000p-2f, -0x1.3c2b980000000p-27f}, {-0x1.ced7b00000000p-1f, 0x1.7867120000000p-26f},
    {-0x1.e2b5d40000000p-2f, 0x1.fe42720000000p-28f}, {-0x1.c38b300000000p-1f, 0x1.cfe84a0000000p-26f},
    {-0x1.07387a0000000p-1f, 0x1.b740040000000p-27f}, {-0x1.b728340000000p-1f, -0x1.465b900000000p-27f},
    {-0x1.1c73b40000000p-1f, 0x1.9465ce0000000p-27f}, {-0x1.a9b6620000000p-1f, -0x1.21d4340000000p-26f},
    {-0x1.30ff800000000p-1f, 0x1.8f47e60000000p-28f}, {-0x1.9b3e040000000p-1f, -0x1.fce1d00000000p-27f},
    {-0x1.44cf320000000p-1f, -0x1.4247760000000p-27f}, {-0x1.8bc8060000000p-1f, -0x1.62a2e80000000p-26f},
    {-0x1.57d6940000000p-1f, 0x1.6e626c0000000p-26f}, {-0x1.7b5df20000000p-1f, -0x1.3557d80000000p-28f},
    {-0x1.6a09e60000000p-1f, -0x1.9fcef40000000p-27f}, {-0x1.6a09e60000000p-1f, -0x1.9fcef40000000p-27f},
    {-0x1.7b5df20000000p-1f, -0x1.3557d80000000p-28f}, {-0x1.57d6940000000p-1f, 0x1.6e626c0000000p-26f},
    {-0x1.8bc8060000000p-1f, -0x1.62a2e80000000p-26f}, {-0x1.44cf320000000p-1f, -0x1.4247760000000p-27f},
    {-0x1.9b3e040000000p-1f, -0x1.fce1d00000000p-27f}, {-0x1.30ff800000000p-1f, 0x1.8f47e60000000p-28f},
    {-0x1.a9b6620000000p-1f, -0x1.21d4340000000p-26f}, {-0x1.1c73b40000000p-1f, 0x1.9465ce0000000p-27f},
    {-0x1.b728340000000p-1f, -0x1.465b900000000p-27f}, {-0x1.07387a0000000p-1f, 0x1.b740040000000p-27f},
    {-0x1.c38b300000000p-1f, 0x1.cfe84a0000000p-26f}, {-0x1.e2b5d40000000p-2f, 0x1.fe42720000000p-28f},
    {-0x1.ced7b00000000p-1f, 0x1.7867120000000p-26f}, {-0x1.b5d1000000000p-2f, -0x1.3c2b980000000p-27f},
    {-0x1.d906bc0000000p-1f, -0x1.e651a80000000p-26f}, {-0x1.87de2a0000000p-2f, -0x1.abaa580000000p-28f},
    {-0x1.e212100000000p-1f, -0x1.3da1ba0000000p-27f}, {-0x1.58f9a80000000p-2f, 0x1.4a9c040000000p-27f},
    {-0x1.e9f4160000000p-1f, 0x1.273a440000000p-26f}, {-0x1.2940620000000p-2f, -0x1.dab3e00000000p-27f},
    {-0x1.f0a7f00000000p-1f, 0x1.1b73ca0000000p-27f}, {-0x1.f19f980000000p-3f, 0x1.37a83a0000000p-29f},
    {-0x1.f6297c0000000p-1f, -0x1.feeb960000000p-26f}, {-0x1.8f8b840000000p-3f, 0x1.cb2cfa0000000p-30f},
    {-0x1.fa75580000000p-1f, 0x1.eeb5d20000000p-30f}, {-0x1.2c81060000000p-3f, -0x1.d1cc280000000p-28f},
    {-0x1.fd88da0000000p-1f, -0x1.e892920000000p-28f}, {-0x1.917a6c0000000p-4f, 0x1.eb25ea0000000p-31f},
    {-0x1.ff621e0000000p-1f, -0x1.bcb6be0000000p-28f}, {-0x1.91f6600000000p-5f, 0x1.de44fe0000000p-30f},
    {-0x1.0000000000000p+0f, 0.0f}, {0.0f, 0.0f},
    {-0x1.ff621e0000000p-1f, -0x1.bcb6be0000000p-28f}, {0x1.91f6600000000p-5f, -0x1.de44fe0000000p-30f},
    {-0x1.fd88da0000000p-1f, -0x1.e892920000000p-28f}, {0x1.917a6c0000000p-4f, -0x1.eb25ea0000000p-31f},
    {-0x1.fa75580000000p-1f, 0x1.eeb5d20000000p-30f}, {0x1.2c81060000000p-3f, 0x1.d1cc280000000p-28f},
    {-0x1.f6297c0000000p-1f, -0x1.feeb960000000p-26f}, {0x1.8f8b840000000p-3f, -0x1.cb2cfa0000000p-30f},
    {-0x1.f0a7f00000000p-1f, 0x1.1b73ca0000000p-27f}, {0x1.f19f980000000p-3f, -0x1.37a83a0000000p-29f},
    {-0x1.e9f4160000000p-1f, 0x1.273a440000000p-26f}, {0x1.2940620000000p-2f, 0x1.dab3e00000000p-27f},
    {-0x1.e212100000000p-1f, -0x1.3da1ba0000000p-27f}, {0x1.58f9a80000000p-2f, -0x1.4a9c040000000p-27f},
    {-0x1.d906bc0000000p-1f, -0x1.e651a80000000p-26f}, {0x1.87de2a0000000p-2f, 0x1.abaa580000000p-28f},
    {-0x1.ced7b00000000p-1f, 0x1.7867120000000p-26f}, {0x1.b5d1000000000p-2f, 0x1.3c2b980000000p-27f},
    {-0x1.c38b300000000p-1f, 0x1.cfe84a0000000p-26f}, {0x1.e2b5d40000000p-2f, -0x1.fe42720000000p-28f},
    {-0x1.b728340000000p-1f, -0x1.465b900000000p-27f}, {0x1.07387a0000000p-1f, -0x1.b740040000000p-27f},
    {-0x1.a9b6620000000p-1f, -0x1.21d4340000000p-26f}, {0x1.1c73b40000000p-1f, -0x1.9465ce0000000p-27f},
    {-0x1.9b3e040000000p-1f, -0x1.fce1d00000000p-27f}, {0x1.30ff800000000p-1f, -0x1.8f47e60000000p-28f},
    {-0x1.8bc8060000000p-1f, -0x1.62a2e80000000p-26f}, {0x1.44cf320000000p-1f, 0x1.4247760000000p-27f},
    {-0x1.7b5df20000000p-1f, -0x1.3557d80000000p-28f}, {0x1.57d6940000000p-1f, -0x1.6e626c0000000p-26f},
    {-0x1.6a09e60000000p-1f, -0x1.9fcef40000000p-27f}, {0x1.6a09e60000000p-1f, 0x1.9fcef40000000p-27f},
    {-0x1.57d6940000000p-1f, 0x1.6e626c0000000p-26f}, {0x1.7b5df20000000p-1f, 0x1.3557d80000000p-28f},
    {-0x1.44cf320000000p-1f, -0x1.4247760000000p-27f}, {0x1.8bc8060000000p-1f, 0x1.62a2e80000000p-26f},
    {-0x1.30ff800000000p-1f, 0x1.8f47e60000000p-28f}, {0x1.9b3e040000000p-1f, 0x1.fce1d00000000p-27f},
    {-0x1.1c73b40000000p-1f, 0x1.9465ce0000000p-27f}, {0x1.a9b6620000000p-1f, 0x1.21d4340000000p-26f},
    {-0x1.07387a0000000p-1f, 0x1.b740040000000p-27f}, {0x1.b728340000000p-1f, 0x1.465b900000000p-27f},
    {-0x1.e2b5d40000000p-2f, 0x1.fe42720000000p-28f}, {0x1.c38b300000000p-1f, -0x1.cfe84a0000000p-26f},
    {-0x1.b5d1000000000p-2f, -0x1.3c2b980000000p-27f}, {0x1.ced7b00000000p-1f, -0x1.7867120000000p-26f},
    {-0x1.87de2a0000000p-2f, -0x1.abaa580000000p-28f}, {0x1.d906bc0000000p-1f, 0x1.e651a80000000p-26f},
    {-0x1.58f9a80000000p-2f, 0x1.4a9c040000000p-27f}, {0x1.e212100000000p-1f, 0x1.3da1ba0000000p-27f},
    {-0x1.2940620000000p-2f, -0x1.dab3e00000000p-27f}, {0x1.e9f4160000000p-1f, -0x1.273a440000000p-26f},
    {-0x1.f19f980000000p-3f, 0x1.37a83a0000000p-29f}, {0x1.f0a7f00000000p-1f, -0x1.1b73ca0000000p-27f},
    {-0x1.8f8b840000000p-3f, 0x1.cb2cfa0000000p-30f}, {0x1.f6297c0000000p-1f, 0x1.feeb960000000p-26f},
    {-0x1.2c81060000000p-3f, -0x1.d1cc280000000p-28f}, {0x1.fa75580000000p-1f, -0x1.eeb5d20000000p-30f},
    {-0x1.917a6c0000000p-4f, 0x1.eb25ea0000000p-31f}, {0x1.fd88da0000000p-1f, 0x1.e892920000000p-28f},
    {-0x1.91f6600000000p-5f, 0x1.de44fe0000000p-30f}, {0x1.ff621e0000000p-1f, 0x1.bcb6be0000000p-28f},
};

__device__ __forceinline__ FF ff_exp(FF x) { return ff_exp(x, kExp2FF); }
__device__ __forceinline__ FF ff_log(FF x) { return ff_log(x, kExp2FF); }
__device__ __forceinline__ FF ff_sin(FF x) { return ff_sin(x, kSinCosFF); }
__device__ __forceinline__ FF ff_sincos(FF x, FF* c) { return ff_sin(x, kSinCosFF, c); }
}  // namespace jcg

// ------------------------------------------------ physics in float pairs ---
// The fp32c table stages' per-node functions, the formulas of the FP64 forms
// in jcg_internal.cuh (same references) evaluated in float pairs.  `S`: the
// cosmology's scalars (Scalar order) as pairs; `e2`, `sc`: the exp and sin
// tables above.
namespace jcg {

struct BgF {
  FF Om, Ok, Ode, w0, wa;
};

// f_de(a) (background.py:90) with ln a given
__device__ __forceinline__ FF ff_fde(const BgF& c, FF a, FF lna) {
  return (-3.f * ((1.f + c.w0) + c.wa)) * lna + (3.f * c.wa) * (a - 1.f);
}
__device__ __forceinline__ FF ff_exp_fde(const BgF& c, FF a, FF lna, const float2* e2) {
  const FF f = ff_fde(c, a, lna);
  return (f.hi == 0.f && f.lo == 0.f) ? ff(1.f) : ff_exp(f, e2);  // w0 = -1, wa = 0: exactly 1
}

// dchi/dln a = R_H / (a sqrt(E^2(a))) (background.py:227-229)
__device__ __forceinline__ FF ff_dchi_dlna(const BgF& b, FF a, FF lna, FF ia, const float2* e2) {
  const FF ef = ff_exp_fde(b, a, lna, e2);
  const FF ia2 = ff_sqr(ia);
  const FF esq = (b.Om * (ia2 * ia) + b.Ok * ia2) + b.Ode * ef;
  return (ffc(2997.92458) * ia) * ff_rsqrt(esq);
}

// growth ODE coefficients D'' = -q D' + r D (background.py:96-106)
__device__ __forceinline__ void ff_growth_qr(const BgF& b, FF x, FF lnx, FF ix, const float2* e2, FF& q, FF& r) {
  const FF ef = ff_exp_fde(b, x, lnx, e2);
  const FF ix2 = ff_sqr(ix), ix3 = ix2 * ix;
  const FF ie2 = ff_rcp((b.Om * ix3 + b.Ok * ix2) + b.Ode * ef);
  const FF omm = (b.Om * ix3) * ie2, omde = (b.Ode * ef) * ie2;
  const FF w = b.w0 + (1.f - x) * b.wa;
  q = (2.f - ff_scale2(omm + (1.f + 3.f * w) * omde, 0.5f)) * ix;
  r = (omm * ix2) * 1.5f;
}

// Eisenstein & Hu 1998, type "eisenhu_osc" (transfer.py:107-153) at k with
// lk = log k, ik = 1 / k: the terms of eh_osc_lki
__device__ __forceinline__ FF ff_eh_osc(const FF* S, FF k, FF lk, FF ik, const float2* e2, const float2* sc) {
  const FF sh_d = S[S_SH_D];
  const FF q = k * S[S_QINV];
  const FF q108 = ff_exp(ffc(1.08) * (lk - S[S_LGQ]), e2);
  const FF Cb = 386.f / (1.f + ffc(69.9) * q108);
  const FF qq = ff_sqr(q);
  const FF L1 = ff_log(ffc(EULER_E) + (ffc(1.8) * S[S_BETA_C]) * q, e2);
  const FF L2 = ff_log(ffc(EULER_E) + ffc(1.8) * q, e2);
  const FF c142 = ffc(14.2) + Cb;
  const FF da = L1 + c142 * qq;
  const FF db = L1 + (S[S_C142AC] + Cb) * qq;
  const FF dn = L2 + c142 * qq;
  const FF dab = da * db;
  const FF r3 = ff_rcp(dab * dn);
  const FF Ta = L1 * (db * dn) * r3;
  const FF Tb = L1 * (da * dn) * r3;
  const FF Tn = L2 * dab * r3;
  const FF ksh = k * sh_d, iksh = ik * S[S_ISH];
  const FF x54 = ksh * ffc(1.0 / 5.4), x54s = ff_sqr(x54);
  const FF x52 = ksh * ffc(1.0 / 5.2);
  const FF bb = S[S_BETA_B] * iksh;
  const FF bn = S[S_BETA_NODE] * iksh;
  const FF d1 = 1.f + ff_sqr(x54s), d2 = 1.f + ff_sqr(x52), d3 = 1.f + ff_sqr(bb) * bb;
  const FF d12 = d1 * d2;
  const FF r6 = ff_rcp(d12 * d3);
  const FF f = d2 * d3 * r6;
  const FF Tc = f * Ta + (1.f - f) * Tb;
  const FF tilde_s = sh_d * ff_rcbrt(1.f + ff_sqr(bn) * bn);
  const FF silk = ff_exp(-ff_exp(ffc(1.4) * (lk - S[S_LGKSILK]), e2), e2);
  const FF arg = k * tilde_s;
  const FF sinc = ff_sin(arg, sc) / arg;
  const FF Tbar = (Tn * (d1 * d3 * r6) + S[S_ALPHA_B] * (d12 * r6) * silk) * sinc;
  return S[S_FB] * Tbar + S[S_FC] * Tc;
}

// type "eisenhu" (transfer.py:88-105)
__device__ __forceinline__ FF ff_eh_nowiggle(const FF* S, FF k, const float2* e2) {
  const FF x = ffc(0.43) * k * S[S_SH_D], x2 = ff_sqr(x);
  const FF ag = S[S_AGAM];
  const FF q = k * S[S_NWQ] / (ag + (1.f - ag) / (1.f + ff_sqr(x2)));
  const FF L = ff_log(ffc(2.0 * EULER_E) + ffc(1.8) * q, e2);
  const FF C = ffc(14.2) + 731.f / (1.f + 62.5f * q);
  return L / (L + C * ff_sqr(q));
}

template <bool NW>
__device__ __forceinline__ FF ff_eh_transfer(const FF* S, FF k, FF lk, FF ik, bool nw, const float2* e2,
                                             const float2* sc) {
  if (NW && nw) return ff_eh_nowiggle(S, k, e2);
  return ff_eh_osc(S, k, lk, ik, e2, sc);
}

}  // namespace jcg
