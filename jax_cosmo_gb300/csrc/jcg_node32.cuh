// The fp32c Limber integrand with its hand-written reverse sweep, shared by
// the Jacobian (jcg_grad32.cu) and the vector-Jacobian product
// (jcg_vjp32.cu): per node (cosmology, ell, a) P(k, a) = Eisenstein-Hu x
// primordial x halofit (transfer.py:107-153, power.py:42-53, 246-260) in FP32
// with MUFU ex2/lg2/rcp/sin/cos, and dP/d(inputs) in the units of the stored
// tangents (an[GTan] for the row inputs, ae[ETan] for the cosmology's
// Eisenstein-Hu inputs).
#pragma once

#include "jcg_fp32.cuh"
#include "jcg_grad.cuh"

namespace jcg {

// ---------------------------------------------------------- Limber adjoint --
// Per-cosmology Eisenstein-Hu inputs of the FP32 integrand.
struct EHg {
  float qinv, lg2_qinv, sh, inv_sh, c18bc, c142ac, alpha_b, beta_b, beta_node, lg2_ksilk, fb, fc, ns3,
      inv_keq;
  float agam, nwq;  // type "eisenhu"
};

// node32_fb for the default operator points (eisenhu_osc, takahashi2012) as
// one sweep; an[T_MUN] is not written (the caller skips that projection).
__device__ __forceinline__ float node32_fb_default(const EHg& e, const float* r, float kh, float lg2kh, float invkh,
                                           float* an, float* ae) {
  // ---- forward (same operations as node32)
  const float k = kh * r[F_INVCHI];
  const float lk = lg2kh + r[F_LG2INVCHI];
  const float invk = invkh * r[F_CHIC];
  const float q = k * e.qinv;
  const float lq = lk + e.lg2_qinv;
  const float q108 = ex2f(1.08f * lq);
  const float rden_c = rcpf(1.f + 69.9f * q108);
  const float Cb = 386.f * rden_c;
  const float A1 = E_F + e.c18bc * q;
  const float A2 = E_F + 1.8f * q;
  const float L1 = LN2_F * lg2f(A1);
  const float L2 = LN2_F * lg2f(A2);
  const float qq = q * q;
  const float cA = 14.2f + Cb, cB = e.c142ac + Cb;
  const float rDa = rcpf(L1 + cA * qq), rDb = rcpf(L1 + cB * qq), rDn = rcpf(L2 + cA * qq);
  const float Ta = L1 * rDa, Tb = L1 * rDb, Tn = L2 * rDn;
  const float ks = k * e.sh;
  const float x54 = ks * (1.f / 5.4f);
  const float x54_2 = x54 * x54;
  const float f = rcpf(1.f + x54_2 * x54_2);
  const float Tc = f * Ta + (1.f - f) * Tb;
  const float iks = invk * e.inv_sh;
  const float x52 = ks * (1.f / 5.2f);
  const float rE52 = rcpf(1.f + x52 * x52);
  const float bb = e.beta_b * iks;
  const float rBb = rcpf(1.f + bb * bb * bb);
  const float ex1 = ex2f(1.4f * (lk - e.lg2_ksilk));
  const float silk = ex2f(-LOG2E_F * ex1);
  const float bn = e.beta_node * iks;
  const float B3 = 1.f + bn * bn * bn;
  const float cbi = ex2f((-1.f / 3.f) * lg2f(B3));
  const float st = e.sh * cbi;
  const float arg = k * st;
  float sn, cs;
  sincos_reduced(arg, &sn, &cs);
  const float rarg = rcpf(arg);
  const float sinc = sn * rarg;
  const float Tbr0 = Tn * rE52 + e.alpha_b * rBb * silk;
  const float Tbar = Tbr0 * sinc;
  const float T = e.fb * Tbar + e.fc * Tc;
  const float eP = ex2f(e.ns3 * lk);
  const float T2 = T * T;
  const float d2l = eP * T2 * r[F_D2FAC];
  const float y = k * r[F_INVKNL];
  const float ly = lk - r[F_LG2KNL];
  const float efy = ex2f(-LOG2E_F * (y * (0.25f + 0.125f * y)));
  const float lg1 = lg2f(1.f + d2l);
  const float pb = ex2f(r[F_BETAN] * lg1);
  const float rden_a = rcpf(1.f + r[F_ALPHAN] * d2l);
  const float Q = pb * rden_a * efy;
  const float d2q = d2l * Q;
  const float H1 = ex2f(r[F_3F1] * ly);
  const float H2 = ex2f(r[F_F2] * ly);
  const float E3b = r[F_LG2CF3] + ly;
  const float H3 = ex2f(r[F_3MGAMMA] * E3b);
  const float rD = rcpf(1.f + r[F_BN] * H2 + H3);
  const float d2hp = r[F_AN] * H1 * rD;
  const float y2 = y * y;
  const float ryn = rcpf(y2 + r[F_NUN]);
  const float Rr = y2 * ryn;
  const float d2h = d2hp * Rr;
  const float S = d2q + d2h;
  const float ik3 = invk * invk * invk;
  const float P = TWO_PI2_F * ik3 * S;
  // ---- reverse, seed dP/dP = 1
  const float Sb = TWO_PI2_F * ik3;
  float invkb = TWO_PI2_F * S * 3.f * invk * invk;
  // d2h = d2hp y^2 / (y^2 + nu)
  const float d2hpb = Sb * Rr;
  const float Rrb = Sb * d2hp;
  const float y2b = Rrb * ryn * (1.f - Rr);
  const float NUNb = -Rrb * Rr * ryn;
  float yb = 2.f * y * y2b;
  const float ANb = d2hpb * H1 * rD;
  const float H1b = d2hpb * r[F_AN] * rD;
  const float Dbar = -d2hpb * d2hp * rD;
  const float BNb = Dbar * H2;
  const float H2b = Dbar * r[F_BN];
  const float u1 = H1b * H1 * LN2_F, u2 = H2b * H2 * LN2_F, u3 = Dbar * H3 * LN2_F;
  const float F3F1b = u1 * ly, F2b = u2 * ly, F3MGb = u3 * E3b, LG2CF3b = u3 * r[F_3MGAMMA];
  float lkb = u1 * r[F_3F1] + u2 * r[F_F2] + u3 * r[F_3MGAMMA];  // through ly
  const float LG2KNLb = -lkb;
  // d2q = d2l Q, Q = (1 + d2l)^beta / (1 + alpha d2l) exp(-f(y))
  float d2lb = Sb * Q;
  const float Qb = Sb * d2l;
  const float pbb = Qb * rden_a * efy;
  const float denab = -Qb * Q * rden_a;
  const float efyb = Qb * pb * rden_a;
  const float ALPHANb = denab * d2l;
  d2lb += denab * r[F_ALPHAN];
  const float vpb = pbb * pb * LN2_F;
  const float BETANb = vpb * lg1;
  d2lb += vpb * r[F_BETAN] * LOG2E_F * rcpf(1.f + d2l);
  yb -= efyb * efy * (0.25f + 0.25f * y);
  float kb = yb * r[F_INVKNL];
  const float INVKNLb = yb * k;
  // d2l = k^(ns+3) T^2 D2FAC
  const float ePb = d2lb * T2 * r[F_D2FAC];
  const float Tbv = d2lb * eP * 2.f * T * r[F_D2FAC];
  const float D2FACb = d2lb * eP * T2;
  const float vep = ePb * eP * LN2_F;
  const float ns3b = vep * lk;
  lkb += vep * e.ns3;
  // T = fb Tbar + fc Tc
  const float fbb = Tbv * Tbar, fcb = Tbv * Tc;
  const float Tbarb = Tbv * e.fb, Tcb = Tbv * e.fc;
  const float Tbr0b = Tbarb * sinc;
  const float sincb = Tbarb * Tbr0;
  float dsinc;
  if (arg < 0.1f) {
    const float a2 = arg * arg;
    dsinc = arg * (-1.f / 3.f + a2 * (1.f / 30.f));
  } else {
    dsinc = (cs - sinc) * rarg;
  }
  const float argb = sincb * dsinc;
  kb += argb * st;
  const float stb = argb * k;
  float shb = stb * cbi;
  const float cbib = stb * e.sh;
  const float B3b = cbib * (-1.f / 3.f) * cbi * rcpf(B3);
  const float bnb = B3b * 3.f * bn * bn;
  const float betanodeb = bnb * iks;
  float iksb = bnb * e.beta_node;
  const float Tnb = Tbr0b * rE52;
  const float E52b = -Tbr0b * Tn * rE52 * rE52;
  const float alphabb = Tbr0b * rBb * silk;
  const float Bbb = -Tbr0b * e.alpha_b * silk * rBb * rBb;
  const float silkb = Tbr0b * e.alpha_b * rBb;
  const float vex = -silkb * silk * ex1 * LN2_F * 1.4f;
  lkb += vex;
  const float lg2ksilkb = -vex;
  const float bbb = Bbb * 3.f * bb * bb;
  const float betabb = bbb * iks;
  iksb += bbb * e.beta_b;
  float ksb = E52b * 2.f * x52 * (1.f / 5.2f);
  invkb += iksb * e.inv_sh;
  const float invshb = iksb * invk;
  // Tc = f Ta + (1 - f) Tb, f = 1 / (1 + (ks / 5.4)^4)
  const float fbar = Tcb * (Ta - Tb);
  const float Tab = Tcb * f, Tbb = Tcb * (1.f - f);
  ksb -= fbar * f * f * 4.f * x54_2 * x54 * (1.f / 5.4f);
  kb += ksb * e.sh;
  shb += ksb * k;
  // Ta = L1 / (L1 + cA q^2), Tb = L1 / (L1 + cB q^2), Tn = L2 / (L2 + cA q^2)
  const float Dab = -Tab * Ta * rDa, Dbb = -Tbb * Tb * rDb, Dnb = -Tnb * Tn * rDn;
  const float L1b = Tab * rDa + Tbb * rDb + Dab + Dbb;
  const float L2b = Tnb * rDn + Dnb;
  const float cAb = (Dab + Dnb) * qq, cBb = Dbb * qq;
  const float Cbb = cAb + cBb;
  float qb = (Dab * cA + Dbb * cB + Dnb * cA) * 2.f * q;
  const float A1b = L1b * rcpf(A1), A2b = L2b * rcpf(A2);
  const float c18bcb = A1b * q;
  qb += A1b * e.c18bc + A2b * 1.8f;
  const float q108b = -Cbb * Cb * rden_c * 69.9f;
  const float lqb = q108b * q108 * LN2_F * 1.08f;
  lkb += lqb;
  kb += qb * e.qinv;
  const float qinvb = qb * k;
  // k = kh INVCHI, lk = lg2 kh + LG2INVCHI, 1/k = CHIC / kh
  const float INVCHIb = kb * kh, CHICb = invkb * invkh;
  an[T_CHIC] = -INVCHIb * r[F_INVCHI] * r[F_INVCHI] - lkb * LOG2E_F * r[F_INVCHI] + CHICb;
  an[T_D2FAC] = D2FACb;
  an[T_KNL] = -INVKNLb * r[F_INVKNL] * r[F_INVKNL] + LG2KNLb * LOG2E_F * r[F_INVKNL];
  an[T_BETAN] = BETANb;
  an[T_ALPHAN] = ALPHANb;
  an[T_AN] = ANb;
  an[T_3F1] = F3F1b;
  an[T_F2] = F2b;
  an[T_BN] = BNb;
  an[T_LG2CF3] = LG2CF3b;
  an[T_3MG] = F3MGb;
  an[T_NUN] = NUNb;
  ae[E_KEQ] = -(qinvb * e.qinv + lqb * LOG2E_F) * e.inv_keq;
  ae[E_SH] = shb - invshb * e.inv_sh * e.inv_sh;
  ae[E_C18BC] = c18bcb;
  ae[E_C142AC] = cBb;
  ae[E_ALPHAB] = alphabb;
  ae[E_BETAB] = betabb;
  ae[E_BETANODE] = betanodeb;
  ae[E_LG2KSILK] = lg2ksilkb;
  ae[E_FB] = fbb;
  ae[E_FC] = fcb;
  ae[E_NS3] = ns3b;
  return P;
}

// The power-spectrum part of node32_fb: from the transfer value T at (k, lk),
// P = k^(ns+3) T^2 D2FAC 2 pi^2 / k^3 (linear) or its halofit form
// (power.py:246-260), and the reverse sweep: an[] of the row's power inputs
// (T_D2FAC, T_KNL, T_BETAN..T_MUN), ae[E_NS3], the adjoint Tbv of T, and
// the adjoints of k, lk and 1/k accumulated into kb, lkb, invkb.  GEN =
// false: takahashi2012 only (lin and mu_n not read).
template <bool GEN>
__device__ __forceinline__ float pk32_fb(const EHg& e, const float* r, float k, float lk, float invk, float T,
                                         bool lin, float* an, float* ae, float& Tbv, float& kb, float& lkb,
                                         float& invkb) {
  const float eP = ex2f(e.ns3 * lk);
  const float T2 = T * T;
  const float d2l = eP * T2 * r[F_D2FAC];
  const float y = k * r[F_INVKNL];
  const float ly = lk - r[F_LG2KNL];
  const float efy = ex2f(-LOG2E_F * (y * (0.25f + 0.125f * y)));
  const float lg1 = lg2f(1.f + d2l);
  const float pb = ex2f(r[F_BETAN] * lg1);
  const float rden_a = rcpf(1.f + r[F_ALPHAN] * d2l);
  const float Q = pb * rden_a * efy;
  const float d2q = d2l * Q;
  const float H1 = ex2f(r[F_3F1] * ly);
  const float H2 = ex2f(r[F_F2] * ly);
  const float E3b = r[F_LG2CF3] + ly;
  const float H3 = ex2f(r[F_3MGAMMA] * E3b);
  const float rD = rcpf(1.f + r[F_BN] * H2 + H3);
  const float d2hp = r[F_AN] * H1 * rD;
  const float y2 = y * y;
  const float ryn = rcpf((GEN ? fmaf(r[F_MUN], y, y2) : y2) + r[F_NUN]);
  const float Rr = y2 * ryn;
  const float d2h = d2hp * Rr;
  const float S = (GEN && lin) ? d2l : d2q + d2h;  // lin: linear_matter_power
  const float ik3 = invk * invk * invk;
  const float P = TWO_PI2_F * ik3 * S;
  // ---- reverse, seed dP/dP = 1
  const float Sb = TWO_PI2_F * ik3;
  const float Sh = (GEN && lin) ? 0.f : Sb;  // adjoint of the halofit terms
  invkb += TWO_PI2_F * S * 3.f * invk * invk;
  // d2h = d2hp y^2 / (y^2 + mu y + nu)
  const float d2hpb = Sh * Rr;
  const float Rrb = Sh * d2hp;
  const float NUNb = -Rrb * Rr * ryn;
  const float MUNb = NUNb * y;
  float yb = GEN ? Rrb * ryn * (2.f * y * (1.f - Rr) - r[F_MUN] * Rr) : 2.f * y * (Rrb * ryn * (1.f - Rr));
  const float ANb = d2hpb * H1 * rD;
  const float H1b = d2hpb * r[F_AN] * rD;
  const float Dbar = -d2hpb * d2hp * rD;
  const float BNb = Dbar * H2;
  const float H2b = Dbar * r[F_BN];
  const float u1 = H1b * H1 * LN2_F, u2 = H2b * H2 * LN2_F, u3 = Dbar * H3 * LN2_F;
  const float F3F1b = u1 * ly, F2b = u2 * ly, F3MGb = u3 * E3b, LG2CF3b = u3 * r[F_3MGAMMA];
  const float lyb = u1 * r[F_3F1] + u2 * r[F_F2] + u3 * r[F_3MGAMMA];
  lkb += lyb;
  const float LG2KNLb = -lyb;
  // d2q = d2l Q, Q = (1 + d2l)^beta / (1 + alpha d2l) exp(-f(y))
  float d2lb = (GEN && lin) ? Sb : Sb * Q;
  const float Qb = Sh * d2l;
  const float pbb = Qb * rden_a * efy;
  const float denab = -Qb * Q * rden_a;
  const float efyb = Qb * pb * rden_a;
  const float ALPHANb = denab * d2l;
  d2lb += denab * r[F_ALPHAN];
  const float vpb = pbb * pb * LN2_F;
  const float BETANb = vpb * lg1;
  d2lb += vpb * r[F_BETAN] * LOG2E_F * rcpf(1.f + d2l);
  yb -= efyb * efy * (0.25f + 0.25f * y);
  kb += yb * r[F_INVKNL];
  const float INVKNLb = yb * k;
  // d2l = k^(ns+3) T^2 D2FAC
  const float ePb = d2lb * T2 * r[F_D2FAC];
  Tbv = d2lb * eP * 2.f * T * r[F_D2FAC];
  const float vep = ePb * eP * LN2_F;
  lkb += vep * e.ns3;
  an[T_D2FAC] = d2lb * eP * T2;
  an[T_KNL] = -INVKNLb * r[F_INVKNL] * r[F_INVKNL] + LG2KNLb * LOG2E_F * r[F_INVKNL];
  an[T_BETAN] = BETANb;
  an[T_ALPHAN] = ALPHANb;
  an[T_AN] = ANb;
  an[T_3F1] = F3F1b;
  an[T_F2] = F2b;
  an[T_BN] = BNb;
  an[T_LG2CF3] = LG2CF3b;
  an[T_3MG] = F3MGb;
  an[T_NUN] = NUNb;
  an[T_MUN] = GEN ? MUNb : 0.f;
  ae[E_NS3] = vep * lk;
  return P;
}

// P of node32 (the forward fp32c integrand) and its reverse sweep, transfer
// type "eisenhu_osc".  an[GTan] (T_CHIC..T_MUN) and ae[ETan] receive
// dP/d(input) in the units of the stored tangents.
template <bool GEN>
__device__ __forceinline__ float node32_fb(const EHg& e, const float* r, float kh, float lg2kh, float invkh,
                                           float* an, float* ae, bool lin) {
  // ---- forward (same operations as node32)
  const float k = kh * r[F_INVCHI];
  const float lk = lg2kh + r[F_LG2INVCHI];
  const float invk = invkh * r[F_CHIC];
  const float q = k * e.qinv;
  const float lq = lk + e.lg2_qinv;
  const float q108 = ex2f(1.08f * lq);
  const float rden_c = rcpf(1.f + 69.9f * q108);
  const float Cb = 386.f * rden_c;
  const float A1 = E_F + e.c18bc * q;
  const float A2 = E_F + 1.8f * q;
  const float L1 = LN2_F * lg2f(A1);
  const float L2 = LN2_F * lg2f(A2);
  const float qq = q * q;
  const float cA = 14.2f + Cb, cB = e.c142ac + Cb;
  const float rDa = rcpf(L1 + cA * qq), rDb = rcpf(L1 + cB * qq), rDn = rcpf(L2 + cA * qq);
  const float Ta = L1 * rDa, Tb = L1 * rDb, Tn = L2 * rDn;
  const float ks = k * e.sh;
  const float x54 = ks * (1.f / 5.4f);
  const float x54_2 = x54 * x54;
  const float f = rcpf(1.f + x54_2 * x54_2);
  const float Tc = f * Ta + (1.f - f) * Tb;
  const float iks = invk * e.inv_sh;
  const float x52 = ks * (1.f / 5.2f);
  const float rE52 = rcpf(1.f + x52 * x52);
  const float bb = e.beta_b * iks;
  const float rBb = rcpf(1.f + bb * bb * bb);
  const float ex1 = ex2f(1.4f * (lk - e.lg2_ksilk));
  const float silk = ex2f(-LOG2E_F * ex1);
  const float bn = e.beta_node * iks;
  const float B3 = 1.f + bn * bn * bn;
  const float cbi = ex2f((-1.f / 3.f) * lg2f(B3));
  const float st = e.sh * cbi;
  const float arg = k * st;
  float sn, cs;
  sincos_reduced(arg, &sn, &cs);
  const float rarg = rcpf(arg);
  const float sinc = sn * rarg;
  const float Tbr0 = Tn * rE52 + e.alpha_b * rBb * silk;
  const float Tbar = Tbr0 * sinc;
  const float T = e.fb * Tbar + e.fc * Tc;
  float Tbv, kb = 0.f, lkb = 0.f, invkb = 0.f;
  const float P = pk32_fb<GEN>(e, r, k, lk, invk, T, lin, an, ae, Tbv, kb, lkb, invkb);
  // T = fb Tbar + fc Tc
  const float fbb = Tbv * Tbar, fcb = Tbv * Tc;
  const float Tbarb = Tbv * e.fb, Tcb = Tbv * e.fc;
  const float Tbr0b = Tbarb * sinc;
  const float sincb = Tbarb * Tbr0;
  float dsinc;
  if (arg < 0.1f) {
    const float a2 = arg * arg;
    dsinc = arg * (-1.f / 3.f + a2 * (1.f / 30.f));
  } else {
    dsinc = (cs - sinc) * rarg;
  }
  const float argb = sincb * dsinc;
  kb += argb * st;
  const float stb = argb * k;
  float shb = stb * cbi;
  const float cbib = stb * e.sh;
  const float B3b = cbib * (-1.f / 3.f) * cbi * rcpf(B3);
  const float bnb = B3b * 3.f * bn * bn;
  const float betanodeb = bnb * iks;
  float iksb = bnb * e.beta_node;
  const float Tnb = Tbr0b * rE52;
  const float E52b = -Tbr0b * Tn * rE52 * rE52;
  const float alphabb = Tbr0b * rBb * silk;
  const float Bbb = -Tbr0b * e.alpha_b * silk * rBb * rBb;
  const float silkb = Tbr0b * e.alpha_b * rBb;
  const float vex = -silkb * silk * ex1 * LN2_F * 1.4f;
  lkb += vex;
  const float lg2ksilkb = -vex;
  const float bbb = Bbb * 3.f * bb * bb;
  const float betabb = bbb * iks;
  iksb += bbb * e.beta_b;
  float ksb = E52b * 2.f * x52 * (1.f / 5.2f);
  invkb += iksb * e.inv_sh;
  const float invshb = iksb * invk;
  // Tc = f Ta + (1 - f) Tb, f = 1 / (1 + (ks / 5.4)^4)
  const float fbar = Tcb * (Ta - Tb);
  const float Tab = Tcb * f, Tbb = Tcb * (1.f - f);
  ksb -= fbar * f * f * 4.f * x54_2 * x54 * (1.f / 5.4f);
  kb += ksb * e.sh;
  shb += ksb * k;
  // Ta = L1 / (L1 + cA q^2), Tb = L1 / (L1 + cB q^2), Tn = L2 / (L2 + cA q^2)
  const float Dab = -Tab * Ta * rDa, Dbb = -Tbb * Tb * rDb, Dnb = -Tnb * Tn * rDn;
  const float L1b = Tab * rDa + Tbb * rDb + Dab + Dbb;
  const float L2b = Tnb * rDn + Dnb;
  const float cAb = (Dab + Dnb) * qq, cBb = Dbb * qq;
  const float Cbb = cAb + cBb;
  float qb = (Dab * cA + Dbb * cB + Dnb * cA) * 2.f * q;
  const float A1b = L1b * rcpf(A1), A2b = L2b * rcpf(A2);
  const float c18bcb = A1b * q;
  qb += A1b * e.c18bc + A2b * 1.8f;
  const float q108b = -Cbb * Cb * rden_c * 69.9f;
  const float lqb = q108b * q108 * LN2_F * 1.08f;
  lkb += lqb;
  kb += qb * e.qinv;
  const float qinvb = qb * k;
  // k = kh INVCHI, lk = lg2 kh + LG2INVCHI, 1/k = CHIC / kh
  const float INVCHIb = kb * kh, CHICb = invkb * invkh;
  an[T_CHIC] = -INVCHIb * r[F_INVCHI] * r[F_INVCHI] - lkb * LOG2E_F * r[F_INVCHI] + CHICb;
  ae[E_KEQ] = -(qinvb * e.qinv + lqb * LOG2E_F) * e.inv_keq;
  ae[E_SH] = shb - invshb * e.inv_sh * e.inv_sh;
  ae[E_C18BC] = c18bcb;
  ae[E_C142AC] = cBb;
  ae[E_ALPHAB] = alphabb;
  ae[E_BETAB] = betabb;
  ae[E_BETANODE] = betanodeb;
  ae[E_LG2KSILK] = lg2ksilkb;
  ae[E_FB] = fbb;
  ae[E_FC] = fcb;
  return P;
}

// node32_fb for transfer type "eisenhu" (transfer.py:88-105).  The no-wiggle
// inputs use the slots of the oscillating fit: ae[E_AGAM] (= E_KEQ) for
// alpha_gamma, ae[E_NWQ] (= E_C18BC) for (T_cmb / 2.7)^2 / (Omega_m h),
// ae[E_SH] for the sound horizon; the other transfer slots are 0.
__device__ __forceinline__ float node32_fb_nw(const EHg& e, const float* r, float kh, float lg2kh,
                                              float invkh, float* an, float* ae, bool lin) {
  const float k = kh * r[F_INVCHI];
  const float lk = lg2kh + r[F_LG2INVCHI];
  const float invk = invkh * r[F_CHIC];
  const float x = 0.43f * k * e.sh, x2 = x * x;
  const float u = rcpf(1.f + x2 * x2);
  const float ge = e.agam + (1.f - e.agam) * u;  // gamma_eff / (Omega_m h)
  const float rge = rcpf(ge);
  const float q = k * e.nwq * rge;
  const float A = 2.f * E_F + 1.8f * q;
  const float L = LN2_F * lg2f(A);
  const float rc = rcpf(1.f + 62.5f * q);
  const float C = 14.2f + 731.f * rc;
  const float qq = q * q;
  const float rDt = rcpf(L + C * qq);
  const float T = L * rDt;
  float Tbv, kb = 0.f, lkb = 0.f, invkb = 0.f;
  const float P = pk32_fb<true>(e, r, k, lk, invk, T, lin, an, ae, Tbv, kb, lkb, invkb);
  // T = L / (L + C q^2)
  const float Lb = Tbv * rDt * (1.f - T);
  const float Dtb = -Tbv * T * rDt;
  float qb = Dtb * C * 2.f * q + Lb * 1.8f * rcpf(A);
  qb -= Dtb * qq * 731.f * 62.5f * rc * rc;
  // q = k nwq / ge, ge = agam + (1 - agam) / (1 + x^4), x = 0.43 k sh
  kb += qb * e.nwq * rge;
  const float nwqb = qb * k * rge;
  const float geb = -qb * q * rge;
  const float agamb = geb * (1.f - u);
  const float xb = -geb * (1.f - e.agam) * 4.f * x2 * x * u * u;
  kb += xb * 0.43f * e.sh;
  const float shb = xb * 0.43f * k;
  const float INVCHIb = kb * kh, CHICb = invkb * invkh;
  an[T_CHIC] = -INVCHIb * r[F_INVCHI] * r[F_INVCHI] - lkb * LOG2E_F * r[F_INVCHI] + CHICb;
#pragma unroll
  for (int j = 0; j < NET; ++j)
    if (j != E_NS3) ae[j] = 0.f;
  ae[E_AGAM] = agamb;
  ae[E_NWQ] = nwqb;
  ae[E_SH] = shb;
  return P;
}


}  // namespace jcg
