// Halofit parameters per Limber node (FP64) and pointwise table queries.
//
// Phase 1, one warp per scale-factor node: the sigma^2(R) root find of
// power.py:96-118 and the spectral moments of power.py:121-139.
// Phase 2, one thread per node: the takahashi2012 coefficients of
// power.py:177-238 and the Limber weights.  (Scalar per-node work done by one
// lane of a warp would hold the float64 pipe for all 32 lanes; GB300's FP64
// rate is ~1/70 of its FP32 rate, so the per-node scalar work runs
// thread-parallel instead.)
#include "jcg_fp32.cuh"
#include "jcg_ff.cuh"
#include "jcg_internal.cuh"
#include "jcg_dual.cuh"

namespace jcg {

constexpr double TWO_PI2 = 2.0 * (PI * PI);  // 2.0 * np.pi**2
constexpr double C2 = C_KMS * C_KMS;          // const.c**2

struct HfParams {
  double knl, neff, C;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// argmin_j (1 - sig_j g2)^2 with the first index on ties (scipy/interpolate.py:47).
// v_j = sig_j g2 is strictly decreasing, so (1 - v_j)^2 is unimodal and the
// minimum is at c - 1 or c, c = #{j : v_j > 1}; c is found by a warp ballot on
// every 8th node and then on the 8 nodes of the bracket.
__device__ __forceinline__ int root_argmin_warp(const double* sig, double g2, int lane) {
  const unsigned full = 0xffffffffu;
  const bool b1 = sig[8 * lane] * g2 > 1.0;
  const int L = __popc(__ballot_sync(full, b1));  // v_{8i} > 1 for i < L
  int c;
  if (L == 0) {
    c = 0;
  } else {
    const int base = 8 * (L - 1) + 1;  // v_{base-1} > 1
    const int j = base + (lane & 7);
    const bool b2 = (lane < 8) && (j < NRT) && (sig[j] * g2 > 1.0);
    c = base + __popc(__ballot_sync(full, b2));
  }
  int best = c < NRT ? c : NRT - 1;
  if (c >= 1) {
    const double dlo = 1.0 - sig[c - 1] * g2;
    const double d2lo = dlo * dlo;
    if (c < NRT) {
      const double dhi = 1.0 - sig[c] * g2;
      best = (d2lo <= dhi * dhi) ? c - 1 : c;
    } else {
      best = c - 1;
    }
  }
  return best;
}

// power.py:96-139 at one scale factor with growth g, for the warp: the root
// find and the moments over all 257 nodes with exp, as the reference.
__device__ HfParams halofit_params_warp(const double* sig, const double* pk3, double g,
                                        const ConstTables* __restrict__ c, int lane) {
  const double g2 = g * g;
  const int best = root_argmin_warp(sig, g2, lane);
  const int ind = best < 1 ? 1 : (best > NRT - 2 ? NRT - 2 : best);
  const double xp_ind = sig[ind] * g2;
  const double lo = sig[1] * g2, hi = sig[NRT - 2] * g2;
  const double xc = fmin(fmax(1.0, lo), hi);  // clip(x, xp[1], xp[-2])
  const int s = (xc - xp_ind >= 0.0) ? 1 : -1;
  const int j2 = ind + s;
  const double xp_j2 = sig[j2] * g2;
  const double slope = (c->logr[j2] - c->logr[ind]) / (xp_j2 - xp_ind);
  const double b = c->logr[ind] - slope * xp_ind;
  const double root = slope * 1.0 + b;
  const double R = fmax(exp(root), 1e-6);  // power.py:113-115
  HfParams hp;
  hp.knl = 1.0 / R;  // power.py:118
  const double inv = 1.0 / hp.knl;  // y = k * (1 / k_nl)
  double s1 = 0.0, s2 = 0.0;
  for (int i = lane; i < NKH; i += 32) {
    const double y = c->kh[i] * inv;
    const double y2 = y * y;
    const double res = pk3[i] * exp(-y2) * g2 / TWO_PI2;
    s1 += c->simpson_kh[i] * (2 * res * y2);
    s2 += c->simpson_kh[i] * (4 * res * (y2 - y2 * y2));
  }
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  hp.neff = s1 - 3.0;
  hp.C = s1 * s1 + s2;
  return hp;
}

// halofit coefficients (power.py:177-244; takahashi2012 or smith2003) into a
// FP64 row; one thread.
__device__ void halofit_coefs(const Bg& bg, double a, double lna, const HfParams& hp, double* row,
                              int model) {
  const double n = hp.neff, C = hp.C;
  double om_m, om_de;
  bg_om_l(bg, a, lna, &om_m, &om_de);
  const double w = bg_w(bg, a);
  row[R_KNL] = hp.knl;
  row[R_NEFF] = n;
  row[R_C] = C;
  row[R_OMM] = om_m;
  row[R_OMDE] = om_de;
  row[R_W] = w;
  const HfCoef<double> h = hf_coefs<double>(model, n, C, om_m, om_de, w);
  row[R_AN] = h.an;
  row[R_BN] = h.bn;
  row[R_CN] = h.cn;
  row[R_GAMMAN] = h.gam;
  row[R_ALPHAN] = h.alpha;
  row[R_BETAN] = h.beta;
  row[R_NUN] = h.nu;
  row[R_MUN] = h.mu;
  row[R_F1] = h.f1;
  row[R_F2] = h.f2;
  row[R_F3] = h.f3;
  row[R_LGKNL] = log(hp.knl);
  row[R_LGCF3] = h.lcf3;
}

__device__ __forceinline__ float ex2a(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2a(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// fp32c: the halofit coefficients (power.py:177-244) in float32 from n_eff, C
// and the float32 background Omega_m(a), Omega_de(a), w(a); the Limber
// integrand consumes them as float32.  Fills the float row and the
// coefficient fields of the float64 row.
__device__ void halofit_coefs_fast(const double* s, float om_m, float om_de, float wv,
                                   const HfParams& hp, double chiv, double g, double* row,
                                   float* f, int model) {
  const float n = (float)hp.neff, C = (float)hp.C, omde = om_de, w = wv;
  const float n2 = n * n, n3 = n2 * n, n4 = n2 * n2;
  constexpr float LOG2_10 = 3.321928094887362f;
  const float l2om = lg2a(om_m);
  float an, bn, cn, gam, alpha, beta, nun, mun, f1, f2, f3, lg2cf3;
  if (model == JCG_PK_SMITH2003) {
    // power.py:182-198, 239-242
    const float e_cn = -0.2807f + 0.6669f * n + 0.3214f * n2 - 0.0793f * C;
    an = ex2a(LOG2_10 * (1.4861f + 1.8369f * n + 1.6762f * n2 + 0.7940f * n3 + 0.1670f * n4 - 0.6206f * C));
    bn = ex2a(LOG2_10 * (0.9463f + 0.9466f * n + 0.3084f * n2 - 0.9400f * C));
    cn = ex2a(LOG2_10 * e_cn);
    gam = 0.8649f + 0.2989f * n + 0.1631f * C;
    alpha = 1.3884f + 0.3700f * n - 0.1452f * n2;
    beta = 0.8291f + 0.9854f * n + 0.3401f * n2;
    mun = ex2a(LOG2_10 * (-3.5442f + 0.1908f * n));
    nun = ex2a(LOG2_10 * (0.9585f + 1.2857f * n));
    const float frac = omde / (1.f - om_m), ofr = 1.f - frac;
    f1 = frac * ex2a(-0.0307f * l2om) + ofr * ex2a(-0.0732f * l2om);
    f2 = frac * ex2a(-0.0585f * l2om) + ofr * ex2a(-0.1423f * l2om);
    f3 = frac * ex2a(0.0743f * l2om) + ofr * ex2a(0.0725f * l2om);
    lg2cf3 = LOG2_10 * e_cn + lg2a(f3);
  } else {
    const float e_an = 1.5222f + 2.8553f * n + 2.3706f * n2 + 0.9903f * n3 + 0.2250f * n4 -
                       0.6038f * C + 0.1749f * omde * (1 + w);
    const float e_bn = -0.5642f + 0.5864f * n + 0.5716f * n2 - 1.5474f * C + 0.2279f * omde * (1 + w);
    const float e_cn = 0.3698f + 2.0404f * n + 0.8161f * n2 + 0.5869f * C;
    an = ex2a(LOG2_10 * e_an);
    bn = ex2a(LOG2_10 * e_bn);
    cn = ex2a(LOG2_10 * e_cn);
    gam = 0.1971f - 0.0843f * n + 0.8460f * C;
    alpha = fabsf(6.0835f + 1.3373f * n - 0.1959f * n2 - 5.5274f * C);
    beta = 2.0379f - 0.7354f * n + 0.3157f * n2 + 1.2490f * n3 + 0.3980f * n4 - 0.1682f * C;
    nun = ex2a(LOG2_10 * (5.2105f + 3.6902f * n));
    mun = 0.f;
    f1 = ex2a(-0.0307f * l2om);
    f2 = ex2a(-0.0585f * l2om);
    f3 = ex2a(0.0743f * l2om);
    lg2cf3 = LOG2_10 * e_cn + 0.0743f * l2om;
  }
  const float knl = (float)hp.knl;
  const float chic = fmaxf((float)chiv, 1.f);
  f[F_INVCHI] = 1.f / chic;
  f[F_CHIC] = chic;
  f[F_LG2INVCHI] = -lg2a(chic);
  f[F_LG2KNL] = lg2a(knl);
  f[F_INVKNL] = 1.f / knl;
  f[F_D2FAC] = (float)(g * g * s[S_PKNORM] * (1.0 / TWO_PI2));
  f[F_BETAN] = beta;
  f[F_ALPHAN] = alpha;
  f[F_AN] = an;
  f[F_3F1] = 3.f * f1;
  f[F_F2] = f2;
  f[F_BN] = bn;
  f[F_LG2CF3] = lg2cf3;
  f[F_3MGAMMA] = 3.f - gam;
  f[F_NUN] = nun;
  f[F_MUN] = mun;
  for (int i = NROW32_USED; i < NROW32; ++i) f[i] = 0.f;
  row[R_KNL] = hp.knl;
  row[R_NEFF] = hp.neff;
  row[R_C] = hp.C;
  row[R_OMM] = om_m;
  row[R_OMDE] = om_de;
  row[R_W] = wv;
  row[R_AN] = an;
  row[R_BN] = bn;
  row[R_CN] = cn;
  row[R_GAMMAN] = gam;
  row[R_ALPHAN] = alpha;
  row[R_BETAN] = beta;
  row[R_NUN] = nun;
  row[R_MUN] = mun;
  row[R_F1] = f1;
  row[R_F2] = f2;
  row[R_F3] = f3;
  row[R_LGKNL] = 0.6931471805599453 * f[F_LG2KNL];
  row[R_LGCF3] = 0.6931471805599453 * f[F_LG2CF3];
  row[R_LGCHIC] = -0.6931471805599453 * f[F_LG2INVCHI];
}

// FP32 row of the compensated fast path from the FP64 row.
__device__ void row32_from_row64(const double* s, const double* r, float* f) {
  const double chic = fmax(r[R_CHI], 1.0);
  constexpr double LOG2E = 1.4426950408889634;
  f[F_INVCHI] = (float)(1.0 / chic);
  f[F_CHIC] = (float)chic;
  f[F_LG2INVCHI] = (float)(-LOG2E * r[R_LGCHIC]);
  f[F_LG2KNL] = (float)(LOG2E * r[R_LGKNL]);
  f[F_INVKNL] = (float)(1.0 / r[R_KNL]);
  f[F_D2FAC] = (float)(r[R_G] * r[R_G] * s[S_PKNORM] / TWO_PI2);
  f[F_BETAN] = (float)r[R_BETAN];
  f[F_ALPHAN] = (float)r[R_ALPHAN];
  f[F_AN] = (float)r[R_AN];
  f[F_3F1] = (float)(3.0 * r[R_F1]);
  f[F_F2] = (float)r[R_F2];
  f[F_BN] = (float)r[R_BN];
  f[F_LG2CF3] = (float)(LOG2E * r[R_LGCF3]);
  f[F_3MGAMMA] = (float)(3.0 - r[R_GAMMAN]);
  f[F_NUN] = (float)r[R_NUN];
  f[F_MUN] = (float)r[R_MUN];
  for (int i = NROW32_USED; i < NROW32; ++i) f[i] = 0.f;
}

// chi and growth at a from the tables (background.py:242, 488) with the
// segment chosen by the reference's rule and the precomputed chi slopes.
__device__ __forceinline__ double chi_at(const CosmoTab* ct, const ConstTables* c, double a, int2 seg) {
  const int k = min(seg.x, seg.y);
  return fmax(ct->chi[seg.x] + ct->chi_slope[k] * (a - c->atab_chi[seg.x]), 0.0);
}

constexpr int HF_WARPS = 8;
// Limber nodes per CTA: the fp32c rows keep every thread busy in the
// thread-per-node phases (256 nodes); the float64 rows, whose warp-per-node
// moments dominate, use 64
__host__ __device__ constexpr int hf_nodes_per_block(bool fast) { return fast ? 256 : 64; }

// Root find of one node by one thread: c = #{j : sig_j g2 > 1} by bisection
// (the sequence is strictly decreasing), then the argmin among c - 1, c with
// the first index on ties -- the same index as argmin((1 - sig g2)^2).
__device__ __forceinline__ double root_knl_thread(const double* sig, double g2,
                                                  const ConstTables* __restrict__ c) {
  int lo = 0, hi = NRT;  // invariant: v_j > 1 for j < lo, v_j <= 1 for j >= hi
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (sig[mid] * g2 > 1.0) lo = mid + 1;
    else hi = mid;
  }
  const int cc = lo;
  int best = cc < NRT ? cc : NRT - 1;
  if (cc >= 1) {
    const double dlo = 1.0 - sig[cc - 1] * g2;
    if (cc < NRT) {
      const double dhi = 1.0 - sig[cc] * g2;
      best = (dlo * dlo <= dhi * dhi) ? cc - 1 : cc;
    } else {
      best = cc - 1;
    }
  }
  const int ind = best < 1 ? 1 : (best > NRT - 2 ? NRT - 2 : best);
  const double xp_ind = sig[ind] * g2;
  const double lo_v = sig[1] * g2, hi_v = sig[NRT - 2] * g2;
  const double xc = fmin(fmax(1.0, lo_v), hi_v);  // clip(x, xp[1], xp[-2])
  const int sgn = (xc - xp_ind >= 0.0) ? 1 : -1;
  const int j2 = ind + sgn;
  const double slope = (c->logr[j2] - c->logr[ind]) / (sig[j2] * g2 - xp_ind);
  const double b = c->logr[ind] - slope * xp_ind;
  const double root = slope * 1.0 + b;
  const double R = fmax(exp(root), 1e-6);  // power.py:113-115
  return 1.0 / R;                          // power.py:118
}

// fp32c: the same root find with the interpolation (power.py:112-115) in
// float pairs: the segment is chosen in float64 exactly as above (the
// decision), then R = exp(root) with root = logr[ind] + slope (1 - xp_ind) by
// the pair quotient and exp.  Returns R = 1 / k_nl.
__device__ __forceinline__ FF root_R_ff(const double* sig, double g2, const ConstTables* __restrict__ c,
                                        const float2* e2) {
  int lo = 0, hi = NRT;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (sig[mid] * g2 > 1.0) lo = mid + 1;
    else hi = mid;
  }
  const int cc = lo;
  int best = cc < NRT ? cc : NRT - 1;
  if (cc >= 1) {
    const double dlo = 1.0 - sig[cc - 1] * g2;
    if (cc < NRT) {
      const double dhi = 1.0 - sig[cc] * g2;
      best = (dlo * dlo <= dhi * dhi) ? cc - 1 : cc;
    } else {
      best = cc - 1;
    }
  }
  const int ind = best < 1 ? 1 : (best > NRT - 2 ? NRT - 2 : best);
  const double xp_ind = sig[ind] * g2;
  const double lo_v = sig[1] * g2, hi_v = sig[NRT - 2] * g2;
  const double xc = fmin(fmax(1.0, lo_v), hi_v);
  const int j2 = ind + ((xc - xp_ind >= 0.0) ? 1 : -1);
  const FF slope = ff_of(c->logr[j2] - c->logr[ind]) / ff_of(sig[j2] * g2 - xp_ind);
  const FF root = ff_of(c->logr[ind]) + slope * ff_of(1.0 - xp_ind);
  const FF R = ff_exp(root, e2);
  return R.hi < 1e-6f ? ff_of(1e-6) : R;  // power.py:115
}

// Three phases per block of Limber nodes:
//  1a thread per node: growth, chi, root find, k_nl; FAST: the exp index
//     range and the Taylor part of the moments;
//  1b warp per node: the exp part of the moments (power.py:121-136);
//  2  thread per node: n_eff, C and the takahashi2012 coefficients.
// A block takes 64 nodes of one cosmology (float64), or 256 consecutive
// nodes of the batch's flat (cosmology, node) index (fp32c, one geometry,
// at least 256 nodes per cosmology: each block spans at most two
// cosmologies, whose tables it holds side by side, and no block runs short),
// or 256 nodes of one cosmology (fp32c otherwise).
__host__ __device__ inline bool hf_flat(const Batch& b) {
  return b.precision == JCG_FP32C && !b.listed && b.max_na >= hf_nodes_per_block(true);
}
template <bool FAST>
__global__ void __launch_bounds__(HF_WARPS * 32, FAST ? 6 : 1)
    halofit_rows_kernel(Batch bt, const ConstTables* __restrict__ c) {
  constexpr int NB = hf_nodes_per_block(FAST);
  constexpr int NSL = FAST ? 2 : 1;  // cosmologies per block at most
  const bool flat = FAST && hf_flat(bt);
  int item0, n0, cnt, nsl;
  if (flat) {
    const long long f0 = (long long)blockIdx.x * NB, nf = (long long)bt.n_items * bt.max_na;
    if (f0 >= nf) return;
    item0 = (int)(f0 / bt.max_na);
    n0 = (int)(f0 - (long long)item0 * bt.max_na);
    cnt = (int)min((long long)NB, nf - f0);
    nsl = n0 + cnt > bt.max_na ? 2 : 1;
  } else {
    item0 = blockIdx.y;
    if (item0 >= bt.n_items) return;
    n0 = blockIdx.x * NB;
    const int na_i = batch_item(bt, item0).geo->na;
    if (n0 >= na_i) return;
    cnt = min(na_i - n0, NB);
    nsl = 1;
  }
  const Item itA = batch_item(bt, item0);
  const Item itB = nsl > 1 ? batch_item(bt, item0 + 1) : itA;
  const GeoHeader* geo = itA.geo;
  const int na = geo->na;
  const int model = pk_model(itA.physics);
  __shared__ double sigS[NSL][NRT];
  __shared__ double pk3[FAST ? 1 : NKH];
  __shared__ double sS[NSL][NSCAL];
  __shared__ double knl_s[NB], inv_s[NB], g_s[NB], chi_s[NB], t1_s[NB], t2_s[NB], s1_s[NB], s2_s[NB];
  __shared__ int ilo_s[NB], ihi_s[NB];
  __shared__ float iv2h_s[NB], iv2l_s[NB], f1_s[NB], f2_s[NB];
  __shared__ float wpfS[NSL][FAST ? NKH : 1], k2h[FAST ? NKH + 1 : 1], k2l[FAST ? NKH + 1 : 1];
  __shared__ float2 e2s[FAST ? 64 : 1];
  if (FAST)
    for (int i = threadIdx.x; i < 64; i += blockDim.x) e2s[i] = c->exp2_ff[i];
  for (int k = 0; k < nsl; ++k) {
    const CosmoTab* ctk = k ? itB.ctab : itA.ctab;
    for (int i = threadIdx.x; i < NRT; i += blockDim.x) sigS[k][i] = ctk->sig[i];
    for (int i = threadIdx.x; i < NSCAL; i += blockDim.x) sS[k][i] = ctk->s[i];
    if (FAST)
      for (int i = threadIdx.x; i < NKH; i += blockDim.x) wpfS[k][i] = ctk->wpk3f[i];
  }
  if (FAST) {
    for (int i = threadIdx.x; i < NKH + 1; i += blockDim.x) {
      k2h[i] = c->kh2_hi[i];
      k2l[i] = c->kh2_lo[i];
    }
  } else {
    for (int i = threadIdx.x; i < NKH; i += blockDim.x) pk3[i] = itA.ctab->pk3[i];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double* A = geo_ptr<double>(geo, geo->off_a);
  const double* WS = geo_ptr<double>(geo, geo->off_wsimp);
  const int64_t* SC = geo_ptr<int64_t>(geo, geo->off_seg_chi);
  const int64_t* SG = geo_ptr<int64_t>(geo, geo->off_seg_grow);
  // node t of the block: its cosmology's slot and its index on the Limber grid
  auto slot_of = [&](int t) { return n0 + t >= na ? 1 : 0; };
  auto node_of = [&](int t) { return n0 + t >= na ? n0 + t - na : n0 + t; };
  // phase 1a
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    const int n = node_of(t), slt = slot_of(t);
    const double* sig = sigS[slt];
    const CosmoTab* ct = slt ? itB.ctab : itA.ctab;
    const double a = A[n];
    double g, knl, inv;
    FF iv2;
    if (FAST) {
      // growth by the segment's node spacing reciprocal (no float64 division)
      const int2 sg = unpack_seg(SG[n]);
      const double sl = (ct->g[sg.y] - ct->g[sg.x]) * c->grow_ida[min(sg.x, sg.y)] * (sg.y > sg.x ? 1.0 : -1.0);
      g = clip_lohi(ct->g[sg.x] + sl * (a - c->atab_grow[sg.x]), 0.0, 1.0);
      const FF R = root_R_ff(sig, g * g, c, e2s);
      inv = ffd(R);
      knl = ffd(ff_rcp(R));
      iv2 = ff_sqr(R);
    } else {
      g = clip_lohi(interp_eval(a, c->atab_grow, ct->g, unpack_seg(SG[n])), 0.0, 1.0);
      knl = root_knl_thread(sig, g * g, c);
      inv = 1.0 / knl;  // y = k * (1 / k_nl)
    }
    g_s[t] = g;
    knl_s[t] = knl;
    inv_s[t] = inv;
    chi_s[t] = chi_at(ct, c, a, unpack_seg(SC[n]));
    int ilo = 0, ihi = NKH - 1;
    double t1 = 0.0, t2 = 0.0;
    if (model == JCG_PK_LINEAR) {
      ihi = -1;  // linear_matter_power: the halofit moments are not used
    } else if (FAST) {
      // exp only for y^2 in [Y2_TAYLOR, Y2_SKIP] (the split point only needs
      // to be consistent, so it is found in FP32); y^2 = kh^2 inv^2 with
      // inv^2 as a float pair for the FP32 terms
      const float linv = LN2_F * lg2f((float)inv);
      constexpr float HLY2T = 0.0f, HLY2S = 2.0471425f;  // 0.5 log(Y2_TAYLOR), 0.5 log(Y2_SKIP)
      ilo = (int)floorf((HLY2T - linv - (float)LOG_KMIN) * (float)(1.0 / DLOGK));
      ihi = (int)ceilf((HLY2S - linv - (float)LOG_KMIN) * (float)(1.0 / DLOGK));
      ilo = max(0, min(ilo, NKH));
      ihi = max(ilo - 1, min(ihi, NKH - 1));
      iv2h_s[t] = iv2.hi;
      iv2l_s[t] = iv2.lo;
      // sum_{i < ilo} w pk3 y^2 e^{-y^2} = sum_m (-1)^m / m! x^(m+1) Q_m[ilo]
      // with x = y_ilo^2 = (kh_ilo inv)^2: t1 = x F(x), and the y^4 moment
      // gives t2 = t1 + x^2 F'(x), F(x) = sum_m R_m[ilo] x^m (Horner with
      // the derivative, float pairs)
      if (ilo > 0) {
        FF kk;
        kk.hi = k2h[ilo], kk.lo = k2l[ilo];
        const FF x = ff_mul(kk, iv2);
        const float2* R = &ct->rtay[0][ilo];
        FF P, D;
        P.hi = R[(NTAYLOR - 1) * (NKH + 1)].x, P.lo = R[(NTAYLOR - 1) * (NKH + 1)].y;
        D.hi = 0.f, D.lo = 0.f;
        for (int m = NTAYLOR - 2; m >= 0; --m) {
          D = ff_add(ff_mul(D, x), P);
          FF r;
          r.hi = R[m * (NKH + 1)].x, r.lo = R[m * (NKH + 1)].y;
          P = ff_add(ff_mul(P, x), r);
        }
        const FF f1 = ff_mul(x, P);
        const FF f2 = ff_mul(ff_mul(x, x), D);
        t1 = ff_to_double(f1);
        t2 = t1 + ff_to_double(f2);
      }
    }
    ilo_s[t] = ilo;
    ihi_s[t] = ihi;
    t1_s[t] = t1;
    t2_s[t] = t2;
  }
  __syncthreads();
  // phase 1b
  for (int t = warp; t < cnt; t += HF_WARPS) {
    const double inv = inv_s[t];
    const float* wpf = wpfS[slot_of(t)];
    double s1 = 0.0, s2 = 0.0;
    if (FAST) {
      // FP32 terms: y^2 = kh^2 inv^2 as a float pair (hi p, lo e), exp(-y^2)
      // from the pair, weights w pk3 rounded once to float
      const float ih = iv2h_s[t], il = iv2l_s[t];
      float f1 = 0.f, f2 = 0.f;
      for (int i = ilo_s[t] + lane; i <= ihi_s[t]; i += 32) {
        const float kh = k2h[i];
        const float p = kh * ih;
        float e = fmaf(kh, ih, -p);
        e = fmaf(kh, il, e);
        e = fmaf(k2l[i], ih, e);
        const float r = wpf[i] * exp_neg_pair(p, e);
        const float y2 = p + e;
        f1 = fmaf(2.f * r, y2, f1);
        f2 = fmaf(4.f * r, y2 * ((1.f - p) - e), f2);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        f1 += __shfl_xor_sync(0xffffffffu, f1, o);
        f2 += __shfl_xor_sync(0xffffffffu, f2, o);
      }
      if (lane == 0) {
        f1_s[t] = f1;
        f2_s[t] = f2;
      }
    } else {
      const double g2 = g_s[t] * g_s[t];
      for (int i = lane; i <= ihi_s[t]; i += 32) {
        const double y = c->kh[i] * inv;
        const double y2 = y * y;
        const double res = pk3[i] * exp(-y2) * g2 / TWO_PI2;
        s1 += c->simpson_kh[i] * (2 * res * y2);
        s2 += c->simpson_kh[i] * (4 * res * (y2 - y2 * y2));
      }
    }
    if (!FAST) {
      s1 = warp_sum(s1);
      s2 = warp_sum(s2);
      if (lane == 0) {
        s1_s[t] = s1;
        s2_s[t] = s2;
      }
    }
  }
  __syncthreads();
  // phase 2
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    const int n = node_of(t), slt = slot_of(t);
    const double* s = sS[slt];
    double* const rows64 = slt ? itB.rows64 : itA.rows64;
    float* const rows32 = slt ? itB.rows32 : itA.rows32;
    float* const u32 = slt ? itB.u32 : itA.u32;
    const double a = A[n];
    double s1 = FAST ? (double)f1_s[t] : s1_s[t], s2 = FAST ? (double)f2_s[t] : s2_s[t];
    if (FAST) {
      const double g2 = g_s[t] * g_s[t] * (1.0 / TWO_PI2);
      s1 = (s1 + 2.0 * t1_s[t]) * g2;
      s2 = (s2 + 4.0 * t2_s[t]) * g2;
    }
    HfParams hp;
    hp.knl = knl_s[t];
    hp.neff = s1 - 3.0;  // power.py:138-139
    hp.C = s1 * s1 + s2;
    double row[NROW64];
    for (int i = 0; i < NROW64; ++i) row[i] = 0.0;
    const double chiv = chi_s[t];
    row[R_CHI] = chiv;
    row[R_G] = g_s[t];
    float f[NROW32];
    if (FAST) {
      // background in FP32 (background.py:122-126, 168, 196, 270-294):
      // E^2(a), Omega_m(a), Omega_de(a), w(a), dchi/da
      const float af = (float)a, ia = rcpf(af), ia2 = ia * ia;
      const float w0 = (float)s[S_W0], wa = (float)s[S_WA];
      const float fde = -3.f * (1.f + w0 + wa) * (LN2_F * lg2f(af)) + 3.f * wa * (af - 1.f);
      const float ef = fde == 0.f ? 1.f : ex2f(fde * LOG2E_F);
      const float om3 = (float)s[S_OMEGA_M] * (ia2 * ia), ode = (float)s[S_OMEGA_DE] * ef;
      const float e2 = om3 + (float)s[S_OMEGA_K] * ia2 + ode;
      const float ie2 = rcpf(e2);
      const float omm = om3 * ie2, omde = ode * ie2, wv = w0 + (1.f - af) * wa;
      halofit_coefs_fast(s, omm, omde, wv, hp, chiv, g_s[t], row, f, model);
      const float dchi = (float)RH * ia2 * rsqrtf(e2);
      const float chic = fmaxf((float)chiv, 1.f);
      row[R_DCHI] = dchi;
      const float uf = (float)WS[n] * dchi * rcpf(chic * chic) * (float)(1.0 / C2);
      row[R_U] = (double)uf;
      if (u32) u32[n] = uf;  // the Limber kernel's float copy
    } else {
      const double lna = log(a);
      const Bg bg = make_bg(s);
      halofit_coefs(bg, a, lna, hp, row, model);
      row[R_LGCHIC] = log(fmax(chiv, 1.0));
      const double dchi = bg_dchioverda_l(bg, a, lna);
      row[R_DCHI] = dchi;
      row[R_U] = WS[n] * dchi / fmax(chiv * chiv, 1.0) / C2;
    }
    if (rows64) {
      double* dst = rows64 + (size_t)n * NROW64;
      if (FAST) {
        // fp32c: the Limber weight and the halofit parameters (the rest of
        // the integrand's inputs are in the FP32 row)
        constexpr int keep[] = {R_CHI, R_G, R_KNL, R_NEFF, R_C, R_DCHI, R_U};
#pragma unroll
        for (int q = 0; q < 7; ++q) dst[keep[q]] = row[keep[q]];
      } else {
        for (int i = 0; i < NROW64; ++i) dst[i] = row[i];
      }
    }
    if (rows32) {
      if (!FAST) row32_from_row64(s, row, f);
      float* dst = rows32 + (size_t)n * NROW32;
      for (int i = 0; i < NROW32; ++i) dst[i] = f[i];
    }
  }
}

void launch_halofit_rows(const Batch& b, const ConstTables* c, cudaStream_t st) {
  const int nb = hf_nodes_per_block(b.precision == JCG_FP32C);
  dim3 grid((b.max_na + nb - 1) / nb, b.n_items);
  if (hf_flat(b)) grid = dim3((unsigned)(((long long)b.n_items * b.max_na + nb - 1) / nb), 1);
  if (b.precision == JCG_FP32C)
    halofit_rows_kernel<true><<<grid, HF_WARPS * 32, 0, st>>>(b, c);
  else
    halofit_rows_kernel<false><<<grid, HF_WARPS * 32, 0, st>>>(b, c);
}

// ------------------------------------------------------ pointwise queries ---
// interp(x, xp, fp) of scipy/interpolate.py:12-37 for any table, by a warp:
// the nearest node by argmin (x - xp)^2 (first index on ties), clipped to
// [1, n - 2], then the segment on the side of sign(clip(x, xp[1], xp[-2]) - xp[ind])
// with clip = min(max(x, lo), hi) and sign 0 taken as +1.
__device__ double interp_ref_warp(double x, const double* xp, const double* fp, int n, int lane) {
  double best = INFINITY;
  int bi = n;
  for (int j = lane; j < n; j += 32) {
    const double d = (x - xp[j]) * (x - xp[j]);
    if (d < best) best = d, bi = j;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ob < best || (ob == best && oi < bi)) best = ob, bi = oi;
  }
  const int ind = bi < 1 ? 1 : (bi > n - 2 ? n - 2 : bi);
  const double xc = fmin(fmax(x, xp[1]), xp[n - 2]);
  const int j2 = ind + ((xc - xp[ind] < 0.0) ? -1 : 1);
  const double sl = (fp[j2] - fp[ind]) / (xp[j2] - xp[ind]);
  const double b = fp[ind] - sl * xp[ind];
  return sl * x + b;
}

// One warp per (cosmology, point).  `what` as documented in jcg.h.  FP64, the
// full (reference) form of the moments.
__global__ void eval_points_kernel(const double* __restrict__ params, int n_cosmo,
                                   const CosmoTab* __restrict__ ctab,
                                   const ConstTables* __restrict__ c, const double* __restrict__ av,
                                   const double* __restrict__ kv, int n, int what_phys,
                                   double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int what = what_phys & 0xff, model = pk_model(what_phys >> 8);
  const long gw = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= (long)n_cosmo * n) return;
  const int ci = (int)(gw / n), pi = (int)(gw % n);
  const CosmoTab* ct = ctab + ci;
  const double* s = ct->s;
  const Bg bg = make_bg(s);
  const double a = av ? av[pi] : 1.0;
  const double k = kv ? kv[pi] : 1.0;
  double v = 0.0;
  auto growth = [&](double x) {
    const int2 sg = interp_segment_inc(x, c->atab_grow, NGROW, logspace_guess(x, NGROW));
    return clip_lohi(interp_eval(x, c->atab_grow, ct->g, sg), 0.0, 1.0);
  };
  auto chi_of = [&](double x) {
    const int2 sg = interp_segment_inc(x, c->atab_chi, NCHI, logspace_guess(x, NCHI));
    return fmax(interp_eval(x, c->atab_chi, ct->chi, sg), 0.0);
  };
  if (what == 0) {
    v = chi_of(a);
  } else if (what == 10 || what == 11) {
    // transverse_comoving_distance (background.py:297-344): k = -sign(Omega_k)
    const double chi = chi_of(a), ok = s[S_OMEGA_K];
    const double sk = sqrt(fabs(ok));
    double fk = chi;
    if (ok > 0.0) fk = RH / sk * sinh(sk * chi / RH);
    else if (ok < 0.0) fk = RH / sk * sin(sk * chi / RH);
    v = what == 10 ? fk : a * fk;  // angular_diameter_distance = a f_k (background.py:347-368)
  } else if (what == 12) {
    // a_of_chi (background.py:245-267): interp(chi, chi table, a table) with the
    // reference's rule on the decreasing chi table
    v = interp_ref_warp(a, ct->chi, c->atab_chi, NCHI, lane);
  } else if (what == 13 && growth_gamma(what_phys >> 8)) {
    // growth_rate with gamma: Omega_m(a)^gamma (background.py:555-582)
    v = pow(bg_omm(bg, a), s[S_GAMMA]);
  } else if (what == 13) {
    // growth_rate (background.py:401-440, 491-512): interp(a, atab, ftab), no clip
    const int2 sg = interp_segment_inc(a, c->atab_grow, NGROW, logspace_guess(a, NGROW));
    v = interp_eval(a, c->atab_grow, ct->f, sg);
  } else if (what == 1) {
    v = growth(a);
  } else if (what == 2) {
    v = bg_H(bg, a);
  } else if (what == 3) {
    v = bg_dchioverda(bg, a);
  } else if (what == 4) {
    v = eh_transfer(s, k);
  } else if (what == 5) {
    v = pk_linear(s, k, growth(a));
  } else {
    const double g = growth(a);
    const HfParams hp = halofit_params_warp(ct->sig, ct->pk3, g, c, lane);
    if (what == 6) {
      double row[NROW64];
      row[R_G] = g;
      halofit_coefs(bg, a, log(a), hp, row, model);
      v = halofit_node(s, row, k, model);
    } else if (what == 7) {
      v = hp.knl;
    } else if (what == 8) {
      v = hp.neff;
    } else {
      v = hp.C;
    }
  }
  if (lane == 0) out[(size_t)ci * n + pi] = v;
}

void launch_eval_points(const double* params, int n_cosmo, CosmoTab* ctab, const ConstTables* c,
                        const double* a, const double* k, int n, int what, double* out,
                        cudaStream_t st) {
  const long warps = (long)n_cosmo * n;
  const int threads = 256;
  const long blocks = (warps * 32 + threads - 1) / threads;
  eval_points_kernel<<<(unsigned)blocks, threads, 0, st>>>(params, n_cosmo, ctab, c, a, k, n, what,
                                                            out);
}

}  // namespace jcg
