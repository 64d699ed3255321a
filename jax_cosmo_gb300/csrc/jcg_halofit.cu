// Halofit parameters per Limber node (FP64) and pointwise table queries.
//
// One warp per scale-factor node: the sigma^2(R) root find of power.py:96-118
// (exact argmin over the 256-node table + the decreasing-table side rule of
// scipy/interpolate.py:47-57) and the spectral moments of power.py:121-139,
// then the takahashi2012 coefficients of power.py:177-238.
#include "jcg_internal.cuh"

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

// power.py:96-139 at one scale factor with growth g, for the warp.
// sig/pk3 may live in shared or global memory.
__device__ HfParams halofit_params_warp(const double* sig, const double* pk3, double g,
                                        const ConstTables* __restrict__ c, int lane) {
  const double g2 = g * g;
  // argmin_j (1 - sigma_j)^2, first index on ties  (scipy/interpolate.py:47)
  double bestd = 0.0;
  int best = -1;
  for (int j = lane; j < NRT; j += 32) {
    const double d = 1.0 - sig[j] * g2;
    const double d2 = d * d;
    if (best < 0 || d2 < bestd) { bestd = d2; best = j; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double od = __shfl_xor_sync(0xffffffffu, bestd, o);
    const int oj = __shfl_xor_sync(0xffffffffu, best, o);
    if (od < bestd || (od == bestd && oj < best)) { bestd = od; best = oj; }
  }
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
  // moments (power.py:121-139): y = k * (1 / k_nl)
  const double inv = 1.0 / hp.knl;
  double s1 = 0.0, s2 = 0.0;
  for (int i = lane; i < NKH; i += 32) {
    const double y = c->kh[i] * inv;
    const double y2 = y * y;
    const double res = pk3[i] * exp(-y2) * g2 / TWO_PI2;
    const double t1 = 2 * res * y2;
    const double t2 = 4 * res * (y2 - y2 * y2);
    s1 += c->simpson_kh[i] * t1;
    s2 += c->simpson_kh[i] * t2;
  }
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  hp.neff = s1 - 3.0;
  hp.C = s1 * s1 + s2;
  return hp;
}

// takahashi2012 coefficients (power.py:177-238) into a FP64 row.
__device__ void halofit_coefs(const Bg& bg, double a, const HfParams& hp, double* row) {
  const double n = hp.neff, C = hp.C;
  const double om_m = bg_omm(bg, a);
  const double om_de = bg_omde(bg, a);
  const double w = bg_w(bg, a);
  const double n2 = n * n, n3 = pow(n, 3.0), n4 = pow(n, 4.0);
  row[R_KNL] = hp.knl;
  row[R_NEFF] = n;
  row[R_C] = C;
  row[R_OMM] = om_m;
  row[R_OMDE] = om_de;
  row[R_W] = w;
  row[R_AN] = pow(10.0, 1.5222 + 2.8553 * n + 2.3706 * n2 + 0.9903 * n3 + 0.2250 * n4 -
                            0.6038 * C + 0.1749 * om_de * (1 + w));
  row[R_BN] = pow(10.0, -0.5642 + 0.5864 * n + 0.5716 * n2 - 1.5474 * C + 0.2279 * om_de * (1 + w));
  row[R_CN] = pow(10.0, 0.3698 + 2.0404 * n + 0.8161 * n2 + 0.5869 * C);
  row[R_GAMMAN] = 0.1971 - 0.0843 * n + 0.8460 * C;
  row[R_ALPHAN] = fabs(6.0835 + 1.3373 * n - 0.1959 * n2 - 5.5274 * C);
  row[R_BETAN] = 2.0379 - 0.7354 * n + 0.3157 * n2 + 1.2490 * n3 + 0.3980 * n4 - 0.1682 * C;
  row[R_NUN] = pow(10.0, 5.2105 + 3.6902 * n);
  row[R_F1] = pow(om_m, -0.0307);
  row[R_F2] = pow(om_m, -0.0585);
  row[R_F3] = pow(om_m, 0.0743);
}

// FP32 row of the compensated fast path from the FP64 row.
__device__ void row32_from_row64(const double* s, const double* r, float* f) {
  const double chic = fmax(r[R_CHI], 1.0);
  f[F_INVCHI] = (float)(1.0 / chic);
  f[F_CHIC] = (float)chic;
  f[F_LG2INVCHI] = (float)(-log2(chic));
  f[F_LG2KNL] = (float)log2(r[R_KNL]);
  f[F_INVKNL] = (float)(1.0 / r[R_KNL]);
  f[F_D2FAC] = (float)(r[R_G] * r[R_G] * s[S_PKNORM] / TWO_PI2);
  f[F_BETAN] = (float)r[R_BETAN];
  f[F_ALPHAN] = (float)r[R_ALPHAN];
  f[F_AN] = (float)r[R_AN];
  f[F_3F1] = (float)(3.0 * r[R_F1]);
  f[F_F2] = (float)r[R_F2];
  f[F_BN] = (float)r[R_BN];
  f[F_LG2CF3] = (float)log2(r[R_CN] * r[R_F3]);
  f[F_3MGAMMA] = (float)(3.0 - r[R_GAMMAN]);
  f[F_NUN] = (float)r[R_NUN];
  for (int i = NROW32_USED; i < NROW32; ++i) f[i] = 0.f;
}

constexpr int HF_WARPS = 8;
constexpr int HF_NODES_PER_BLOCK = 64;

__global__ void __launch_bounds__(HF_WARPS * 32)
    halofit_rows_kernel(Batch bt, const ConstTables* __restrict__ c) {
  const int item = blockIdx.y;
  if (item >= bt.n_items) return;
  const Item it = batch_item(bt, item);
  const GeoHeader* geo = it.geo;
  const int na = geo->na;
  const int n0 = blockIdx.x * HF_NODES_PER_BLOCK;
  if (n0 >= na) return;
  __shared__ double sig[NRT];
  __shared__ double pk3[NKH];
  __shared__ double s[NSCAL];
  __shared__ double chi[NCHI];
  __shared__ double gt[NGROW];
  const CosmoTab* ct = it.ctab;
  for (int i = threadIdx.x; i < NRT; i += blockDim.x) sig[i] = ct->sig[i];
  for (int i = threadIdx.x; i < NKH; i += blockDim.x) pk3[i] = ct->pk3[i];
  for (int i = threadIdx.x; i < NSCAL; i += blockDim.x) s[i] = ct->s[i];
  for (int i = threadIdx.x; i < NCHI; i += blockDim.x) chi[i] = ct->chi[i];
  for (int i = threadIdx.x; i < NGROW; i += blockDim.x) gt[i] = ct->g[i];
  __syncthreads();
  const Bg bg = make_bg(s);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double* A = geo_ptr<double>(geo, geo->off_a);
  const double* WS = geo_ptr<double>(geo, geo->off_wsimp);
  const int64_t* SC = geo_ptr<int64_t>(geo, geo->off_seg_chi);
  const int64_t* SG = geo_ptr<int64_t>(geo, geo->off_seg_grow);
  const int n_end = min(na, n0 + HF_NODES_PER_BLOCK);
  for (int n = n0 + warp; n < n_end; n += HF_WARPS) {
    const double a = A[n];
    const double chiv = fmax(interp_eval(a, c->atab_chi, chi, unpack_seg(SC[n])), 0.0);
    const double g = clip_lohi(interp_eval(a, c->atab_grow, gt, unpack_seg(SG[n])), 0.0, 1.0);
    const HfParams hp = halofit_params_warp(sig, pk3, g, c, lane);
    if (lane == 0) {
      double row[NROW64];
      for (int i = 0; i < NROW64; ++i) row[i] = 0.0;
      row[R_CHI] = chiv;
      row[R_G] = g;
      halofit_coefs(bg, a, hp, row);
      const double dchi = bg_dchioverda(bg, a);
      row[R_DCHI] = dchi;
      row[R_U] = WS[n] * dchi / fmax(chiv * chiv, 1.0) / C2;
      if (it.rows64) {
        double* dst = it.rows64 + (size_t)n * NROW64;
        for (int i = 0; i < NROW64; ++i) dst[i] = row[i];
      }
      if (it.rows32) {
        float f[NROW32];
        row32_from_row64(s, row, f);
        float* dst = it.rows32 + (size_t)n * NROW32;
        for (int i = 0; i < NROW32; ++i) dst[i] = f[i];
      }
    }
  }
}

void launch_halofit_rows(const Batch& b, const ConstTables* c, cudaStream_t st) {
  dim3 grid((b.max_na + HF_NODES_PER_BLOCK - 1) / HF_NODES_PER_BLOCK, b.n_items);
  halofit_rows_kernel<<<grid, HF_WARPS * 32, 0, st>>>(b, c);
}

// ------------------------------------------------------ pointwise queries ---
// One warp per (cosmology, point).  `what` as documented in jcg.h.
__global__ void eval_points_kernel(const double* __restrict__ params, int n_cosmo,
                                   const CosmoTab* __restrict__ ctab,
                                   const ConstTables* __restrict__ c, const double* __restrict__ av,
                                   const double* __restrict__ kv, int n, int what,
                                   double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
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
  if (what == 0) {
    const int2 sg = interp_segment_inc(a, c->atab_chi, NCHI, logspace_guess(a, NCHI));
    v = fmax(interp_eval(a, c->atab_chi, ct->chi, sg), 0.0);
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
      halofit_coefs(bg, a, hp, row);
      v = halofit_node(s, row, k);
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
