// Internal layouts and device helpers shared by the libjcg translation units.
//
// Numbers of nodes, grid formulas and operation order follow jax_cosmo (paths
// relative to the jax_cosmo project root); each helper cites the line it restates.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "../../include/jcg.h"

namespace jcg {

// ------------------------------------------------------------------ sizes ---
constexpr int NCHI = 256;    // background.py:199  radial_comoving_distance steps
constexpr int NGROW = 128;   // background.py:443  _growth_factor_ODE steps
constexpr int NRT = 256;     // power.py:93        log R nodes of the sigma^2(R) table
constexpr int NKH = 257;     // power.py:111,136   simps(..., 256) over ln k
constexpr int NROMB = 129;   // power.py:77        romb(divmax=7): 2 + 1 + 2 + ... + 64
constexpr int NZP = 257;     // probes.py:51       simps(integrand, z, zmax, 256)
constexpr int NNORM = 257;   // redshift.py:30     simps(pz_fn, 0, zmax, 256)
constexpr int MAXTR = JCG_MAX_TRACERS;
constexpr int MAXPAIR = JCG_MAX_PAIRS;

// physical constants: constants.py:9-27
constexpr double C_KMS = 299792.458;
constexpr double TCMB = 2.726;
constexpr double RH = 2997.92458;
constexpr double H0 = 100.0;
constexpr double PI = 3.141592653589793;
constexpr double EULER_E = 2.718281828459045;  // np.exp(1.0)

// ------------------------------------------------ cosmology-wide constants ---
// Grids shared by every cosmology and every geometry, built once per device.
constexpr int NTAYLOR = 20;      // Taylor terms of exp(-y^2) below y^2 = 1 (1/19! < 1e-17)

// Number of SMs of the current device (grid sizing); 152 if the query fails.
inline int device_sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      n <= 0)
    return 152;
  return n;
}

struct ConstTables {
  double atab_chi[NCHI];   // logspace(-3, 0, 256)
  double lna_chi[NCHI];    // log(atab_chi): the RK4 abscissae of background.py:231
  double atab_grow[NGROW]; // logspace(-3, 0, 128)
  double logk[NKH];        // linspace(log 1e-4, log 1e4, 257)
  double kh[NKH];          // exp(logk)
  double kh3[NKH];         // kh**3
  double logr[NRT];        // linspace(log 1e-4, log 10, 256)
  double simpson_kh[NKH];  // Simpson weights (1,4,2,...,4,1) * dx/3 on the ln k grid
  double romb_logk[NROMB]; // romb abscissae in evaluation order (scipy/integrate.py:129-146)
  double E[NKH * NRT];     // exp(-(k_i r_j)^2), i-major: power.py:99-109
  float2 Eff[NKH * NRT];   // the same as float pairs (hi, lo) (fp32c sigma^2(R) sums)
  double kpw[NTAYLOR][NKH];  // simpson_kh[i] * kh[i]^(2(m+1)): the Taylor prefix sums' weights
  double romb_w[NROMB];      // romb's Richardson combination as weights on romb_logk's values
  // cosmology-independent factors of the table kernel's right-hand sides
  double romb_k[NROMB];      // exp(romb_logk)
  double romb_ik[NROMB];     // 1 / romb_k
  double romb_kw2[NROMB];    // k (k W(8k))^2, W the top-hat window (power.py:70-75)
  double ikh[NKH];           // 1 / kh
  double chi_a[NCHI];        // exp(lna_chi): the chi RK4 nodes
  double chi_ia[NCHI];       // 1 / chi_a
  double chi_lnam[NCHI];     // step midpoints lna_chi[i-1] + (lna_chi[i] - lna_chi[i-1]) / 2 (i >= 1)
  double chi_am[NCHI];       // exp(chi_lnam)
  double chi_iam[NCHI];      // 1 / chi_am
  double grow_lna[NGROW];    // log(atab_grow)
  double grow_ia[NGROW];     // 1 / atab_grow
  double grow_am[NGROW];     // step midpoints atab_grow[i-1] + (atab_grow[i] - atab_grow[i-1]) / 2 (i >= 1)
  double grow_lnam[NGROW];   // log(grow_am)
  double grow_iam[NGROW];    // 1 / grow_am
  // fp32c halofit moments: kh[i]^2 as a float pair hi + lo, with a virtual
  // node kh[NKH] = kh[NKH - 1] e^dlnk; the Taylor tables' factors
  // rho_m = e^(-2 (m + 1) dlnk) and c_m = (-1)^m / m! as float pairs
  float simpson_f[NKH];      // simpson_kh, float
  float kh2_hi[NKH + 1];
  float kh2_lo[NKH + 1];
  float tay_rho[NTAYLOR][2];
  float tay_c[NTAYLOR][2];
  // fp32c table stages in float pairs (hi, lo): the tables of the pair exp
  // and sin, and pair copies of the abscissae and factors above
  float2 exp2_ff[64];          // 2^(j/64)
  float2 sincos_ff[256];       // sin, cos of j pi/64, j < 128 (interleaved)
  float2 romb_k_ff[NROMB], romb_logk_ff[NROMB], romb_ik_ff[NROMB], romb_kw2_ff[NROMB];
  float2 kh_ff[NKH], logk_ff[NKH], ikh_ff[NKH], kh3_ff[NKH], simpson_ff[NKH];
  float2 chi_a_ff[NCHI], lna_chi_ff[NCHI], chi_ia_ff[NCHI], chi_am_ff[NCHI], chi_lnam_ff[NCHI], chi_iam_ff[NCHI];
  float2 grow_a_ff[NGROW], grow_lna_ff[NGROW], grow_ia_ff[NGROW], grow_am_ff[NGROW], grow_lnam_ff[NGROW],
      grow_iam_ff[NGROW];
  double chi_ida[NCHI];        // 1 / (atab_chi[i + 1] - atab_chi[i]) (i < NCHI - 1)
  double grow_ida[NGROW];      // 1 / (atab_grow[i + 1] - atab_grow[i]) (i < NGROW - 1)
  float2 chi_ida_ff[NCHI], grow_ida_ff[NGROW], logr_ff[NRT];  // pair copies of the three above
  float2 atab_chi_ff[NCHI];    // pair copy of atab_chi
  float2 chi_h6_ff[NCHI];      // (lna_chi[i] - lna_chi[i - 1]) / 6 as pairs (i >= 1; 0 at i = 0)
  float2 romb_w_ff[NROMB];     // pair copy of romb_w
};

// ------------------------------------------------- per-cosmology tables -----
// Scalars of one cosmology (FP64).  Index names for CosmoTab::s.
enum Scalar {
  S_OMEGA_C = 0, S_OMEGA_B, S_H, S_NS, S_SIGMA8, S_OMEGA_K, S_W0, S_WA,
  S_OMEGA_M, S_OMEGA_DE,
  // Eisenstein & Hu 1998 (transfer.py:47-153)
  S_K_EQ, S_Z_EQ, S_Z_D, S_R_D, S_R_EQ, S_SH_D, S_K_SILK, S_ALPHA_C, S_BETA_C,
  S_ALPHA_B, S_BETA_B, S_BETA_NODE, S_FB, S_FC,
  S_SIGMASQR8,  // power.py:56-78 at R = 8
  S_PKNORM,     // sigma8^2 / sigmasqr(8): power.py:47
  S_G1,         // growth_factor(a = 1) from the table (power.py:44 with a = 1)
  S_LGQ,        // log(13.41 k_eq): log q = log k - S_LGQ (transfer.py:122)
  S_LGKSILK,    // log(k_silk)
  S_QINV,       // 1 / (13.41 k_eq)
  S_ISH,        // 1 / sh_d
  S_C142AC,     // 14.2 / alpha_c
  S_AGAM,       // alpha_gamma of the no-wiggle fit (transfer.py:88-92)
  S_NWQ,        // (T_cmb / 2.7)^2 / (Omega_m h): q = k S_NWQ / (gamma_eff / (Omega_m h)) (transfer.py:93-100)
  S_TFNW,       // 1: transfer type "eisenhu" (no wiggles), 0: "eisenhu_osc"
  S_GAMMA,      // growth-rate index gamma (JCG_GROWTH_GAMMA), else 0
  S_NSCALAR
};
constexpr int NSCAL = 40;
// ln k grid of the spectral moments: simps over [ln 1e-4, ln 1e4], 256 intervals (power.py:136)
constexpr double LOG_KMIN = -0x1.26bb1bbb55515p+3;  // np.log(1e-4)
constexpr double DLOGK = (0x1.26bb1bbb55516p+3 - -0x1.26bb1bbb55515p+3) / 256.0;
constexpr double Y2_TAYLOR = 1.0;   // below: exp(-y^2) by its Taylor series (NTAYLOR terms)
constexpr double Y2_SKIP = 60.0;    // above: exp(-y^2) y^4 P k^3 < 1e-20 of the sum
constexpr int PAD_CT = 7;        // keeps sizeof(CosmoTab) a multiple of 64
static_assert(S_NSCALAR <= NSCAL, "scalar block too small");

// Per-cosmology Eisenstein-Hu inputs of the FP32 transfer function
// (transfer.py:47-97 reduced to the factors eh32_T multiplies by).
struct EH32 {
  float qinv, lg2_qinv, sh, inv_sh, c18bc, c142ac, alpha_b, beta_b, beta_node, lg2_ksilk, fb, fc,
      ns3;
  float agam, nwq;  // type "eisenhu": alpha_gamma, (T_cmb / 2.7)^2 / (Omega_m h)
  int nw;           // 1: type "eisenhu"
};
static_assert(sizeof(EH32) == 64, "EH32 is 64 bytes");

struct CosmoTab {
  double s[NSCAL];
  double chi[NCHI];    // background.py:231-233  chi table on atab_chi
  double g[NGROW];     // background.py:483      growth table on atab_grow
  double f[NGROW];     // background.py:485      growth rate dlnD/dlna on atab_grow
  double sig[NRT];     // sigma^2(R_j) at a = 1 without the g(a)^2 factor
  double pk3[NKH];     // linear_matter_power(k_i, a=1) * k_i^3
  double chi_slope[NCHI];  // slope of the chi table on segment [k, k+1] (k < 255)
  float chi32[NCHI];       // chi table, float (FP32 lensing kernel)
  float slope32[NCHI];     // chi_slope, float
  float wpk3f[NKH + 15];   // simpson_kh[i] * pk3[i], float (fp32c halofit moments); padded to 64 bytes
  // fp32c: the small-y part of the halofit moments as a Taylor series in y^2.
  // Float pairs R_m[i] = c_m Q_m[i], c_m = (-1)^m / m!,
  // Q_m[i] = sum_{k < i} w_k P(k_k) k_k^3 (k_k / k_i)^(2(m+1)), m < NTAYLOR
  float2 rtay[NTAYLOR][NKH + 1];
  EH32 eh32;               // fp32c Limber integrand's transfer inputs (from s)
  double pad[PAD_CT];
};
static_assert(sizeof(CosmoTab) % 64 == 0, "CosmoTab must keep 64-byte alignment");

// the EH32 of a cosmology from its scalars, once per cosmology (table stage)
__device__ inline void make_eh32(const double* s, EH32* e) {
  const double qinv = 1.0 / (13.41 * s[S_K_EQ]);
  e->qinv = (float)qinv;
  e->lg2_qinv = (float)log2(qinv);
  e->sh = (float)s[S_SH_D];
  e->inv_sh = (float)(1.0 / s[S_SH_D]);
  e->c18bc = (float)(1.8 * s[S_BETA_C]);
  e->c142ac = (float)(14.2 / s[S_ALPHA_C]);
  e->alpha_b = (float)s[S_ALPHA_B];
  e->beta_b = (float)s[S_BETA_B];
  e->beta_node = (float)s[S_BETA_NODE];
  e->lg2_ksilk = (float)log2(s[S_K_SILK]);
  e->fb = (float)s[S_FB];
  e->fc = (float)s[S_FC];
  e->ns3 = (float)(s[S_NS] + 3.0);
  e->agam = (float)s[S_AGAM];
  e->nwq = (float)s[S_NWQ];
  e->nw = s[S_TFNW] != 0.0;
}


// ------------------------------------------------- per-(cosmology, a) rows --
// FP64 row written by the halofit-row kernel for every Limber node.
enum Row64 {
  R_CHI = 0,   // radial_comoving_distance(a)              angular_cl.py:70
  R_G,         // growth_factor(a)                         power.py:44
  R_KNL,       // k_nl                                     power.py:118
  R_NEFF,      // n_eff                                    power.py:138
  R_C,         // C                                        power.py:139
  R_OMM,       // Omega_m(a)                               power.py:177
  R_OMDE,      // Omega_de(a)                              power.py:178
  R_W,         // w(a)                                     power.py:179
  R_DCHI,      // dchioverda(a)                            angular_cl.py:91
  R_AN, R_BN, R_CN, R_GAMMAN, R_ALPHAN, R_BETAN, R_NUN,    // power.py:200-224
  R_F1, R_F2, R_F3,                                        // power.py:228-238
  R_U,         // simpson weight * dchi / max(chi^2,1) / c^2
  R_LGKNL,     // log(k_nl)
  R_LGCF3,     // log(c_n f3)
  R_LGCHIC,    // log(max(chi, 1))
  R_MUN,       // mu_n (smith2003, power.py:197; 0 for takahashi2012, power.py:223)
  NROW64_USED
};
constexpr int NROW64 = 24;
static_assert(NROW64_USED <= NROW64, "row too small");

// FP32 row for the compensated fast path (derived, MUFU-friendly forms).
enum Row32 {
  F_INVCHI = 0,  // 1 / max(chi, 1)
  F_LG2INVCHI,   // log2(1 / max(chi, 1))
  F_LG2KNL,      // log2(k_nl)
  F_D2FAC,       // g^2 * pknorm / (2 pi^2)
  F_BETAN, F_ALPHAN, F_AN, F_3F1, F_F2, F_BN, F_LG2CF3, F_3MGAMMA, F_NUN,
  F_INVKNL,      // 1 / k_nl
  F_CHIC,        // max(chi, 1)
  F_MUN,         // mu_n
  NROW32_USED
};
constexpr int NROW32 = 16;
static_assert(NROW32_USED <= NROW32, "fp32 row too small");

// Physics switches of a request.
__host__ __device__ __forceinline__ int pk_model(int physics) { return physics & JCG_PK_MASK; }
__host__ __device__ __forceinline__ bool tf_nowiggle(int physics) { return (physics & JCG_TF_NOWIGGLE) != 0; }
__host__ __device__ __forceinline__ bool growth_gamma(int physics) { return (physics & JCG_GROWTH_GAMMA) != 0; }
// doubles per cosmology in a parameter array: 8, or 9 with gamma
__host__ __device__ __forceinline__ int param_stride(int physics) { return growth_gamma(physics) ? 9 : 8; }

// ------------------------------------------------------ geometry tables ----
// Cosmology-independent description of one request, stored at the start of the
// geometry buffer (device), followed by the tables at the offsets below
// (offsets in units of 8 bytes from the buffer start).
struct GeoHeader {
  int magic;
  int n_tr, n_wl, n_nc, n_ell, n_limber, na, n_cls, n_groups;
  int custom_nodes;        // 1: nodes are caller-given redshifts (in the z section)
  int kind[MAXTR];
  int group[MAXTR];        // lensing group (distinct probe zmax) of a WL tracer
  int pair_i[MAXPAIR], pair_j[MAXPAIR];
  double zmax;             // angular_cl.py:63
  double dx_limber;        // (1 - z2a(zmax)) / N
  double nz_a[MAXTR], nz_b[MAXTR], nz_z0[MAXTR], nz_zmax[MAXTR];
  double bias[MAXTR], mult[MAXTR], noise[MAXTR], probe_zmax[MAXTR];
  int bias_kind[MAXTR];    // JCG_BIAS_*: NC galaxy bias, WL NLA bias (NONE: no IA)
  double bias_eta[MAXTR], bias_z0[MAXTR];
  int special_bias;        // 1: some tracer has IA or a redshift-dependent bias
  int has_delta;           // 1: some WeakLensing tracer has a single-plane n(z)
  int physics;             // JCG_PK_* | JCG_TF_*
  int nz_kind[MAXTR];      // JCG_NZ_*
  int64_t nzp_off[MAXTR];  // offset of tracer t's points in the n(z) point list
  int64_t nzp_total;       // points over all tracers
  double group_zmax[MAXTR];
  double nz_norm[MAXTR];   // redshift.py:30
  // offsets (8-byte units)
  int64_t off_a, off_z, off_wsimp, off_awl;
  int64_t off_seg_chi, off_seg_grow, off_seg_chiwl;  // int32 pairs, packed as int64 per node
  int64_t off_nzl;                                   // [n_tr][na] n_t(z_n)
  int64_t off_ell, off_ellfac;                       // [n_ell], [n_tr][n_ell]
  int64_t off_lg2ellh;                               // [n_ell] log2(ell + 1/2) (fp32 path)
  int64_t off_kh4;                                   // [n_ell] float4 (l + 1/2, log2(l + 1/2), 1 / (l + 1/2), 0)
  int64_t off_ef32;                                  // [n_tr][n_ell] float ell factors
  int64_t off_ap[MAXTR];                             // per group [na][NZP] a' nodes
  int64_t off_segp[MAXTR];                           // per group [na][NZP] packed segments
  int64_t off_q32[MAXTR];      // per group [na][NZP] int32: nearest node | segment << 16
  int64_t off_dx32[MAXTR];     // per group [na][NZP] float: a' - atab_chi[nearest]
  int64_t off_W32[MAXTR];      // per WL tracer [na][NZP] float weights
  int64_t off_qwl32;           // [na] int32 chi_wl query (nearest | segment << 16)
  int64_t off_dxwl32;          // [na] float
  int64_t off_W[MAXTR];                              // per WL tracer [na][NZP] weights
  int64_t total;                                     // bytes / 8
};
constexpr int GEO_MAGIC = 0x4a434731;  // "JCG1"

// ----------------------------------------------------------- batch ---------
// A batch of items = (cosmology, geometry) pairs.  The uniform form derives
// every pointer from strides; the listed form reads an Item array (ragged
// requests of the serving loop).
struct Item {
  const double* params;  // 8 parameters
  const GeoHeader* geo;
  CosmoTab* ctab;
  double* rows64;        // [na][NROW64]
  float* rows32;         // [na][NROW32]
  double* kern;          // [n_tr][na]
  double* cl;            // [n_cls][n_ell] (output)
  int precision;
  int physics;           // JCG_PK_* | JCG_TF_*
  float* u32;            // fp32c, may be NULL: [na] the Limber weight u of the FP64 row, as float
  float* kern32;         // fp32c, may be NULL: [n_tr][na] the radial kernels, as float
};

struct Batch {
  int n_items;
  int listed;            // 0: uniform strides, 1: items[]
  const Item* items;
  // uniform form
  const double* params;
  const GeoHeader* geo;
  CosmoTab* ctab;
  double* rows64;
  float* rows32;
  double* kern;
  double* cl;
  float* u32;            // uniform fp32c form (else NULL): [n_items][max_na]
  float* kern32;         // uniform fp32c form (else NULL): [n_items][max_tr][max_na]
  int precision;
  int max_na, max_ell, max_cls, max_tr;
  int n_wl, n_wl_groups;  // uniform form: WeakLensing tracers and lensing groups
  int chi_wbase;          // uniform form: first chi table segment a Limber node or lensing point can fall in
  int special_bias;       // uniform form: IA or a redshift-dependent bias present
  int has_delta;          // uniform form: a single-plane WeakLensing n(z) present
  int physics;            // uniform form: JCG_PK_* | JCG_TF_*
  int physics_or;         // OR of the items' switches (selects kernel variants)
};

__device__ __forceinline__ Item batch_item(const Batch& b, int i) {
  if (b.listed) return b.items[i];
  Item it;
  const int na = b.max_na;
  it.params = b.params + (size_t)param_stride(b.physics) * i;
  it.geo = b.geo;
  it.ctab = b.ctab + i;
  it.rows64 = b.rows64 ? b.rows64 + (size_t)i * na * NROW64 : nullptr;
  it.rows32 = b.rows32 ? b.rows32 + (size_t)i * na * NROW32 : nullptr;
  it.kern = b.kern + (size_t)i * b.max_tr * na;
  it.cl = b.cl + (size_t)i * b.max_cls * b.max_ell;
  it.precision = b.precision;
  it.physics = b.physics;
  it.u32 = b.u32 ? b.u32 + (size_t)i * na : nullptr;
  it.kern32 = b.kern32 ? b.kern32 + (size_t)i * b.max_tr * na : nullptr;
  return it;
}

template <typename T>
__device__ __forceinline__ const T* geo_ptr(const GeoHeader* g, int64_t off) {
  return reinterpret_cast<const T*>(reinterpret_cast<const double*>(g) + off);
}

// ------------------------------------------------------- exact helpers -----
// numpy's float power uses fast paths for these scalar exponents
// (x**2 -> square, x**1 -> copy, x**0.5 -> sqrt, x**-1 -> reciprocal).
__device__ __forceinline__ double npow(double x, double y) {
  if (y == 2.0) return x * x;
  if (y == 1.0) return x;
  if (y == 0.5) return sqrt(x);
  if (y == -1.0) return 1.0 / x;
  if (y == 0.0) return 1.0;
  return pow(x, y);
}

// jnp.clip(x, lo) / jnp.clip(x, lo, hi)
__device__ __forceinline__ double clip_lo(double x, double lo) { return fmax(x, lo); }
__device__ __forceinline__ double clip_lohi(double x, double lo, double hi) {
  return fmin(fmax(x, lo), hi);
}

// numpy linspace node i of [start, stop] with `div` intervals: i*step + start,
// exact stop at i == div (numpy/core/function_base.py linspace).
__device__ __forceinline__ double np_linspace(double start, double stop, int div, int i) {
  if (i == div) return stop;
  const double step = (stop - start) / (double)div;
  return __dadd_rn(__dmul_rn((double)i, step), start);
}

// Nearest node of argmin((x - xp)^2) over an increasing table (first index on
// ties), found from a bracketing guess and a local scan; then the side rule of
// scipy/interpolate.py:47-57.  Returns packed (i0, i1) of the segment used.
__device__ __forceinline__ int2 interp_segment_inc(double x, const double* xp, int n, int guess) {
  int lo = guess < 0 ? 0 : (guess > n - 1 ? n - 1 : guess);
  // walk to the bracketing position: xp[lo] <= x < xp[lo+1] (or an end)
  while (lo > 0 && xp[lo] > x) --lo;
  while (lo < n - 1 && xp[lo + 1] <= x) ++lo;
  // candidates lo-1 .. lo+2, argmin with first-index tie rule
  int best = -1;
  double bestd = 0.0;
  for (int j = lo - 1; j <= lo + 2; ++j) {
    if (j < 0 || j >= n) continue;
    const double d = x - xp[j];
    const double d2 = d * d;
    if (best < 0 || d2 < bestd) { best = j; bestd = d2; }
  }
  int ind = best < 1 ? 1 : (best > n - 2 ? n - 2 : best);
  const double xc = clip_lohi(x, xp[1], xp[n - 2]);
  const double sgn = xc - xp[ind];
  const int s = (sgn >= 0.0) ? 1 : -1;  // copysign(1, sign(.)) with sign(0) = 0 -> +1
  return make_int2(ind, ind + s);
}

// The linear evaluation of scipy/interpolate.py:55-59 on a chosen segment.
__device__ __forceinline__ double interp_eval(double x, const double* xp, const double* fp, int2 seg) {
  const double a = (fp[seg.y] - fp[seg.x]) / (xp[seg.y] - xp[seg.x]);
  const double b = fp[seg.x] - a * xp[seg.x];
  return a * x + b;
}

__device__ __forceinline__ int64_t pack_seg(int2 s) {
  return (int64_t)(((uint64_t)(uint32_t)s.y << 32) | (uint32_t)s.x);
}
__device__ __forceinline__ int2 unpack_seg(int64_t v) {
  return make_int2((int)(uint32_t)(v & 0xffffffffu), (int)(uint32_t)((uint64_t)v >> 32));
}

// Guess for logspace(-3, 0, n): position of x in log10 units.
__device__ __forceinline__ int logspace_guess(double x, int n) {
  if (!(x > 0.0)) return 0;
  const double t = (log10(x) + 3.0) * (double)(n - 1) / 3.0;
  if (t < 0.0) return 0;
  if (t > (double)(n - 1)) return n - 1;
  return (int)t;
}

// 2^(j/64), j = 0..63, correctly rounded (table of the exponential below).
__device__ __constant__ const double kExp2Tab64[64] = {
    0x1.0000000000000p+0, 0x1.02c9a3e778061p+0, 0x1.059b0d3158574p+0, 0x1.0874518759bc8p+0,
    0x1.0b5586cf9890fp+0, 0x1.0e3ec32d3d1a2p+0, 0x1.11301d0125b51p+0, 0x1.1429aaea92de0p+0,
    0x1.172b83c7d517bp+0, 0x1.1a35beb6fcb75p+0, 0x1.1d4873168b9aap+0, 0x1.2063b88628cd6p+0,
    0x1.2387a6e756238p+0, 0x1.26b4565e27cddp+0, 0x1.29e9df51fdee1p+0, 0x1.2d285a6e4030bp+0,
    0x1.306fe0a31b715p+0, 0x1.33c08b26416ffp+0, 0x1.371a7373aa9cbp+0, 0x1.3a7db34e59ff7p+0,
    0x1.3dea64c123422p+0, 0x1.4160a21f72e2ap+0, 0x1.44e086061892dp+0, 0x1.486a2b5c13cd0p+0,
    0x1.4bfdad5362a27p+0, 0x1.4f9b2769d2ca7p+0, 0x1.5342b569d4f82p+0, 0x1.56f4736b527dap+0,
    0x1.5ab07dd485429p+0, 0x1.5e76f15ad2148p+0, 0x1.6247eb03a5585p+0, 0x1.6623882552225p+0,
    0x1.6a09e667f3bcdp+0, 0x1.6dfb23c651a2fp+0, 0x1.71f75e8ec5f74p+0, 0x1.75feb564267c9p+0,
    0x1.7a11473eb0187p+0, 0x1.7e2f336cf4e62p+0, 0x1.82589994cce13p+0, 0x1.868d99b4492edp+0,
    0x1.8ace5422aa0dbp+0, 0x1.8f1ae99157736p+0, 0x1.93737b0cdc5e5p+0, 0x1.97d829fde4e50p+0,
    0x1.9c49182a3f090p+0, 0x1.a0c667b5de565p+0, 0x1.a5503b23e255dp+0, 0x1.a9e6b5579fdbfp+0,
    0x1.ae89f995ad3adp+0, 0x1.b33a2b84f15fbp+0, 0x1.b7f76f2fb5e47p+0, 0x1.bcc1e904bc1d2p+0,
    0x1.c199bdd85529cp+0, 0x1.c67f12e57d14bp+0, 0x1.cb720dcef9069p+0, 0x1.d072d4a07897cp+0,
    0x1.d5818dcfba487p+0, 0x1.da9e603db3285p+0, 0x1.dfc97337b9b5fp+0, 0x1.e502ee78b3ff6p+0,
    0x1.ea4afa2a490dap+0, 0x1.efa1bee615a27p+0, 0x1.f50765b6e4540p+0, 0x1.fa7c1819e90d8p+0,
};

// exp(x) for -700 < x <= 0 by the table-driven method of P. T. P. Tang
// ("Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15, 1989): x = (64 m + j) ln2/64 + r
// with |r| <= ln2/128, exp(x) = 2^m 2^(j/64) e^r, e^r by its Taylor polynomial
// of degree 6 (truncation < 3e-20 relative).  ln2/64 is split in a 40-bit
// high part (exact products for |k| < 2^13) and the rest.  `tab` is a copy of
// kExp2Tab64 in shared memory (lanes index it independently).
__device__ __forceinline__ double exp_tang(double x, const double* tab) {
  constexpr double INV_LN2_64 = 92.33248261689366;
  constexpr double LN2_64_HI = 0x1.62e42fefa2000p-7;
  constexpr double LN2_64_LO = 0x1.9ef35793c7673p-47;
  const double kd = rint(x * INV_LN2_64);
  const double r = fma(-kd, LN2_64_LO, fma(-kd, LN2_64_HI, x));
  double p = 1.0 / 720.0;
  p = fma(p, r, 1.0 / 120.0);
  p = fma(p, r, 1.0 / 24.0);
  p = fma(p, r, 1.0 / 6.0);
  p = fma(p, r, 0.5);
  p = fma(p, r, 1.0);
  p = fma(p, r, 1.0);
  const int k = (int)kd;
  const double two_m = __hiloint2double(((k >> 6) + 1023) << 20, 0);
  return tab[k & 63] * p * two_m;
}

// --------------------------------------------------------- background ------
// background.py:25-196, 270-294 with the reference operation order.
struct Bg {
  double Om, Ok, Ode, w0, wa;
};
__device__ __forceinline__ Bg make_bg(const double* s) {
  Bg b;
  b.Om = s[S_OMEGA_M];
  b.Ok = s[S_OMEGA_K];
  b.Ode = s[S_OMEGA_DE];
  b.w0 = s[S_W0];
  b.wa = s[S_WA];
  return b;
}
__device__ __forceinline__ double bg_w(const Bg& c, double a) { return c.w0 + (1.0 - a) * c.wa; }
// f_de with ln a given (background.py:90)
__device__ __forceinline__ double bg_fde_l(const Bg& c, double a, double lna) {
  return -3.0 * (1.0 + c.w0 + c.wa) * lna + 3.0 * c.wa * (a - 1.0);
}
__device__ __forceinline__ double bg_fde(const Bg& c, double a) { return bg_fde_l(c, a, log(a)); }
// E^2(a) (background.py:122-126); a^-3, a^-2 by products of 1/a (no float64
// pow), exp(f_de) skipped when f_de == 0 (w0 = -1, wa = 0), where it is 1.
__device__ __forceinline__ double bg_esqr_l(const Bg& c, double a, double lna, double* efde) {
  const double f = bg_fde_l(c, a, lna);
  const double ef = (f == 0.0) ? 1.0 : exp(f);
  if (efde) *efde = ef;
  const double ia = 1.0 / a, ia2 = ia * ia;
  return c.Om * (ia2 * ia) + c.Ok * ia2 + c.Ode * ef;
}
__device__ __forceinline__ double bg_esqr(const Bg& c, double a) { return bg_esqr_l(c, a, log(a), nullptr); }
__device__ __forceinline__ double bg_H(const Bg& c, double a) { return H0 * sqrt(bg_esqr(c, a)); }

// ---------------------------------------------------- background scans ----
// One RK4 step of the growth ODE (background.py:96-111) from (y0, y1) = (D, dD/da):
// dy0/da = y1, dy1/da = -q y1 + r y0, coefficients at the step's start (qa0,
// ra0), midpoint (qm, rm) and end (qa1, ra1).
template <class T>
__device__ __forceinline__ void growth_rk4_step(const T& y0, const T& y1, const T& qa0, const T& ra0, const T& qm,
                                                const T& rm, const T& qa1, const T& ra1, double hh, T& o0, T& o1) {
  const T k1a = y1, k1b = -qa0 * y1 + ra0 * y0;
  const T y0b = y0 + hh * k1a / 2, y1b = y1 + hh * k1b / 2;
  const T k2a = y1b, k2b = -qm * y1b + rm * y0b;
  const T y0c = y0 + hh * k2a / 2, y1c = y1 + hh * k2b / 2;
  const T k3a = y1c, k3b = -qm * y1c + rm * y0c;
  const T y0d = y0 + hh * k3a, y1d = y1 + hh * k3b;
  const T k4a = y1d, k4b = -qa1 * y1d + ra1 * y0d;
  o0 = y0 + 1.0 / 6.0 * hh * (k1a + 2 * k2a + 2 * k3a + k4a);
  o1 = y1 + 1.0 / 6.0 * hh * (k1b + 2 * k2b + 2 * k3b + k4b);
}

// 2 x 2 row-major products: r = a b, and a vector v <- a v
__device__ __forceinline__ void mat2_mul(const double* a, const double* b, double* r) {
  const double r0 = a[0] * b[0] + a[1] * b[2], r1 = a[0] * b[1] + a[1] * b[3];
  const double r2 = a[2] * b[0] + a[3] * b[2], r3 = a[2] * b[1] + a[3] * b[3];
  r[0] = r0, r[1] = r1, r[2] = r2, r[3] = r3;
}

// Growth ODE values from the per-step matrices Mv[i] (2 x 2 row-major,
// Mv[0] = I; y_i = M_i y_{i-1}) for one warp: y_i = M_i ... M_1 y_0 by a
// warp scan of matrix products, lane l holding steps 4l .. 4l + 3.  Returns
// D at the lane's 4 nodes in d4 and writes y_i to Yv[i][2] if Yv is set; the
// result is D at the last node.
__device__ __forceinline__ double growth_scan_warp(const double* Mv, double ya, double yb, int lane, double* d4,
                                                   double* Yv) {
  double A[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) A[q] = Mv[lane * 16 + q];
  for (int k = 1; k < 4; ++k) mat2_mul(Mv + (lane * 4 + k) * 4, A, A);
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    double P[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) P[q] = __shfl_up_sync(0xffffffffu, A[q], o);
    if (lane >= o) mat2_mul(A, P, A);
  }
  double E[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) E[q] = __shfl_up_sync(0xffffffffu, A[q], 1);
  if (lane == 0) E[0] = 1.0, E[1] = 0.0, E[2] = 0.0, E[3] = 1.0;
  double u0 = E[0] * ya + E[1] * yb, u1 = E[2] * ya + E[3] * yb;
  for (int k = 0; k < 4; ++k) {
    const double* M = Mv + (lane * 4 + k) * 4;
    const double v0 = M[0] * u0 + M[1] * u1, v1 = M[2] * u0 + M[3] * u1;
    u0 = v0, u1 = v1;
    d4[k] = u0;
    if (Yv) {
      Yv[(lane * 4 + k) * 2 + 0] = u0;
      Yv[(lane * 4 + k) * 2 + 1] = u1;
    }
  }
  return __shfl_sync(0xffffffffu, u0, 31);
}

// chi table (background.py:227-233) for one warp: prefix sums of the RK4
// increments h/6 (f_{i-1} + 2 fm_i + 2 fm_i + f_i) in ln a (scipy/ode.py:21,
// the first step has h = 0), then chi_i = Y[-1] - Y_i.  fnode: f at the
// nodes; fmid[i]: f at the midpoint of step i (i >= 1).  Lane l holds nodes
// 8l .. 8l + 7; the sums are associated per lane, then across lanes.
__device__ __forceinline__ void chi_scan_warp(const double* fnode, const double* fmid, const double* lna, int lane,
                                              double* out) {
  double loc[8], s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int i = lane * 8 + k;
    if (i > 0) {
      const double hh = lna[i] - lna[i - 1];
      s += 1.0 / 6.0 * hh * (fnode[i - 1] + 2 * fmid[i] + 2 * fmid[i] + fnode[i]);
    }
    loc[k] = s;
  }
  double x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double u = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += u;
  }
  double off = __shfl_up_sync(0xffffffffu, x, 1);
  if (lane == 0) off = 0.0;
  const double tot = __shfl_sync(0xffffffffu, x, 31);
#pragma unroll
  for (int k = 0; k < 8; ++k) out[lane * 8 + k] = tot - (off + loc[k]);
}

// ------------------------------------------------------ bias models -------
constexpr double IA_C1_RHOCRIT = 5e-14 * 2.7750e11;  // C_1 rho_crit (constants.py), NLA normalisation

// growth_factor(cosmo, a) (background.py:371-398): clip(interp(a), 0, 1)
__device__ __forceinline__ double growth_at(const double* gtab, const ConstTables* c, double a) {
  const int2 sg = interp_segment_inc(a, c->atab_grow, NGROW, logspace_guess(a, NGROW));
  return clip_lohi(interp_eval(a, c->atab_grow, gtab, sg), 0.0, 1.0);
}

// b(cosmo, z) of tracer t's bias model (bias.py:10-57), D = growth_factor(z2a(z))
__device__ __forceinline__ double bias_at(const GeoHeader* g, int t, double z, double D) {
  switch (g->bias_kind[t]) {
    case JCG_BIAS_INV_GROWTH: return g->bias[t] / D;
    case JCG_BIAS_DES_Y1: return g->bias[t] * pow((1.0 + z) / (1.0 + g->bias_z0[t]), g->bias_eta[t]);
    default: return g->bias[t];
  }
}
// Omega_m(a), Omega_de(a) sharing one E^2 (background.py:168, 196)
__device__ __forceinline__ void bg_om_l(const Bg& c, double a, double lna, double* omm, double* omde) {
  double ef;
  const double e2 = bg_esqr_l(c, a, lna, &ef);
  const double ia = 1.0 / a;
  *omm = c.Om * (ia * ia * ia) / e2;
  *omde = c.Ode * ef / e2;
}
__device__ __forceinline__ double bg_omm(const Bg& c, double a) {
  double m, d;
  bg_om_l(c, a, log(a), &m, &d);
  return m;
}
__device__ __forceinline__ double bg_omde(const Bg& c, double a) {
  double m, d;
  bg_om_l(c, a, log(a), &m, &d);
  return d;
}
// dchi/da = rh / (a^2 E(a)) (background.py:294)
__device__ __forceinline__ double bg_dchioverda_l(const Bg& c, double a, double lna) {
  return RH / ((a * a) * sqrt(bg_esqr_l(c, a, lna, nullptr)));
}
__device__ __forceinline__ double bg_dchioverda(const Bg& c, double a) {
  return bg_dchioverda_l(c, a, log(a));
}

// ------------------------------------------------------ Eisenstein & Hu ----
// transfer.py:107-153 (eisenhu_osc), per-k part, FP64, at k with lk = log k
// and ik = 1 / k.  Powers are taken as exp(y log x) with the logs shared
// between terms (log k, log q); the divisions are shared too: one reciprocal
// for the three T_tilde denominators, one for the three damping factors, and
// rcbrt for tilde_s.  On GB300 a float64 pow costs about two exps and a
// division about ten float64 operations; the shared forms change results only
// at the 1e-15 level.
__device__ __forceinline__ double eh_osc_lki(const double* s, double k, double lk, double ik) {
  const double sh_d = s[S_SH_D];
  const double q = k * s[S_QINV];
  const double q108 = exp(1.08 * (lk - s[S_LGQ]));
  const double Cb = 386.0 / (1.0 + 69.9 * q108);
  const double qq = q * q;
  const double L1 = log(EULER_E + 1.8 * s[S_BETA_C] * q);
  const double L2 = log(EULER_E + 1.8 * q);
  const double da = L1 + (14.2 + Cb) * qq;
  const double db = L1 + (s[S_C142AC] + Cb) * qq;
  const double dn = L2 + (14.2 + Cb) * qq;
  const double dab = da * db;
  const double r3 = 1.0 / (dab * dn);
  const double Ta = L1 * (db * dn) * r3;
  const double Tb = L1 * (da * dn) * r3;
  const double Tn = L2 * dab * r3;
  const double ksh = k * sh_d, iksh = ik * s[S_ISH];
  const double x54 = ksh * (1.0 / 5.4), x54s = x54 * x54;
  const double x52 = ksh * (1.0 / 5.2);
  const double bb = s[S_BETA_B] * iksh;
  const double bn = s[S_BETA_NODE] * iksh;
  const double d1 = 1.0 + x54s * x54s, d2 = 1.0 + x52 * x52, d3 = 1.0 + bb * bb * bb;
  const double d12 = d1 * d2;
  const double r6 = 1.0 / (d12 * d3);
  const double f = d2 * d3 * r6;
  const double Tc = f * Ta + (1.0 - f) * Tb;
  const double tilde_s = sh_d * rcbrt(1.0 + bn * bn * bn);
  const double silk = exp(-exp(1.4 * (lk - s[S_LGKSILK])));
  const double arg = k * tilde_s;
  const double sinc = sin(arg) / arg;
  const double Tbar = (Tn * (d1 * d3 * r6) + s[S_ALPHA_B] * (d12 * r6) * silk) * sinc;
  return s[S_FB] * Tbar + s[S_FC] * Tc;
}

// type "eisenhu" (transfer.py:88-105): gamma_eff = Omega_m h (alpha_g +
// (1 - alpha_g) / (1 + (0.43 k s)^4)), q = k (T_cmb / 2.7)^2 / gamma_eff
__device__ __forceinline__ double eh_nowiggle(const double* s, double k) {
  const double x = 0.43 * k * s[S_SH_D], x2 = x * x;
  const double ag = s[S_AGAM];
  const double q = k * s[S_NWQ] / (ag + (1.0 - ag) / (1.0 + x2 * x2));
  const double L = log(2.0 * EULER_E + 1.8 * q);
  const double C = 14.2 + 731.0 / (1.0 + 62.5 * q);
  return L / (L + C * q * q);
}

// T(k) of the cosmology's transfer type (S_TFNW); NW = false: the scalars
// are known to hold type "eisenhu_osc"
template <bool NW = true>
__device__ __forceinline__ double eh_transfer_lki(const double* s, double k, double lk, double ik) {
  if (NW && s[S_TFNW] != 0.0) return eh_nowiggle(s, k);
  return eh_osc_lki(s, k, lk, ik);
}

__device__ __forceinline__ double eh_transfer_lk(const double* s, double k, double lk) {
  return eh_transfer_lki(s, k, lk, 1.0 / k);
}

__device__ __forceinline__ double eh_transfer(const double* s, double k) {
  return eh_transfer_lk(s, k, log(k));
}

// dchi/dln a = dchioverda(a) a = R_H / (a sqrt(E^2(a))) (background.py:227-229)
// with ln a and 1 / a given
__device__ __forceinline__ double dchi_dlna_c(const Bg& b, double a, double lna, double ia) {
  const double f = bg_fde_l(b, a, lna);
  const double ef = (f == 0.0) ? 1.0 : exp(f);
  const double ia2 = ia * ia;
  const double e2 = b.Om * (ia2 * ia) + b.Ok * ia2 + b.Ode * ef;
  return RH * ia * rsqrt(e2);
}

// growth ODE coefficients D'' = -q D' + r D (background.py:96-106) with ln x
// and 1 / x given
__device__ __forceinline__ void growth_qr_c(const Bg& b, double x, double lnx, double ix, double& q, double& r) {
  const double f = bg_fde_l(b, x, lnx);
  const double ef = (f == 0.0) ? 1.0 : exp(f);
  const double ix2 = ix * ix, ix3 = ix2 * ix;
  const double ie2 = 1.0 / (b.Om * ix3 + b.Ok * ix2 + b.Ode * ef);
  const double omm = b.Om * ix3 * ie2, omde = b.Ode * ef * ie2;
  q = (2.0 - 0.5 * (omm + (1.0 + 3.0 * bg_w(b, x)) * omde)) * ix;
  r = 1.5 * omm * ix2;
}

// linear_matter_power(k, a) with g = growth_factor(a): power.py:42-53
__device__ __forceinline__ double pk_linear_lk(const double* s, double k, double lk, double g) {
  const double t = eh_transfer_lk(s, k, lk);
  double pk = exp(s[S_NS] * lk) * (t * t) * (g * g);
  return pk * s[S_PKNORM];
}
__device__ __forceinline__ double pk_linear(const double* s, double k, double g) {
  return pk_linear_lk(s, k, log(k), g);
}

// Non-linear power at one node (power.py:246-260), FP64, with log k given and
// the row's log k_nl and log(c_n f3): halofit (takahashi2012 or smith2003 by
// the row's coefficients; d2h = d2h' / (1 + mu/y + nu/y^2) evaluated as
// d2h' y^2 / (y^2 + mu y + nu)), or the linear power for JCG_PK_LINEAR
// (nonlinear_fn = linear_matter_power).
__device__ __forceinline__ double halofit_node_lk(const double* s, const double* row, double k,
                                                  double lk, int model) {
  const double pklin = pk_linear_lk(s, k, lk, row[R_G]);
  if (model == JCG_PK_LINEAR) return pklin;
  const double k3 = k * k * k;
  const double d2l = k3 * pklin / (2.0 * (PI * PI));
  const double y = k / row[R_KNL];
  const double ly = lk - row[R_LGKNL];
  const double fy = y / 4.0 + (y * y) / 8.0;
  const double d2q =
      d2l * (exp(row[R_BETAN] * log(1.0 + d2l)) / (1 + row[R_ALPHAN] * d2l)) * exp(-fy);
  const double d2hprime =
      row[R_AN] * exp(3 * row[R_F1] * ly) /
      (1.0 + row[R_BN] * exp(row[R_F2] * ly) + exp((3.0 - row[R_GAMMAN]) * (row[R_LGCF3] + ly)));
  const double y2 = y * y;
  const double d2h = d2hprime * y2 / ((y2 + row[R_MUN] * y) + row[R_NUN]);
  return 2.0 * (PI * PI) / k3 * (d2q + d2h);
}
__device__ __forceinline__ double halofit_node(const double* s, const double* row, double k, int model) {
  return halofit_node_lk(s, row, k, log(k), model);
}

// ------------------------------------------------------------- launches ----
// Host-side launchers implemented in the kernel translation units.
void launch_const_init(ConstTables* c, cudaStream_t st);
void launch_geometry_build(const GeoHeader& h, double* geo, const double* pz, const ConstTables* c,
                           cudaStream_t st);
void launch_nz_points(const GeoHeader& h, const double* z_nodes, double* out, cudaStream_t st);
void launch_cosmo_tables(const Batch& b, const ConstTables* c, cudaStream_t st);
void launch_halofit_rows(const Batch& b, const ConstTables* c, cudaStream_t st);
// a lensing point's record (segment query, offset, the NW weights) as float4s,
// staged per warp in shared memory and read back by broadcast (fewer
// shared-memory/shuffle operations per point than one shuffle per value)
template <int NW>
struct KuRec {
  static constexpr int N4 = (NW + 2 + 3) / 4;
};
__host__ __device__ inline size_t ku_rec_bytes(int nw) { return sizeof(float4) * 8 * 32 * (size_t)((nw + 2 + 3) / 4); }
template <int NW>
__device__ __forceinline__ void ku_put_rec(float4* rec, int q, float dx, const float* w) {
  float v[4 * KuRec<NW>::N4];
  v[0] = __int_as_float(q);
  v[1] = dx;
#pragma unroll
  for (int u = 0; u < NW; ++u) v[2 + u] = w[u];
#pragma unroll
  for (int u = NW + 2; u < 4 * KuRec<NW>::N4; ++u) v[u] = 0.f;
#pragma unroll
  for (int i = 0; i < KuRec<NW>::N4; ++i) rec[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
}
template <int NW>
__device__ __forceinline__ void ku_get_rec(const float4* rec, int& q, float& dx, float* w) {
  float v[4 * KuRec<NW>::N4];
#pragma unroll
  for (int i = 0; i < KuRec<NW>::N4; ++i) {
    const float4 r = rec[i];
    v[4 * i] = r.x, v[4 * i + 1] = r.y, v[4 * i + 2] = r.z, v[4 * i + 3] = r.w;
  }
  q = __float_as_int(v[0]);
  dx = v[1];
#pragma unroll
  for (int u = 0; u < NW; ++u) w[u] = v[2 + u];
}

void launch_tracer_kernels(const Batch& b, const ConstTables* c, cudaStream_t st);
void launch_limber(const Batch& b, const ConstTables* c, int lt, cudaStream_t st);
// derivatives (jcg_grad.cu)
size_t grad_workspace_bytes(const GeoHeader& h, int n_cosmo, int precision);
void grad_run(const GeoHeader* geo, const GeoHeader& h, const double* params, int n_cosmo, int precision,
              double* cl, double* jac, void* ws, const ConstTables* c, cudaStream_t st, int gamma_dir = -1,
              const int* seg_in = nullptr, int* seg_out = nullptr);
// one request of a ragged Jacobian batch; cl / jac NULL: carved from the workspace
struct GradReq {
  const GeoHeader* h;      // host copy of the header
  const GeoHeader* geo;    // device geometry
  const double* params;    // device, 8 parameters
  double* cl;
  double* jac;
  double* out;             // log-likelihood + gradient [9] (vector-Jacobian form)
  double* vbar;            // the likelihood's cotangent of C_ell (set by grad_run_listed, vector-Jacobian form)
};
int grad_listed_auto_split(const GradReq* r, int n, int precision);
// vjp: the vector-Jacobian form (fp32c log-likelihood requests): no Jacobian,
// the items' C_ell by the forward form of the product kernel; the caller then
// forms the cotangents and launches launch_vjp32_grad on *gb_out
size_t grad_listed_bytes(const GradReq* r, int n, int n_split, int precision, bool vjp = false);
struct GradBatch;
cudaError_t grad_run_listed(GradReq* r, int n, int n_split, int precision, void* ws, const ConstTables* c,
                            cudaStream_t st, bool vjp = false, GradBatch* gb_out = nullptr);
void launch_vjp32_grad(const GradBatch& gb, cudaStream_t st, unsigned stages);
// vector-Jacobian product of angular_cl, uniform batch (jcg_grad.cu)
size_t vjp_workspace_bytes(const GeoHeader& h, int n_cosmo, int precision);
void vjp_run(const GeoHeader* geo, const GeoHeader& h, const double* params, int n_cosmo, int precision,
             const double* vbar, double* cl, double* grad, void* ws, const ConstTables* c, cudaStream_t st,
             int gamma_dir, unsigned stages = 31u);
// host-to-device copy of a small host table through a pinned staging ring of
// the calling thread (jcg_api.cu): returns without waiting for the stream
cudaError_t stage_h2d(void* dst_dev, const void* src_host, size_t bytes, cudaStream_t st);
// log-likelihood and its gradient for a fixed inverse covariance (jcg_stats.cu)
struct ReqLL {
  const double* cl;     // [n_cls][n_ell]
  const double* jac;    // [n_cls][n_ell][8], or NULL: the cotangent form below
  double* vbar;         // [n_cls][n_ell]: receives -P r (d logL / dC_ell) when jac is NULL
  const double* data;   // [n_cls * n_ell]
  const double* prec;   // [n_ell][n_cls][n_cls]
  double* out;          // [9]
  double* part;         // [n_tiles][9] partial sums of the ell tiles (workspace)
  int n_cls, n_ell;
};
constexpr int RL_ELL = 8;  // ell per CTA of the request log-likelihood
__host__ __device__ inline int rl_tiles(int n_ell) { return (n_ell + RL_ELL - 1) / RL_ELL; }
void launch_request_loglike(const ReqLL* items_dev, int n, int max_tiles, int max_cls, cudaStream_t st);
// pointwise queries of the table functions (API: background / power modules)
void launch_eval_points(const double* params, int n_cosmo, CosmoTab* ctab, const ConstTables* c,
                        const double* a, const double* k, int n, int what, double* out,
                        cudaStream_t st);

}  // namespace jcg
