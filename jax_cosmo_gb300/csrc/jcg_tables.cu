// Table builds: the device-wide constant grids, the per-request geometry tables
// and the per-cosmology background / normalisation tables (FP64).
//
// jax_cosmo references: background.py:199-242 (chi), background.py:443-488
// (growth), power.py:56-78 (sigmasqr / romb), power.py:86-111 (sigma^2(R)),
// redshift.py:27-31 (n(z) normalisation), probes.py:16-99 (tracer grids),
// angular_cl.py:63-96 (Limber grid).
#include "jcg_fp32.cuh"
#include "jcg_internal.cuh"
#include "jcg_dual.cuh"
#include "jcg_ff.cuh"

namespace jcg {

// np.log(1e-4), np.log(1e4), np.log(1e1) as NumPy returns them.
__device__ __constant__ double kLogKMin = -0x1.26bb1bbb55515p+3;
__device__ __constant__ double kLogKMax = 0x1.26bb1bbb55516p+3;
__device__ __constant__ double kLogRMax = 0x1.26bb1bbb55516p+1;

// ------------------------------------------------------------ constants -----
__global__ void const_init_kernel(ConstTables* c) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  // logspace(-3, 0, n) = 10 ** linspace(-3, 0, n)
  for (int i = tid; i < NCHI; i += nth) {
    const double y = np_linspace(-3.0, 0.0, NCHI - 1, i);
    const double a = pow(10.0, y);
    c->atab_chi[i] = a;
    const double x = log(a);
    c->lna_chi[i] = x;
    c->chi_a[i] = exp(x);
    c->chi_ia[i] = 1.0 / exp(x);
    double xm = 0.0;
    if (i > 0) {
      const double x0 = log(pow(10.0, np_linspace(-3.0, 0.0, NCHI - 1, i - 1)));
      xm = x0 + (x - x0) / 2;
    }
    c->chi_lnam[i] = xm;
    c->chi_am[i] = i > 0 ? exp(xm) : 0.0;
    c->chi_iam[i] = i > 0 ? 1.0 / exp(xm) : 0.0;
  }
  for (int i = tid; i < NGROW; i += nth) {
    const double x = pow(10.0, np_linspace(-3.0, 0.0, NGROW - 1, i));
    c->atab_grow[i] = x;
    c->grow_lna[i] = log(x);
    c->grow_ia[i] = 1.0 / x;
    double xm = 0.0;
    if (i > 0) {
      const double xp = pow(10.0, np_linspace(-3.0, 0.0, NGROW - 1, i - 1));
      xm = xp + (x - xp) / 2;
    }
    c->grow_am[i] = xm;
    c->grow_lnam[i] = i > 0 ? log(xm) : 0.0;
    c->grow_iam[i] = i > 0 ? 1.0 / xm : 0.0;
  }
  const double dxk = (kLogKMax - kLogKMin) / 256.0;
  for (int i = tid; i < NKH; i += nth) {
    const double lk = np_linspace(kLogKMin, kLogKMax, NKH - 1, i);
    const double k = exp(lk);
    c->logk[i] = lk;
    c->kh[i] = k;
    c->ikh[i] = 1.0 / k;
    c->kh3[i] = pow(k, 3.0);
    const double w = (i == 0 || i == NKH - 1) ? 1.0 : ((i & 1) ? 4.0 : 2.0);
    const double sw = dxk / 3 * w;
    c->simpson_kh[i] = sw;
    c->simpson_f[i] = (float)sw;
    const double k2 = k * k;
    c->kh2_hi[i] = (float)k2;
    c->kh2_lo[i] = (float)(k2 - (double)(float)k2);
    if (i == NKH - 1) {
      const double kv2 = k2 * exp(2.0 * DLOGK);
      c->kh2_hi[NKH] = (float)kv2;
      c->kh2_lo[NKH] = (float)(kv2 - (double)(float)kv2);
    }
    double kp = k2;
    for (int m = 0; m < NTAYLOR; ++m) {
      c->kpw[m][i] = sw * kp;
      kp *= k2;
    }
  }
  for (int j = tid; j < NRT; j += nth) {
    c->logr[j] = np_linspace(kLogKMin, kLogRMax, NRT - 1, j);
  }
  for (int m = tid; m < NTAYLOR; m += nth) {
    const double rho = exp(-2.0 * DLOGK * (m + 1));
    double cm = 1.0;
    for (int j = 1; j <= m; ++j) cm /= (double)j;
    if (m & 1) cm = -cm;
    c->tay_rho[m][0] = (float)rho;
    c->tay_rho[m][1] = (float)(rho - (double)(float)rho);
    c->tay_c[m][0] = (float)cm;
    c->tay_c[m][1] = (float)(cm - (double)(float)cm);
  }
  // romb(int_sigma, -4, 3, divmax=7) abscissae in evaluation order
  // (scipy/integrate.py:129-146): a, b, then the new midpoints of each level.
  if (tid == 0) {
    const double a = -4.0, b = 3.0;
    int pos = 0;
    c->romb_logk[pos++] = a;
    c->romb_logk[pos++] = b;
    for (int lev = 1; lev <= 7; ++lev) {
      const int numtosum = (1 << lev) / 2;
      const double h = (1.0 * b - 1.0 * a) / numtosum;
      const double lox = a + 0.5 * h;
      for (int m = 0; m < numtosum; ++m) c->romb_logk[pos++] = lox + h * (double)m;
    }
  }
  __syncthreads();
  for (int e = tid; e < NROMB; e += nth) {
    const double k = exp(c->romb_logk[e]);
    const double x = k * 8.0;
    const double wf = 3.0 * (sin(x) - x * cos(x)) / (x * x * x);
    const double kw = k * wf;
    c->romb_k[e] = k;
    c->romb_ik[e] = 1.0 / k;
    c->romb_kw2[e] = k * (kw * kw);
  }
  // romb is linear in the integrand values: the weight of abscissa e is the
  // combination (scipy/integrate.py:131-159, divmax = 7) of the unit vector e
  for (int e = tid; e < NROMB; e += nth) {
    const double a = -4.0, b = 3.0, intrange = b - a;
    double ordsum = 0.5 * ((e == 0 ? 1.0 : 0.0) + (e == 1 ? 1.0 : 0.0));
    double state[8];
    for (int i = 0; i < 8; ++i) state[i] = intrange * ordsum;
    int pos = 2;
    for (int lev = 1; lev <= 7; ++lev) {
      const int n = 1 << lev, numtosum = n / 2;
      ordsum += (e >= pos && e < pos + numtosum) ? 1.0 : 0.0;
      pos += numtosum;
      double x = intrange * ordsum / (double)n;
      double ns[8];
      ns[0] = x;
      for (int kk = 0; kk < 7; ++kk) {
        const double tmp = ldexp(1.0, 2 * (kk + 1));
        x = (tmp * x - state[kk]) / (tmp - 1.0);
        ns[kk + 1] = x;
      }
      for (int i = 0; i < 8; ++i) state[i] = ns[i];
    }
    c->romb_w[e] = state[7];
  }
  // exp(-(k_i r_j)^2), i-major
  for (int q = tid; q < NKH * NRT; q += nth) {
    const int i = q / NRT, j = q % NRT;
    const double lk = np_linspace(kLogKMin, kLogKMax, NKH - 1, i);
    const double lr = np_linspace(kLogKMin, kLogRMax, NRT - 1, j);
    const double y = exp(lk) * exp(lr);
    const double e = exp(-(y * y));
    c->E[q] = e;
    const float hi = (float)e;
    c->Eff[q] = make_float2(hi, (float)(e - (double)hi));
  }
}

// float-pair copies of the grids (after const_init_kernel), and the tables
// of the pair exp (2^(j/64)) and sin (sin, cos of j pi/64)
__device__ __forceinline__ float2 f2_of(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

__global__ void const_ff_kernel(ConstTables* c) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  for (int j = tid; j < 64; j += nth) c->exp2_ff[j] = f2_of(kExp2Tab64[j]);
  for (int j = tid; j < 128; j += nth) {
    const double a = (double)j * (PI / 64.0);
    c->sincos_ff[2 * j] = f2_of(sin(a));
    c->sincos_ff[2 * j + 1] = f2_of(cos(a));
  }
  for (int e = tid; e < NROMB; e += nth) {
    c->romb_w_ff[e] = f2_of(c->romb_w[e]);
    c->romb_k_ff[e] = f2_of(c->romb_k[e]);
    c->romb_logk_ff[e] = f2_of(c->romb_logk[e]);
    c->romb_ik_ff[e] = f2_of(c->romb_ik[e]);
    c->romb_kw2_ff[e] = f2_of(c->romb_kw2[e]);
  }
  for (int i = tid; i < NKH; i += nth) {
    c->kh_ff[i] = f2_of(c->kh[i]);
    c->logk_ff[i] = f2_of(c->logk[i]);
    c->ikh_ff[i] = f2_of(c->ikh[i]);
    c->kh3_ff[i] = f2_of(c->kh3[i]);
    c->simpson_ff[i] = f2_of(c->simpson_kh[i]);
  }
  for (int i = tid; i < NCHI; i += nth) {
    c->chi_a_ff[i] = f2_of(c->chi_a[i]);
    c->lna_chi_ff[i] = f2_of(c->lna_chi[i]);
    c->chi_ia_ff[i] = f2_of(c->chi_ia[i]);
    c->chi_am_ff[i] = f2_of(c->chi_am[i]);
    c->chi_lnam_ff[i] = f2_of(c->chi_lnam[i]);
    c->chi_iam_ff[i] = f2_of(c->chi_iam[i]);
    c->chi_ida[i] = i < NCHI - 1 ? 1.0 / (c->atab_chi[i + 1] - c->atab_chi[i]) : 0.0;
    c->chi_ida_ff[i] = f2_of(c->chi_ida[i]);
    c->atab_chi_ff[i] = f2_of(c->atab_chi[i]);
    c->chi_h6_ff[i] = f2_of(i > 0 ? (c->lna_chi[i] - c->lna_chi[i - 1]) * (1.0 / 6.0) : 0.0);
  }
  for (int j = tid; j < NRT; j += nth) c->logr_ff[j] = f2_of(c->logr[j]);
  for (int i = tid; i < NGROW; i += nth) {
    c->grow_a_ff[i] = f2_of(c->atab_grow[i]);
    c->grow_lna_ff[i] = f2_of(c->grow_lna[i]);
    c->grow_ia_ff[i] = f2_of(c->grow_ia[i]);
    c->grow_am_ff[i] = f2_of(c->grow_am[i]);
    c->grow_lnam_ff[i] = f2_of(c->grow_lnam[i]);
    c->grow_iam_ff[i] = f2_of(c->grow_iam[i]);
    c->grow_ida[i] = i < NGROW - 1 ? 1.0 / (c->atab_grow[i + 1] - c->atab_grow[i]) : 0.0;
    c->grow_ida_ff[i] = f2_of(c->grow_ida[i]);
  }
}

void launch_const_init(ConstTables* c, cudaStream_t st) {
  const_init_kernel<<<128, 256, 0, st>>>(c);
  const_ff_kernel<<<4, 256, 0, st>>>(c);
}

// ------------------------------------------------------------- geometry -----
__device__ __forceinline__ double smail_pz(const GeoHeader& h, int t, double z) {
  // redshift.py:75-77: z**a * exp(-((z / z0) ** b))
  return npow(z, h.nz_a[t]) * exp(-npow(z / h.nz_z0[t], h.nz_b[t]));
}

// Un-normalised pz_fn of tracer t at z, the `idx`-th point of its n(z) point
// list: Smail analytically, a tabulated tracer from the caller's values.
__device__ __forceinline__ double tracer_pz(const GeoHeader& h, const double* pz, int t, int64_t idx, double z) {
  if (h.nz_kind[t] == JCG_NZ_TABLE) return pz[h.nzp_off[t] + idx];
  if (h.nz_kind[t] == JCG_NZ_DELTA) return z == h.nz_z0[t] ? 1.0 : 0.0;  // redshift.py:121-122
  return smail_pz(h, t, z);
}

// n(z) normalisation (redshift.py:27-31): simps(pz_fn, 0, zmax, 256); also
// stores the header at the start of the geometry buffer.
__global__ void geo_norm_kernel(GeoHeader h, double* geo, const double* pz) {
  GeoHeader* dh = reinterpret_cast<GeoHeader*>(geo);
  const int t = threadIdx.x;
  if (t == 0) *dh = h;
  __syncthreads();
  if (t < h.n_tr) {
    const double zm = h.nz_zmax[t];
    const double dx = (zm - 0.0) / 256;
    double acc = 0.0;
    for (int m = 0; m < 128; ++m) {
      const double y0 = tracer_pz(h, pz, t, 2 * m, np_linspace(0.0, zm, 256, 2 * m));
      const double y1 = tracer_pz(h, pz, t, 2 * m + 1, np_linspace(0.0, zm, 256, 2 * m + 1));
      const double y2 = tracer_pz(h, pz, t, 2 * m + 2, np_linspace(0.0, zm, 256, 2 * m + 2));
      acc += y0 + 4 * y1 + y2;
    }
    dh->nz_norm[t] = h.nz_kind[t] == JCG_NZ_DELTA ? 1.0 : dx / 3 * acc;  // delta_nz: _norm = 1
  }
}

// The points of every tracer's n(z) point list (the same expressions as the
// geometry build below, so that tabulated values sit at the exact points).
__global__ void nz_points_kernel(GeoHeader h, const double* __restrict__ zn, double* out) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  const int na = h.na, N = h.n_limber;
  const double a0 = 1.0 / (1.0 + h.zmax);
  for (int64_t q = tid; q < h.nzp_total; q += nth) {
    int t = 0;
    while (t + 1 < h.n_tr && h.nzp_off[t + 1] <= q) ++t;
    const int64_t idx = q - h.nzp_off[t];
    double z;
    if (idx < NZP) {
      z = np_linspace(0.0, h.nz_zmax[t], 256, (int)idx);
    } else if (idx < NZP + na) {
      const int n = (int)(idx - NZP);
      z = zn ? zn[n] : 1.0 / np_linspace(a0, 1.0, N, n) - 1.0;
    } else {
      const int64_t r = idx - NZP - na;
      const int n = (int)(r / NZP), j = (int)(r % NZP);
      const double zl = zn ? zn[n] : 1.0 / np_linspace(a0, 1.0, N, n) - 1.0;
      z = np_linspace(zl, h.group_zmax[h.group[t]], NZP - 1, j);
    }
    out[q] = z;
  }
}

void launch_nz_points(const GeoHeader& h, const double* z_nodes, double* out, cudaStream_t st) {
  nz_points_kernel<<<296, 256, 0, st>>>(h, z_nodes, out);
}

__global__ void geo_tables_kernel(const GeoHeader* __restrict__ hp, double* geo, const double* __restrict__ pz,
                                  const ConstTables* __restrict__ c) {
  const GeoHeader& h = *hp;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  const int na = h.na, N = h.n_limber;
  const double a0 = 1.0 / (1.0 + h.zmax);  // z2a(zmax)
  double* A = geo + h.off_a;
  double* Z = geo + h.off_z;
  double* WS = geo + h.off_wsimp;
  double* AWL = geo + h.off_awl;
  int64_t* SC = reinterpret_cast<int64_t*>(geo + h.off_seg_chi);
  int64_t* SG = reinterpret_cast<int64_t*>(geo + h.off_seg_grow);
  int64_t* SW = reinterpret_cast<int64_t*>(geo + h.off_seg_chiwl);
  double* NZL = geo + h.off_nzl;
  // Limber nodes: linspace(z2a(zmax), 1, N + 1)  (angular_cl.py:96), or the
  // caller's redshift nodes (already in Z) for probe kernels at arbitrary z.
  for (int n = tid; n < na; n += nth) {
    double a, z, w;
    if (h.custom_nodes) {
      z = Z[n];
      a = 1.0 / (1.0 + z);
      w = 0.0;
    } else {
      a = np_linspace(a0, 1.0, N, n);
      z = 1.0 / a - 1.0;  // a2z (utils.py:7)
      w = (n == 0 || n == N) ? 1.0 : ((n & 1) ? 4.0 : 2.0);
    }
    A[n] = a;
    Z[n] = z;
    WS[n] = h.dx_limber / 3 * w;
    const double awl = 1.0 / (1.0 + z);  // z2a(a2z(a)) in probes.py:27
    AWL[n] = awl;
    SC[n] = pack_seg(interp_segment_inc(a, c->atab_chi, NCHI, logspace_guess(a, NCHI)));
    SG[n] = pack_seg(interp_segment_inc(a, c->atab_grow, NGROW, logspace_guess(a, NGROW)));
    const int2 swl = interp_segment_inc(awl, c->atab_chi, NCHI, logspace_guess(awl, NCHI));
    SW[n] = pack_seg(swl);
    reinterpret_cast<int32_t*>(geo + h.off_qwl32)[n] = swl.x | (min(swl.x, swl.y) << 16);
    reinterpret_cast<float*>(geo + h.off_dxwl32)[n] = (float)(awl - c->atab_chi[swl.x]);
    for (int t = 0; t < h.n_tr; ++t) NZL[(size_t)t * na + n] = tracer_pz(h, pz, t, NZP + n, z) / h.nz_norm[t];
  }
  // ell grid factors (probes.py:73; NumberCounts: 1)
  const double* ell = geo + h.off_ell;
  double* EF = geo + h.off_ellfac;
  double* LG = geo + h.off_lg2ellh;
  for (int q = tid; q < h.n_tr * h.n_ell; q += nth) {
    const int t = q / h.n_ell, l = q % h.n_ell;
    const double e = ell[l];
    double f = 1.0;
    if (h.kind[t] == JCG_TRACER_WL) {
      f = sqrt((e - 1) * (e) * (e + 1) * (e + 2)) / ((e + 0.5) * (e + 0.5));
    }
    EF[q] = f;
    reinterpret_cast<float*>(geo + h.off_ef32)[q] = (float)f;
    if (t == 0) {
      LG[l] = log2(e + 0.5);
      reinterpret_cast<float4*>(geo + h.off_kh4)[l] =
          make_float4((float)(e + 0.5), (float)log2(e + 0.5), (float)(1.0 / (e + 0.5)), 0.f);
    }
  }
  // lensing grids: z' = linspace(z, zmax_probe, 257) per Limber node (probes.py:51)
  for (int g = 0; g < h.n_groups; ++g) {
    const double zp_max = h.group_zmax[g];
    double* AP = geo + h.off_ap[g];
    int64_t* SP = reinterpret_cast<int64_t*>(geo + h.off_segp[g]);
    for (int q = tid; q < na * NZP; q += nth) {
      const int n = q / NZP, j = q % NZP;
      const double z = h.custom_nodes ? Z[n] : 1.0 / np_linspace(a0, 1.0, N, n) - 1.0;
      const double zp = np_linspace(z, zp_max, NZP - 1, j);
      const double ap = 1.0 / (1.0 + zp);
      AP[q] = ap;
      const int2 sg = interp_segment_inc(ap, c->atab_chi, NCHI, logspace_guess(ap, NCHI));
      SP[q] = pack_seg(sg);
      // FP32 lensing kernel: nearest node | segment << 16, and a' - a[nearest]
      reinterpret_cast<int32_t*>(geo + h.off_q32[g])[q] = sg.x | (min(sg.x, sg.y) << 16);
      reinterpret_cast<float*>(geo + h.off_dx32[g])[q] = (float)(ap - c->atab_chi[sg.x]);
      const double dx = (zp_max - z) / 256;
      const double w = (j == 0 || j == NZP - 1) ? 1.0 : ((j & 1) ? 4.0 : 2.0);
      for (int t = 0; t < h.n_tr; ++t) {
        if (h.kind[t] != JCG_TRACER_WL || h.group[t] != g) continue;
        double* W = geo + h.off_W[t];
        // single-plane tracers take no part in the z' integral (probes.py:53-64)
        const double wv = h.nz_kind[t] == JCG_NZ_DELTA
                              ? 0.0
                              : dx / 3 * w * (tracer_pz(h, pz, t, NZP + na + (int64_t)q, zp) / h.nz_norm[t]);
        W[q] = wv;
        reinterpret_cast<float*>(geo + h.off_W32[t])[q] = (float)wv;
      }
    }
  }
}

void launch_geometry_build(const GeoHeader& h, double* geo, const double* pz, const ConstTables* c,
                           cudaStream_t st) {
  geo_norm_kernel<<<1, 32, 0, st>>>(h, geo, pz);
  geo_tables_kernel<<<148, 256, 0, st>>>(reinterpret_cast<const GeoHeader*>(geo), geo, pz, c);
}

// ------------------------------------------------------ cosmology tables ----

// NW: some item may use the transfer type "eisenhu" (a separate
// instantiation keeps the default one's registers).  FAST (fp32c): the
// per-node evaluations (chi and growth right-hand sides, the Romberg
// integrand, P(k) k^3) in float-pair arithmetic on the FP32 pipe; the scans,
// sigma8's weighted sum and the tables' values stay float64.  Most phases
// keep one or two warps of a block busy, so the fp32c form is held to 64
// registers: four blocks per SM overlap their phases.
template <bool NW, bool FAST>
__global__ void __launch_bounds__(256, FAST ? 4 : 3) cosmo_tables_kernel(Batch bt, const ConstTables* __restrict__ c) {
  const int item = blockIdx.x;
  if (item >= bt.n_items) return;
  const Item it = batch_item(bt, item);
  __shared__ double s[NSCAL];
  __shared__ double inc[NCHI];
  __shared__ double fnode[NCHI];
  __shared__ double pq[NKH];
  __shared__ double qa[NGROW], ra[NGROW], qm[NGROW], rm[NGROW];
  __shared__ double fr[NROMB];
  __shared__ double pk3[NKH];
  __shared__ double chis[NCHI];
  __shared__ double gs[NGROW];
  __shared__ double mv[4 * NGROW];  // per-step growth matrices
  __shared__ double yv[2 * NGROW];  // growth ODE solution (D, dD/da) unnormalised
  __shared__ float2 wpp[NKH];       // fp32c: w pk3 as float pairs
  __shared__ FF sff[FAST ? NSCAL : 1];                  // fp32c: the scalars as pairs
  __shared__ float2 e2s[FAST ? 64 : 1], scs[FAST ? 256 : 1];  // tables of the pair exp and sin
  FF* pk3ff = reinterpret_cast<FF*>(pq);                // fp32c: P(k) k^3 as pairs (pq is free until then)
  const int t = threadIdx.x;
  for (int i = t; i < NSCAL; i += blockDim.x) {
    s[i] = it.ctab->s[i];  // from cosmo_scalars_kernel
    if (FAST) sff[i] = ff_of(s[i]);
  }
  if (FAST) {
    for (int i = t; i < 64; i += blockDim.x) e2s[i] = c->exp2_ff[i];
    for (int i = t; i < 256; i += blockDim.x) scs[i] = c->sincos_ff[i];
  }
  __syncthreads();
  const Bg bg = make_bg(s);
  const auto F2 = [](float2 v) { return FF{v.x, v.y}; };
  BgF bgf;
  if (FAST) bgf = BgF{sff[S_OMEGA_M], sff[S_OMEGA_K], sff[S_OMEGA_DE], sff[S_W0], sff[S_WA]};
  // chi RK4 in ln a (background.py:227-231, scipy/ode.py:11-19): the
  // right-hand side does not depend on chi, so each step needs f at its two
  // ends (shared with the neighbouring steps) and at its midpoint.
  if (FAST) {
    if (t < NCHI) {
      fnode[t] = ffd(ff_dchi_dlna(bgf, F2(c->chi_a_ff[t]), F2(c->lna_chi_ff[t]), F2(c->chi_ia_ff[t]), e2s));
      if (t > 0) inc[t] = ffd(ff_dchi_dlna(bgf, F2(c->chi_am_ff[t]), F2(c->chi_lnam_ff[t]), F2(c->chi_iam_ff[t]), e2s));
    }
    if (t < NGROW) {
      FF q, r;
      ff_growth_qr(bgf, F2(c->grow_a_ff[t]), F2(c->grow_lna_ff[t]), F2(c->grow_ia_ff[t]), e2s, q, r);
      qa[t] = ffd(q), ra[t] = ffd(r);
      if (t > 0) {
        ff_growth_qr(bgf, F2(c->grow_am_ff[t]), F2(c->grow_lnam_ff[t]), F2(c->grow_iam_ff[t]), e2s, q, r);
        qm[t] = ffd(q), rm[t] = ffd(r);
      }
    }
    if (t < NROMB) {
      const FF logk = F2(c->romb_logk_ff[t]);
      const FF T = ff_eh_transfer<NW>(sff, F2(c->romb_k_ff[t]), logk, F2(c->romb_ik_ff[t]), s[S_TFNW] != 0.0, e2s, scs);
      fr[t] = ffd(F2(c->romb_kw2_ff[t]) * (ff_sqr(T) * ff_exp(sff[S_NS] * logk, e2s)));
    }
  } else {
    if (t < NCHI) {
      fnode[t] = dchi_dlna_c(bg, c->chi_a[t], c->lna_chi[t], c->chi_ia[t]);
      if (t > 0) inc[t] = dchi_dlna_c(bg, c->chi_am[t], c->chi_lnam[t], c->chi_iam[t]);
    }
    // growth ODE coefficients at nodes and midpoints
    if (t < NGROW) {
      growth_qr_c(bg, c->atab_grow[t], c->grow_lna[t], c->grow_ia[t], qa[t], ra[t]);
      if (t > 0) growth_qr_c(bg, c->grow_am[t], c->grow_lnam[t], c->grow_iam[t], qm[t], rm[t]);
    }
    // sigmasqr(8) integrand at the romb nodes (power.py:70-75): the window
    // factor k (k W(8k))^2 is a constant of the node
    if (t < NROMB) {
      const double logk = c->romb_logk[t];
      const double T = eh_transfer_lki<NW>(s, c->romb_k[t], logk, c->romb_ik[t]);
      fr[t] = c->romb_kw2[t] * ((T * T) * exp(s[S_NS] * logk));
    }
  }
  __syncthreads();
  // growth: one RK4 step is linear in y = (D, dD/da), y_i = M_i y_{i-1};
  // threads 128 + i form M_i (the step on the unit vectors), warp 1 scans
  if (t >= 128 && t < 128 + NGROW) {
    const int i = t - 128;
    double* M = mv + 4 * i;
    if (i == 0) {
      M[0] = 1.0, M[1] = 0.0, M[2] = 0.0, M[3] = 1.0;
    } else {
      const double hh = c->atab_grow[i] - c->atab_grow[i - 1];
      double o0, o1;
      growth_rk4_step(1.0, 0.0, qa[i - 1], ra[i - 1], qm[i], rm[i], qa[i], ra[i], hh, o0, o1);
      M[0] = o0, M[2] = o1;
      growth_rk4_step(0.0, 1.0, qa[i - 1], ra[i - 1], qm[i], rm[i], qa[i], ra[i], hh, o0, o1);
      M[1] = o0, M[3] = o1;
    }
  }
  const int warp = t >> 5, lane = t & 31;
  if (warp == 0) {
    chi_scan_warp(fnode, inc, c->lna_chi, lane, chis);
  } else if (warp == 2) {
    // sigmasqr(8) (power.py:70-78): romb is linear in the integrand values,
    // sum_e w_e f_e with the weights of its Richardson combination
    double acc = 0.0;
    for (int e = lane; e < NROMB; e += 32) acc = fma(c->romb_w[e], fr[e], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const double sig8 = 1.0 / (2.0 * (PI * PI)) * acc;
      s[S_SIGMASQR8] = sig8;
      s[S_PKNORM] = (s[S_SIGMA8] * s[S_SIGMA8]) / sig8;
    }
  }
  __syncthreads();
  if (warp == 1) {
    double d4[4];
    const double yf = growth_scan_warp(mv, c->atab_grow[0], 1.0, lane, d4, yv);
    for (int k = 0; k < 4; ++k) {
      const int i = lane * 4 + k;
      const double g = d4[k] / yf;
      gs[i] = g;
      // dlnD/dlna = a / D dD/da (background.py:484-485)
      it.ctab->f[i] = yv[2 * i + 1] / yf * c->atab_grow[i] / g;
    }
  }
  __syncthreads();
  if (t == 0) {
    // growth_factor(1.0) (power.py:44 with the default a = 1)
    const int2 sg = interp_segment_inc(1.0, c->atab_grow, NGROW, NGROW - 1);
    s[S_G1] = clip_lohi(interp_eval(1.0, c->atab_grow, gs, sg), 0.0, 1.0);
  }
  __syncthreads();
  // linear P(k_i, a = 1) * k_i^3 on the halofit k grid (power.py:102, 124)
  if (FAST) {
    const FF g1 = ff_of(s[S_G1]);
    const FF fac = ff_sqr(g1) * ff_of(s[S_PKNORM]);  // sigma8^2 / sigmasqr(8), set above
    for (int i = t; i < NKH; i += blockDim.x) {
      const FF lk = F2(c->logk_ff[i]);
      const FF tk = ff_eh_transfer<NW>(sff, F2(c->kh_ff[i]), lk, F2(c->ikh_ff[i]), s[S_TFNW] != 0.0, e2s, scs);
      const FF p = ff_exp(sff[S_NS] * lk, e2s) * ff_sqr(tk) * fac * F2(c->kh3_ff[i]);
      pk3[i] = ffd(p);
      // sigma^2(R) sums' k-node factor w pk k^3 / (2 pi^2) as a pair
      const FF w = F2(c->simpson_ff[i]) * p * ffc(1.0 / (2.0 * (PI * PI)));
      wpp[i] = make_float2(w.hi, w.lo);
      pk3ff[i] = p;
    }
  } else {
    for (int i = t; i < NKH; i += blockDim.x) {
      const double tk = eh_transfer_lki<NW>(s, c->kh[i], c->logk[i], c->ikh[i]);
      const double g1 = s[S_G1];
      pk3[i] = exp(s[S_NS] * c->logk[i]) * (tk * tk) * (g1 * g1) * s[S_PKNORM] * c->kh3[i];
    }
  }
  __syncthreads();
  // sigma^2(R_j) without g^2: simps over ln k of pk k^3 exp(-(k R)^2) / (2 pi^2),
  // with the Simpson weights and 1 / (2 pi^2) folded into the k-node factor:
  // one FMA per (k, R) term
  if (!FAST) {
    for (int i = t; i < NKH; i += blockDim.x) pq[i] = c->simpson_kh[i] * (pk3[i] / (2.0 * (PI * PI)));
    __syncthreads();
  }
  CosmoTab* out = it.ctab;
  if (FAST) {
    // fp32c: the same sums in float-pair arithmetic (about 1e-13 relative, all
    // terms positive): the FP32 pipe instead of the 1/64-rate FP64 one; the
    // halofit root find on this table then takes the same nodes as with
    // float64 sums except within ~1e-13 of a decision boundary
    for (int j = t; j < NRT; j += blockDim.x) {
      float ah = 0.f, al = 0.f;
      for (int i = 0; i < NKH; ++i) ff_acc_prod(ah, al, wpp[i], c->Eff[i * NRT + j]);
      out->sig[j] = (double)ah + (double)al;
    }
    __syncthreads();
  } else {
    for (int j = t; j < NRT; j += blockDim.x) {
      double acc = 0.0;
      for (int i = 0; i < NKH; ++i) acc = fma(pq[i], c->E[i * NRT + j], acc);
      out->sig[j] = acc;
    }
  }
  for (int i = t; i < NSCAL; i += blockDim.x) out->s[i] = s[i];
  for (int i = t; i < NCHI; i += blockDim.x) {
    // segment [i, i+1] slope of the chi table: the `a` of scipy/interpolate.py:55
    // (fp32c: times the reciprocal of the node spacing)
    const double sl = (i < NCHI - 1)
                          ? (FAST ? (chis[i + 1] - chis[i]) * c->chi_ida[i]
                                  : (chis[i + 1] - chis[i]) / (c->atab_chi[i + 1] - c->atab_chi[i]))
                          : 0.0;
    out->chi_slope[i] = sl;
    out->chi32[i] = (float)chis[i];
    out->slope32[i] = (float)sl;
  }
  if (FAST) {
    // fp32c halofit moments: w pk3 as float pairs (float copy for the exp
    // terms), then the Taylor tables by the contracting recurrence
    // Q_m[i + 1] = (Q_m[i] + w_i pk3_i) rho_m in float pairs, one lane per m
    for (int i = t; i < NKH + 15; i += blockDim.x) {
      float hi = 0.f;
      if (i < NKH) {
        const FF w = F2(c->simpson_ff[i]) * pk3ff[i];
        hi = w.hi;
        wpp[i] = make_float2(w.hi, w.lo);
      }
      out->wpk3f[i] = hi;
    }
    __syncthreads();
    if (t < NTAYLOR) {
      const int m = t;
      FF rho, cm, q;
      rho.hi = c->tay_rho[m][0], rho.lo = c->tay_rho[m][1];
      cm.hi = c->tay_c[m][0], cm.lo = c->tay_c[m][1];
      q.hi = 0.f, q.lo = 0.f;
      float2* dst = out->rtay[m];
      dst[0] = make_float2(0.f, 0.f);
      for (int i = 0; i < NKH; ++i) {
        FF w;
        w.hi = wpp[i].x, w.lo = wpp[i].y;
        q = ff_mul(ff_add(q, w), rho);
        const FF r = ff_mul(cm, q);
        dst[i + 1] = make_float2(r.hi, r.lo);
      }
    }
  }
  for (int i = t; i < NCHI; i += blockDim.x) out->chi[i] = chis[i];
  for (int i = t; i < NGROW; i += blockDim.x) out->g[i] = gs[i];
  for (int i = t; i < NKH; i += blockDim.x) out->pk3[i] = pk3[i];
  // the fp32c Limber kernel's transfer inputs, by a warp that the Taylor
  // recurrences (warp 0) leave idle
  if (t == 32) make_eh32(s, &out->eh32);
}

// The scalars, one half warp per cosmology: the independent pow / sqrt /
// log calls of each level of the chain on different lanes at once
// (cosmo_scalars_warpT), so the chain's latency is 5 calls deep.  Both
// halves of a warp run (the last one on a copy of the last cosmology when
// the count is odd) since the shuffles need every lane.
__global__ void __launch_bounds__(128) cosmo_scalars_kernel(Batch bt) {
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 4, lane = threadIdx.x & 15;
  if (((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2 >= bt.n_items) return;  // whole warps only
  const bool valid = g < bt.n_items;
  const Item it = batch_item(bt, valid ? g : bt.n_items - 1);
  double sv[NSCAL];
  cosmo_scalars_warpT<double>(it.params, sv, lane, tf_nowiggle(it.physics));
  double v0 = 0.0, v1 = 0.0, v2 = 0.0;
#pragma unroll
  for (int k = 0; k < 16; ++k)
    if (k == lane) v0 = sv[k], v1 = sv[k + 16], v2 = k + 32 < NSCAL ? sv[k + 32] : 0.0;
  if (valid) {
    it.ctab->s[lane] = v0;
    it.ctab->s[lane + 16] = v1;
    if (lane + 32 < NSCAL) it.ctab->s[lane + 32] = v2;
  }
}

// Growth for JCG_GROWTH_GAMMA (background.py:515-582): f(a) = Omega_m(a)^gamma
// at the 128 nodes of the growth table and at the RK4 midpoints in ln a,
// exp((ln a_{i-1} + ln a_i) / 2).  The reference's odeint with a right-hand
// side independent of y is y_i = y_{i-1} + h/6 (f_{i-1} + 2 f_m + 2 f_m + f_i),
// y_0 = ln a_0 (scipy/ode.py:6-22); g_i = exp(y_i) / exp(y_last).  Replaces
// the growth-ODE tables cosmo_tables wrote (nothing there depends on them
// but growth(a = 1) = 1, the same for both) and stores the growth rate f at
// the nodes and gamma in the scalars.  One CTA per cosmology.
__global__ void __launch_bounds__(128) growth_gamma_kernel(Batch bt, const ConstTables* __restrict__ c) {
  const int item = blockIdx.x;
  if (item >= bt.n_items) return;
  const Item it = batch_item(bt, item);
  if (!growth_gamma(it.physics)) return;
  __shared__ double fn[NGROW], fm[NGROW], ys[NGROW];
  CosmoTab* ct = it.ctab;
  const double gam = it.params[8];
  const Bg bg = make_bg(ct->s);
  const int t = threadIdx.x;
  for (int i = t; i < NGROW; i += blockDim.x) {
    const double lna = c->grow_lna[i];
    fn[i] = pow(bg_omm(bg, exp(lna)), gam);
    if (i > 0) {
      const double lp = c->grow_lna[i - 1];
      fm[i] = pow(bg_omm(bg, exp(lp + (lna - lp) / 2)), gam);
    }
  }
  __syncthreads();
  if (t == 0) {
    double y = c->grow_lna[0];
    ys[0] = y;
    for (int i = 1; i < NGROW; ++i) {
      const double h = c->grow_lna[i] - c->grow_lna[i - 1];
      y = y + 1.0 / 6.0 * h * (((fn[i - 1] + 2.0 * fm[i]) + 2.0 * fm[i]) + fn[i]);
      ys[i] = y;
    }
  }
  __syncthreads();
  const double el = exp(ys[NGROW - 1]);
  for (int i = t; i < NGROW; i += blockDim.x) {
    ct->g[i] = exp(ys[i]) / el;
    ct->f[i] = fn[i];
  }
  if (t == 0) ct->s[S_GAMMA] = gam;
}

void launch_cosmo_tables(const Batch& b, const ConstTables* c, cudaStream_t st) {
  cosmo_scalars_kernel<<<(b.n_items + 7) / 8, 128, 0, st>>>(b);
  if (tf_nowiggle(b.physics_or))
    b.precision == JCG_FP32C ? cosmo_tables_kernel<true, true><<<b.n_items, 256, 0, st>>>(b, c)
                             : cosmo_tables_kernel<true, false><<<b.n_items, 256, 0, st>>>(b, c);
  else
    b.precision == JCG_FP32C ? cosmo_tables_kernel<false, true><<<b.n_items, 256, 0, st>>>(b, c)
                             : cosmo_tables_kernel<false, false><<<b.n_items, 256, 0, st>>>(b, c);
  if (growth_gamma(b.physics_or)) growth_gamma_kernel<<<b.n_items, 128, 0, st>>>(b, c);
}

}  // namespace jcg
