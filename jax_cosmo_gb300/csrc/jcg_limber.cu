// Fused Limber integral (angular_cl.py:49-98).
//
//   C_ij(l) = ef_i(l) ef_j(l) * sum_a  P_nl(k = (l + 1/2) / max(chi_a, 1), a) * M_ij(a)
//   M_ij(a) = w_a * dchi/da / max(chi_a^2, 1) / c^2 * K_i(a) K_j(a)
//
// w_a are the Simpson weights of simps(integrand, z2a(zmax), 1, N)
// (scipy/integrate.py:195-198), K_i the ell-independent radial kernels and
// ef_i the WeakLensing ell factor (probes.py:73; 1 for NumberCounts).
//
// One CTA per (ell tile, cosmology).  The a axis is walked in chunks of TA
// nodes: the chunk's per-a rows and M_ij are staged in shared memory, every
// thread evaluates Eisenstein-Hu x primordial x halofit at (ell, a) nodes into
// a P tile, then the CTA contracts the P tile with M into per-thread
// accumulators.  FP64: the reference's formula order.  FP32C: MUFU forms of the
// same formulas (ex2/lg2/rcp/sin), per-chunk partial sums added with Kahan
// compensation across chunks.
#include "jcg_internal.cuh"
#include "jcg_fp32.cuh"

namespace jcg {

constexpr int LB_THREADS = 256;
constexpr int LB_TA = 32;   // a nodes per chunk
constexpr int LB_MAXLT = 32;
constexpr int LB_MAXO = (LB_MAXLT * MAXPAIR + LB_THREADS - 1) / LB_THREADS;  // 17

// Per-cosmology Eisenstein & Hu constants of the FP32 node.
// Eisenstein-Hu T(k) in FP32 (transfer.py:88-153, either type) at k, lk =
// log2 k, invk = 1 / k.
template <bool GEN>
__device__ __forceinline__ float eh32_T(const EH32& e, float k, float lk, float invk) {
  float T;
  if (GEN && e.nw) {
    // type "eisenhu" (transfer.py:88-105)
    const float x = 0.43f * k * e.sh, x2 = x * x;
    const float q = k * e.nwq * rcpf(e.agam + (1.f - e.agam) * rcpf(1.f + x2 * x2));
    const float L = LN2_F * lg2f(2.f * E_F + 1.8f * q);
    T = L * rcpf(L + (14.2f + 731.f * rcpf(1.f + 62.5f * q)) * (q * q));
  } else {
    // cold dark matter transfer (EH98 10-12, 17-18)
    const float q = k * e.qinv;
    const float lq = lk + e.lg2_qinv;
    const float q108 = ex2f(1.08f * lq);
    const float Cb = 386.f * rcpf(1.f + 69.9f * q108);
    const float L1 = LN2_F * lg2f(E_F + e.c18bc * q);
    const float L2 = LN2_F * lg2f(E_F + 1.8f * q);
    const float qq = q * q;
    const float Ta = L1 * rcpf(L1 + (14.2f + Cb) * qq);
    const float Tb = L1 * rcpf(L1 + (e.c142ac + Cb) * qq);
    const float Tn = L2 * rcpf(L2 + (14.2f + Cb) * qq);
    const float ks = k * e.sh;
    const float x54 = ks * (1.f / 5.4f);
    const float x54_2 = x54 * x54;
    const float f = rcpf(1.f + x54_2 * x54_2);
    const float Tc = f * Ta + (1.f - f) * Tb;
    // baryon transfer (EH98 14, 19, 21-24)
    const float iks = invk * e.inv_sh;
    const float x52 = ks * (1.f / 5.2f);
    const float bb = e.beta_b * iks;
    const float silk = ex2f(-LOG2E_F * ex2f(1.4f * (lk - e.lg2_ksilk)));
    const float bn = e.beta_node * iks;
    const float st = e.sh * ex2f((-1.f / 3.f) * lg2f(1.f + bn * bn * bn));
    const float arg = k * st;
    const float sinc = sin_reduced(arg) * rcpf(arg);
    const float Tbar = (Tn * rcpf(1.f + x52 * x52) + e.alpha_b * rcpf(1.f + bb * bb * bb) * silk) * sinc;
    T = e.fb * Tbar + e.fc * Tc;
  }
  return T;
}

// primordial x transfer x halofit (power.py:42-53, 246-260) at one node in
// FP32 from tk = T(k)^2 k^(n_s + 3): k = kh / max(chi, 1), lk = log2 k,
// invk = 1 / k.
// lin: the linear power (nonlinear_fn = linear_matter_power).  GEN = false:
// the default operator points only (takahashi2012; lin and mu_n are not
// read), so that instantiation keeps its registers.
template <bool GEN>
__device__ __forceinline__ float pk32_T(const EH32& e, const float* r, float k, float lk, float invk, float tk,
                                        bool lin) {
  // linear and halofit power
  const float d2l = tk * r[F_D2FAC];
  if (GEN && lin) return TWO_PI2_F * (invk * invk * invk) * d2l;
  const float y = k * r[F_INVKNL];
  const float ly = lk - r[F_LG2KNL];
  const float fy = y * (0.25f + 0.125f * y);
  const float d2q = d2l * ex2f(r[F_BETAN] * lg2f(1.f + d2l)) * rcpf(1.f + r[F_ALPHAN] * d2l) *
                    ex2f(-LOG2E_F * fy);
  const float yf1 = ex2f(r[F_3F1] * ly);
  const float yf2 = ex2f(r[F_F2] * ly);
  const float ycg = ex2f(r[F_3MGAMMA] * (r[F_LG2CF3] + ly));
  const float y2 = y * y;
  // d2h' / (1 + mu / y + nu / y^2) as d2h' y^2 / (y^2 + mu y + nu)
  const float d2h =
      r[F_AN] * yf1 * rcpf(1.f + r[F_BN] * yf2 + ycg) * y2 * rcpf((GEN ? fmaf(r[F_MUN], y, y2) : y2) + r[F_NUN]);
  return TWO_PI2_F * (invk * invk * invk) * (d2q + d2h);
}

// Both at one node: kh = l + 1/2, lg2kh = log2(kh), invkh = 1 / kh.
template <bool GEN>
__device__ __forceinline__ float node32(const EH32& e, const float* r, float kh, float lg2kh,
                                        float invkh, bool lin) {
  const float k = kh * r[F_INVCHI];
  const float lk = lg2kh + r[F_LG2INVCHI];
  const float invk = invkh * r[F_CHIC];
  const float T = eh32_T<GEN>(e, k, lk, invk);
  return pk32_T<GEN>(e, r, k, lk, invk, ex2f(e.ns3 * lk) * (T * T), lin);
}

// T(k)^2 k^(n_s + 3) table of the fp32c Limber kernel: NTT nodes uniform in
// log2 k over the range of one CTA's nodes, values by 4-point Lagrange
// interpolation (error O(h^4): about 1e-7 relative for the baryon wiggles at
// this spacing, below the FP32 evaluation's own error)
constexpr int NTT = 2048;
__device__ __forceinline__ float tt_interp(const float* tab, float lk, float lk0, float ih) {
  const float u = (lk - lk0) * ih;
  int i = __float2int_rd(u);
  i = max(1, min(i, NTT - 3));
  const float t = u - (float)i;
  const float tm1 = t - 1.f, tm2 = t - 2.f, tp1 = t + 1.f;
  const float a = tm1 * tm2, b = tp1 * t;
  return (-1.f / 6.f) * (t * a) * tab[i - 1] + 0.5f * (tp1 * a) * tab[i] - 0.5f * (b * tm2) * tab[i + 1] +
         (1.f / 6.f) * (b * tm1) * tab[i + 2];
}


// ---------------------------------------------------------------- kernel ---
// MAXO: accumulators per thread, >= ceil(LT * n_cls / LB_THREADS).
template <bool FP32, int MAXO>
__global__ void __launch_bounds__(LB_THREADS)
    limber_kernel(Batch bt, const ConstTables* __restrict__ c, int LT) {
  using T = typename std::conditional<FP32, float, double>::type;
  constexpr int RW = FP32 ? NROW32 : NROW64;
  const int item = blockIdx.y;
  if (item >= bt.n_items) return;
  const Item it = batch_item(bt, item);
  const GeoHeader* geo = it.geo;
  const int n_ell = geo->n_ell, n_cls = geo->n_cls, na = geo->na;
  const int model = pk_model(it.physics);
  const bool lin = model == JCG_PK_LINEAR;
  const int l0 = blockIdx.x * LT;
  if (l0 >= n_ell) return;
  const int lt = min(LT, n_ell - l0);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* s = reinterpret_cast<double*>(smem_raw);    // NSCAL
  EH32* e32 = reinterpret_cast<EH32*>(s + NSCAL);     // 1 (padded to 8 doubles)
  double* ellv = s + NSCAL + 8;                        // LB_MAXLT: l + 1/2 (FP64 path)
  double* lellv = ellv + LB_MAXLT;                     // LB_MAXLT: log(l + 1/2)
  float* kh32 = reinterpret_cast<float*>(lellv + LB_MAXLT);  // 3 * LB_MAXLT floats
  T* rowsS = reinterpret_cast<T*>(kh32 + 3 * LB_MAXLT);      // TA * RW
  T* Ms = rowsS + LB_TA * RW;                                // TA * n_cls
  T* Pt = Ms + LB_TA * n_cls;                                // TA * LT
  const int tid = threadIdx.x;
  const double* ELL = geo_ptr<double>(geo, geo->off_ell);
  const double* EF = geo_ptr<double>(geo, geo->off_ellfac);
  for (int i = tid; i < NSCAL; i += LB_THREADS) s[i] = it.ctab->s[i];
  for (int l = tid; l < lt; l += LB_THREADS) {
    const double e = ELL[l0 + l] + 0.5;
    ellv[l] = e;
    lellv[l] = log(e);
    kh32[3 * l + 0] = (float)e;                               // k = kh / max(chi, 1)
    kh32[3 * l + 1] = (float)(1.4426950408889634 * log(e));   // log2(kh)
    kh32[3 * l + 2] = (float)(1.0 / e);                       // 1 / kh
  }
  __syncthreads();
  if (FP32 && tid == 0) make_eh32(s, e32);
  __syncthreads();
  const double* rows64 = it.rows64;
  const float* rows32 = it.rows32;
  const double* kern = it.kern;
  const int nout = lt * n_cls;
  T acc[MAXO], comp[MAXO];
#pragma unroll
  for (int r = 0; r < MAXO; ++r) {
    acc[r] = 0;
    comp[r] = 0;
  }
  for (int base = 0; base < na; base += LB_TA) {
    const int tc = min(LB_TA, na - base);
    // stage rows
    if (FP32) {
      for (int i = tid; i < tc * RW; i += LB_THREADS)
        rowsS[i] = (T)rows32[(size_t)base * NROW32 + i];
    } else {
      for (int i = tid; i < tc * RW; i += LB_THREADS)
        rowsS[i] = (T)rows64[(size_t)base * NROW64 + i];
    }
    // M_ij(a) = u_a K_i(a) K_j(a)
    for (int q = tid; q < tc * n_cls; q += LB_THREADS) {
      const int t = q / n_cls, p = q - (q / n_cls) * n_cls;
      const int n = base + t;
      const double ki = kern[(size_t)geo->pair_i[p] * na + n];
      const double kj = kern[(size_t)geo->pair_j[p] * na + n];
      const double u = rows64[(size_t)n * NROW64 + R_U];
      if (FP32)
        Ms[t * n_cls + p] = (T)((float)ki * (float)kj * (float)u);
      else
        Ms[t * n_cls + p] = (T)((ki * kj) * u);
    }
    __syncthreads();
    // P tile: nodes (t, l)
    for (int q = tid; q < tc * lt; q += LB_THREADS) {
      const int t = q / lt, l = q - (q / lt) * lt;
      T pv;
      if (FP32) {
        pv = (T)node32<true>(*e32, reinterpret_cast<const float*>(rowsS) + t * NROW32, kh32[3 * l],
                       kh32[3 * l + 1], kh32[3 * l + 2], lin);
      } else {
        const double* row = reinterpret_cast<const double*>(rowsS) + t * NROW64;
        const double k = ellv[l] / fmax(row[R_CHI], 1.0);
        pv = (T)halofit_node_lk(s, row, k, lellv[l] - row[R_LGCHIC], model);
      }
      Pt[t * LT + l] = pv;
    }
    __syncthreads();
    // contraction
#pragma unroll
    for (int r = 0; r < MAXO; ++r) {
      const int o = tid + r * LB_THREADS;
      if (o < nout) {
        const int l = o % lt, p = o / lt;
        T part = 0;
        for (int t = 0; t < tc; ++t) part += Pt[t * LT + l] * Ms[t * n_cls + p];
        if (FP32) {
          const T y = part - comp[r];
          const T tt = acc[r] + y;
          comp[r] = (tt - acc[r]) - y;
          acc[r] = tt;
        } else {
          acc[r] += part;
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < MAXO; ++r) {
    const int o = tid + r * LB_THREADS;
    if (o < nout) {
      const int l = o % lt, p = o / lt;
      const int ell = l0 + l;
      const double efi = EF[(size_t)geo->pair_i[p] * n_ell + ell];
      const double efj = EF[(size_t)geo->pair_j[p] * n_ell + ell];
      const double v = FP32 ? ((double)acc[r] - (double)comp[r]) : (double)acc[r];
      it.cl[(size_t)p * n_ell + ell] = v * efi * efj;
    }
  }
}

// ------------------------------------------------------- fp32c kernel ----
// The fp32c Limber integral with a register-blocked contraction: a work unit
// is (ell, 4 consecutive spectra, residue of the a node mod nsplit); per a
// node it loads P(ell, a) once and M_ij(a) of its 4 spectra as one float4
// (a broadcast within the warp), and keeps 4 Kahan-compensated accumulators.
// Small outputs (lt x ceil(n_cls / 4) < LB_THREADS) split the a nodes over
// nsplit units, added in float64 at the end.  The kernels K_i(a) and the
// weights u_a of a chunk are staged once as floats, then M_ij(a) =
// (K_i K_j) u in the order of the generic kernel.
constexpr int L32_MAXU = 5;  // ceil(LB_MAXLT * ceil(MAXPAIR / 4) / LB_THREADS)

struct L32Layout {
  size_t e32, kh32, rows, ks, us, ms, pt, red, tab, total;
};
__host__ __device__ inline L32Layout l32_layout(int n_tr, int n_cls, int LT) {
  L32Layout L;
  size_t o = NSCAL * 8;
  L.e32 = o;
  o += 8 * 8;
  L.kh32 = o;
  o += 4 * LB_MAXLT * 4;
  L.rows = o;
  o += (size_t)LB_TA * NROW32 * 4;
  L.ks = o;
  o += (size_t)n_tr * LB_TA * 4;
  L.us = o;
  o += LB_TA * 4;
  o = (o + 15) & ~(size_t)15;
  L.ms = o;
  o += (size_t)LB_TA * ((n_cls + 3) & ~3) * 4;
  L.pt = o;
  o += (size_t)LB_TA * LT * 4;
  o = (o + 15) & ~(size_t)15;
  L.red = o;
  o += (size_t)LB_THREADS * 4 * 8;
  L.tab = o;
  o += (size_t)(NTT + 16) * 4;
  L.total = o;
  return L;
}

// GEN: the non-default operator points (transfer type "eisenhu", smith2003,
// linear_matter_power) are read from each item.
template <int MAXU, bool GEN>
__global__ void __launch_bounds__(LB_THREADS, MAXU <= 1 ? 5 : (MAXU <= 3 ? 3 : 2))
    limber32_kernel(Batch bt, const ConstTables* __restrict__ c, int LT) {
  const int item = blockIdx.y;
  if (item >= bt.n_items) return;
  const Item it = batch_item(bt, item);
  const GeoHeader* geo = it.geo;
  const int n_ell = geo->n_ell, n_cls = geo->n_cls, na = geo->na, n_tr = geo->n_tr;
  const bool lin = pk_model(it.physics) == JCG_PK_LINEAR;
  const int l0 = blockIdx.x * LT;
  if (l0 >= n_ell) return;
  const int lt = min(LT, n_ell - l0);
  const int npg = (n_cls + 3) >> 2, ncp = npg * 4;
  const int items = lt * npg;
  const int nsplit = items >= LB_THREADS ? 1 : min(8, LB_THREADS / items);
  const int units = items * nsplit;
  const L32Layout L = l32_layout(n_tr, n_cls, LT);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EH32* e32 = reinterpret_cast<EH32*>(smem_raw + L.e32);
  float4* kh4 = reinterpret_cast<float4*>(smem_raw + L.kh32);
  float* rowsS = reinterpret_cast<float*>(smem_raw + L.rows);
  float* Ks = reinterpret_cast<float*>(smem_raw + L.ks);
  float* us = reinterpret_cast<float*>(smem_raw + L.us);
  float* Ms = reinterpret_cast<float*>(smem_raw + L.ms);
  const float4* Ms4 = reinterpret_cast<const float4*>(Ms);
  float* Pt = reinterpret_cast<float*>(smem_raw + L.pt);
  double* red = reinterpret_cast<double*>(smem_raw + L.red);
  const int tid = threadIdx.x;
  const double* EF = geo_ptr<double>(geo, geo->off_ellfac);
  // k = kh / max(chi, 1): kh = l + 1/2, log2(kh), 1 / kh from the geometry;
  // the transfer inputs from the table stage
  const float4* KH4 = geo_ptr<float4>(geo, geo->off_kh4);
  for (int l = tid; l < lt; l += LB_THREADS) kh4[l] = KH4[l0 + l];
  for (int i = tid; i < (int)(sizeof(EH32) / 4); i += LB_THREADS)
    reinterpret_cast<int*>(e32)[i] = reinterpret_cast<const int*>(&it.ctab->eh32)[i];
  __syncthreads();
  // T^2 k^(n_s+3) table over this CTA's log2 k range: lg2(l + 1/2) of its ell plus the
  // range of log2(1 / max(chi, 1)) over the item's nodes
  float* Ttab = reinterpret_cast<float*>(smem_raw + L.tab);
  float* wmm = Ttab + NTT;  // [8] warp minima, [8] warp maxima
  {
    float mn = 3.0e38f, mx = -3.0e38f;
    for (int n = tid; n < na; n += LB_THREADS) {
      const float v = it.rows32[(size_t)n * NROW32 + F_LG2INVCHI];
      mn = fminf(mn, v);
      mx = fmaxf(mx, v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((tid & 31) == 0) wmm[tid >> 5] = mn, wmm[8 + (tid >> 5)] = mx;
  }
  __syncthreads();
  float tlk0, tih;
  {
    float mn = wmm[0], mx = wmm[8];
#pragma unroll
    for (int w = 1; w < LB_THREADS / 32; ++w) mn = fminf(mn, wmm[w]), mx = fmaxf(mx, wmm[8 + w]);
    const float lo = kh4[0].y + mn - 0.01f, hi = kh4[lt - 1].y + mx + 0.01f;
    const float h = (hi - lo) * (1.f / (float)(NTT - 3));
    tlk0 = lo - h;  // node 0; nodes 1 .. NTT - 2 span [lo, hi]
    tih = 1.f / h;
    for (int j = tid; j < NTT; j += LB_THREADS) {
      const float lkj = tlk0 + (float)j * h;
      const float T = eh32_T<GEN>(*e32, ex2f(lkj), lkj, ex2f(-lkj));
      Ttab[j] = ex2f(e32->ns3 * lkj) * (T * T);
    }
  }
  // (t, l) and (t, p) from flat indices without integer division: q < 32 * 136,
  // so (q + 1/2) / n in float is off by far less than 1 / (2 n) of an integer
  const float inv_lt = 1.f / (float)lt, inv_ncp = 1.f / (float)ncp;
  const float* rows32 = it.rows32;
  const double* rows64 = it.rows64;
  const double* kern = it.kern;
  const float* kern32 = it.kern32;
  const float* u32 = it.u32;
  float acc[MAXU][4], comp[MAXU][4];
#pragma unroll
  for (int r = 0; r < MAXU; ++r)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[r][j] = 0.f, comp[r][j] = 0.f;
  for (int base = 0; base < na; base += LB_TA) {
    const int tc = min(LB_TA, na - base);
    for (int i = tid; i < tc * NROW32; i += LB_THREADS) rowsS[i] = rows32[(size_t)base * NROW32 + i];
    for (int q = tid; q < n_tr * tc; q += LB_THREADS) {
      const int tr = q / tc, t = q - tr * tc;
      Ks[tr * LB_TA + t] = kern32 ? kern32[(size_t)tr * na + base + t] : (float)kern[(size_t)tr * na + base + t];
    }
    for (int t = tid; t < tc; t += LB_THREADS)
      us[t] = u32 ? u32[base + t] : (float)rows64[(size_t)(base + t) * NROW64 + R_U];
    __syncthreads();
    // M_ij(a) = (K_i K_j) u_a, zero-padded to ncp spectra
    for (int q = tid; q < tc * ncp; q += LB_THREADS) {
      const int t = __float2int_rz(((float)q + 0.5f) * inv_ncp), p = q - t * ncp;
      float m = 0.f;
      if (p < n_cls) m = Ks[geo->pair_i[p] * LB_TA + t] * Ks[geo->pair_j[p] * LB_TA + t] * us[t];
      Ms[q] = m;
    }
    // P tile: nodes (t, l)
    for (int q = tid; q < tc * lt; q += LB_THREADS) {
      const int t = __float2int_rz(((float)q + 0.5f) * inv_lt), l = q - t * lt;
      const float4 kk = kh4[l];
      const float* r = rowsS + t * NROW32;
      const float k = kk.x * r[F_INVCHI];
      const float lk = kk.y + r[F_LG2INVCHI];
      const float invk = kk.z * r[F_CHIC];
      Pt[t * LT + l] = pk32_T<GEN>(*e32, r, k, lk, invk, tt_interp(Ttab, lk, tlk0, tih), lin);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < MAXU; ++r) {
      const int u = tid + r * LB_THREADS;
      if (u < units) {
        const int itm = u % items, sp = u / items;
        const int l = itm % lt, pg = itm / lt;
        float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;
        for (int t = sp; t < tc; t += nsplit) {
          const float pv = Pt[t * LT + l];
          const float4 m = Ms4[t * npg + pg];
          p0 = fmaf(pv, m.x, p0);
          p1 = fmaf(pv, m.y, p1);
          p2 = fmaf(pv, m.z, p2);
          p3 = fmaf(pv, m.w, p3);
        }
        const float part[4] = {p0, p1, p2, p3};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float y = part[j] - comp[r][j];
          const float tt = acc[r][j] + y;
          comp[r][j] = (tt - acc[r][j]) - y;
          acc[r][j] = tt;
        }
      }
    }
    __syncthreads();
  }
  // a nodes split over nsplit units: partial sums added in float64
  if (nsplit > 1) {
    if (tid < units) {
#pragma unroll
      for (int j = 0; j < 4; ++j) red[tid * 4 + j] = (double)acc[0][j] - (double)comp[0][j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < MAXU; ++r) {
    const int u = tid + r * LB_THREADS;
    if (u < items) {
      const int l = u % lt, pg = u / lt;
      const int ell = l0 + l;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int p = pg * 4 + j;
        if (p >= n_cls) break;
        double v;
        if (nsplit > 1) {
          v = 0.0;
          for (int sp = 0; sp < nsplit; ++sp) v += red[(u + sp * items) * 4 + j];
        } else {
          v = (double)acc[r][j] - (double)comp[r][j];
        }
        const double efi = EF[(size_t)geo->pair_i[p] * n_ell + ell];
        const double efj = EF[(size_t)geo->pair_j[p] * n_ell + ell];
        it.cl[(size_t)p * n_ell + ell] = v * efi * efj;
      }
    }
  }
}

template <int MAXU, bool GEN = false>
static void launch_limber32_t(const Batch& b, const ConstTables* c, int lt, cudaStream_t st) {
  const L32Layout L = l32_layout(b.max_tr, b.max_cls, lt);
  cudaFuncSetAttribute(limber32_kernel<MAXU, GEN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total);
  dim3 grid((b.max_ell + lt - 1) / lt, b.n_items);
  limber32_kernel<MAXU, GEN><<<grid, LB_THREADS, L.total, st>>>(b, c, lt);
}

size_t limber_smem_bytes(bool fp32, int n_cls, int LT) {
  const size_t el = fp32 ? 4 : 8;
  const size_t rw = fp32 ? NROW32 : NROW64;
  return (NSCAL + 8 + 2 * LB_MAXLT) * 8 + 3 * LB_MAXLT * 4 +
         el * (LB_TA * rw + (size_t)LB_TA * n_cls + (size_t)LB_TA * LT);
}

template <bool FP32, int MAXO>
static void launch_limber_t(const Batch& b, const ConstTables* c, int lt, size_t smem, dim3 grid,
                            cudaStream_t st) {
  cudaFuncSetAttribute(limber_kernel<FP32, MAXO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  limber_kernel<FP32, MAXO><<<grid, LB_THREADS, smem, st>>>(b, c, lt);
}

template <bool FP32>
static void launch_limber_p(const Batch& b, const ConstTables* c, int lt, size_t smem, dim3 grid,
                            cudaStream_t st) {
  const int need = (lt * b.max_cls + LB_THREADS - 1) / LB_THREADS;
  if (need <= 1) launch_limber_t<FP32, 1>(b, c, lt, smem, grid, st);
  else if (need <= 2) launch_limber_t<FP32, 2>(b, c, lt, smem, grid, st);
  else if (need <= 4) launch_limber_t<FP32, 4>(b, c, lt, smem, grid, st);
  else if (need <= 8) launch_limber_t<FP32, 8>(b, c, lt, smem, grid, st);
  else launch_limber_t<FP32, LB_MAXO>(b, c, lt, smem, grid, st);
}

void launch_limber(const Batch& b, const ConstTables* c, int lt, cudaStream_t st) {
  if (b.precision == JCG_FP32C) {
    // units per thread: the split path needs one, otherwise lt x ceil(n_cls / 4)
    const int items = lt * ((b.max_cls + 3) / 4);
    const int need = items >= LB_THREADS ? (items + LB_THREADS - 1) / LB_THREADS : 1;
    if (b.physics_or != 0) {
      if (need <= 1) launch_limber32_t<1, true>(b, c, lt, st);
      else if (need <= 2) launch_limber32_t<2, true>(b, c, lt, st);
      else if (need <= 3) launch_limber32_t<3, true>(b, c, lt, st);
      else launch_limber32_t<L32_MAXU, true>(b, c, lt, st);
    } else if (need <= 1) {
      launch_limber32_t<1>(b, c, lt, st);
    } else if (need <= 2) {
      launch_limber32_t<2>(b, c, lt, st);
    } else if (need <= 3) {
      launch_limber32_t<3>(b, c, lt, st);
    } else {
      launch_limber32_t<L32_MAXU>(b, c, lt, st);
    }
    return;
  }
  const size_t smem = limber_smem_bytes(false, b.max_cls, lt);
  dim3 grid((b.max_ell + lt - 1) / lt, b.n_items);
  launch_limber_p<false>(b, c, lt, smem, grid, st);
}

}  // namespace jcg
