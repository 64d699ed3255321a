// FP32 compensated ("fp32c") stages of the Jacobian dC_ell/dtheta: the radial
// kernels with tangents and the Limber integrand with its reverse sweep.
//
// The tables, halofit rows and their tangents come from the FP64 stages
// (jcg_grad.cu) -- background ODEs, sigma8, the root find and the spectral
// moments stay in float64 -- and are handed over as FP32 rows (GTan layout,
// jcg_grad.cuh).  Here, per Limber node (cosmology, ell, a):
//
//   P(k, a)           Eisenstein-Hu x primordial x takahashi2012 in FP32 with
//                     MUFU ex2/lg2/rcp/sin/cos (the forward fp32c integrand);
//   dP/d(inputs)      hand-written reverse sweep of the same operations;
//   dP/dtheta         the adjoints contracted with the inputs' tangents;
//   C, dC/dtheta      sum_a [P M, dP M + P dM] in FP32 per chunk of a nodes,
//                     chunks added with Kahan compensation, then FP64.
#include "jcg_fp32.cuh"
#include "jcg_grad.cuh"
#include "jcg_node32.cuh"

namespace jcg {

// ---------------------------------------------------------- radial kernels --
// One warp per node, lanes over the 257 lensing z' points, the WeakLensing
// tracers of one lensing group per pass; `npc` nodes per CTA (fewer for small
// batches, so that the grid still covers the GPU).  Lensing efficiency (probes.py:44-51) with tangents:
//   r_j = max(chi'_j - chi, 0) / max(chi'_j, 1)
//   dr_j = ic_j (dchi'_j (1 - r_j [chi'_j > 1]) - dchi)  where chi'_j > chi
// accumulated as sum W r, sum W ic, sum W ic (1 - r) dchi'.
constexpr int GK_NODES = 128;  // nodes per CTA at most (8 warps x 16)

// REV (vector-Jacobian form): the shear integral's tangents are not formed
// (written as 0; grad_kernrev32_kernel applies their cotangents in reverse),
// the NumberCounts, NLA and single-plane terms keep theirs.  UW: the shear
// values come from grad_kernval32u_kernel (uniform batch), this kernel adds
// the other terms only.
template <int TP, bool REV, bool UW = false>
__global__ void __launch_bounds__(256, 2) grad_kern32_kernel(GradBatch gb, const ConstTables* __restrict__ c, int npc) {
  const int item = blockIdx.y;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const GeoHeader* geo = gi.geo;
  const int na = geo->na, n_tr = geo->n_tr;
  const int n0 = blockIdx.x * npc;
  if (n0 >= na) return;
  // passes: WeakLensing tracers of one lensing group, up to TP per pass
  __shared__ int ptr_t[JCG_MAX_TRACERS * TP];
  __shared__ int pgroup[JCG_MAX_TRACERS];
  __shared__ int npass_s;
  if (threadIdx.x == 0) {
    int np = 0;
    for (int g = 0; g < geo->n_groups; ++g) {
      int u = TP;
      for (int t = 0; t < n_tr; ++t) {
        if (geo->kind[t] != JCG_TRACER_WL || geo->group[t] != g) continue;
        if (u == TP) {
          pgroup[np] = g;
          for (int v = 0; v < TP; ++v) ptr_t[np * TP + v] = -1;
          ++np;
          u = 0;
        }
        ptr_t[(np - 1) * TP + u++] = t;
      }
    }
    npass_s = np;
  }
  __shared__ __align__(16) float ctab[NDIR + 1][NCHI];  // chi, then its tangents
  __shared__ __align__(16) float stab[NDIR + 1][NCHI];  // segment slopes, then tangents
  const TabD* tb = gi.tab;
  {
    const float4* sc = reinterpret_cast<const float4*>(&tb->c32[0][0]);
    const float4* ss = reinterpret_cast<const float4*>(&tb->s32[0][0]);
    float4* dc = reinterpret_cast<float4*>(&ctab[0][0]);
    float4* ds = reinterpret_cast<float4*>(&stab[0][0]);
    for (int i = threadIdx.x; i < (NDIR + 1) * NCHI / 4; i += blockDim.x) {
      dc[i] = sc[i];
      ds[i] = ss[i];
    }
  }
  __syncthreads();
  const int npass = UW ? 0 : npass_s;
  const float* chi = ctab[0];
  const float* slope = stab[0];
  const float(*dchi)[NCHI] = ctab + 1;
  const float(*dslope)[NCHI] = stab + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double* Z = geo_ptr<double>(geo, geo->off_z);
  const double* AWL = geo_ptr<double>(geo, geo->off_awl);
  const int32_t* QWL = geo_ptr<int32_t>(geo, geo->off_qwl32);
  const float* DXWL = geo_ptr<float>(geo, geo->off_dxwl32);
  const double* NZL = geo_ptr<double>(geo, geo->off_nzl);
  const int dir = lane & 7;
  const double om = tb->sv[S_OMEGA_M];
  const float cff = (float)(3.0 * (H0 * H0) * om / 2.0 / C_KMS);  // probes.py:71
  const float dlcf = (float)(tb->sd[dir][S_OMEGA_M] / om);         // d ln(cf)
  const int n_end = min(na, n0 + npc);
  for (int n = n0 + warp; n < n_end; n += 8) {
    const int qw = QWL[n];
    const int xw = qw & 0xffff, mw = qw >> 16;
    const float craw_w = chi[xw] + slope[mw] * DXWL[n];
    const float chi_wl = fmaxf(craw_w, 0.f);
    float dchi_wl[NDIR];
#pragma unroll
    for (int d = 0; d < NDIR; ++d) dchi_wl[d] = craw_w > 0.f ? dchi[d][xw] + dslope[d][mw] * DXWL[n] : 0.f;
    (void)dchi_wl;
    const float zp1 = (float)(1.0 + Z[n]);
    const size_t row = (size_t)n * NZP;
    // WeakLensing tracers: passes of up to TP tracers of one lensing group
    for (int pass = 0; pass < npass; ++pass) {
      const int g = pgroup[pass];
      int tl[TP];
      const float* W[TP];
#pragma unroll
      for (int u = 0; u < TP; ++u) {
        tl[u] = ptr_t[pass * TP + u];
        W[u] = tl[u] >= 0 ? geo_ptr<float>(geo, geo->off_W32[tl[u]]) + row : nullptr;
      }
      float av[TP], at[TP], ad[TP][NDIR];
#pragma unroll
      for (int u = 0; u < TP; ++u) {
        av[u] = 0.f;
        at[u] = 0.f;
#pragma unroll
        for (int d = 0; d < NDIR; ++d) ad[u][d] = 0.f;
      }
      const int32_t* Q32 = geo_ptr<int32_t>(geo, geo->off_q32[g]) + row;
      const float* DX32 = geo_ptr<float>(geo, geo->off_dx32[g]) + row;
      for (int j = lane; j < NZP; j += 32) {
        const int q = Q32[j];
        const int x = q & 0xffff, m = q >> 16;
        const float dx = DX32[j];
        const float craw = chi[x] + slope[m] * dx;
        const float chip = fmaxf(craw, 0.f);
        const float diff = chip - chi_wl;
        if (!(diff > 0.f)) continue;  // then craw > 0 too
        const float ic = rcpf(fmaxf(chip, 1.f));
        const float r = diff * ic;
        if (REV) {
#pragma unroll
          for (int u = 0; u < TP; ++u)
            if (tl[u] >= 0) av[u] = fmaf(W[u][j], r, av[u]);
          continue;
        }
        const float h = chip > 1.f ? ic * (1.f - r) : ic;
        float dcp[NDIR];
#pragma unroll
        for (int d = 0; d < NDIR; ++d) dcp[d] = fmaf(dslope[d][m], dx, dchi[d][x]) * h;
#pragma unroll
        for (int u = 0; u < TP; ++u) {
          if (tl[u] >= 0) {
            const float w = W[u][j];
            av[u] = fmaf(w, r, av[u]);
            at[u] = fmaf(w, ic, at[u]);
#pragma unroll
            for (int d = 0; d < NDIR; ++d) ad[u][d] = fmaf(w, dcp[d], ad[u][d]);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < TP; ++u) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          av[u] += __shfl_xor_sync(0xffffffffu, av[u], o);
          if (!REV) {
            at[u] += __shfl_xor_sync(0xffffffffu, at[u], o);
#pragma unroll
            for (int d = 0; d < NDIR; ++d) ad[u][d] += __shfl_xor_sync(0xffffffffu, ad[u][d], o);
          }
        }
      }
      if (lane < NDIR) {
        float dcw = 0.f;
#pragma unroll
        for (int d = 0; d < NDIR; ++d)
          if (d == dir) dcw = dchi_wl[d];
#pragma unroll
        for (int u = 0; u < TP; ++u) {
          const int t = tl[u];
          if (t < 0) continue;
          float adir = 0.f;
#pragma unroll
          for (int d = 0; d < NDIR; ++d)
            if (d == dir) adir = ad[u][d];
          // K = (cf (1 + z) chi acc + NLA) (1 + m), FP32 (the stored precision)
          const float m1 = 1.f + (float)geo->mult[t];
          const float fac = cff * zp1;
          const float acc = av[u];
          const float kv = fac * chi_wl * acc;
          const float kd = REV ? 0.f : fac * (dlcf * chi_wl * acc + dcw * acc + chi_wl * (adir - dcw * at[u]));
          float* dst = gi.kernf + ((size_t)t * na + n) * (NDIR + 1);
          if (dir == 0) dst[0] = kv * m1;
          dst[1 + dir] = kd * m1;
        }
      }
    }
    // NumberCounts tracers, and the NLA term of WeakLensing tracers with IA
    // (added to the shear part written above, times 1 + m): four tracers at a
    // time, lanes 8u .. 8u + 7 on tracer u
    __syncwarp();
    {
      for (int t = lane >> 3; t < n_tr; t += 4) {
        const bool wl = geo->kind[t] == JCG_TRACER_WL;
        const bool delta = wl && geo->nz_kind[t] == JCG_NZ_DELTA;
        if (wl && !delta && geo->bias_kind[t] == JCG_BIAS_NONE) continue;
        if (delta) {
          // single plane (probes.py:53-64): K = cf (1 + z) chi r (1 + m),
          // r = clip(chi(z0) - chi, 0) / clip(chi(z0), 1), replacing the
          // (zero) z' integral written above
          float dcw = 0.f;
#pragma unroll
          for (int d = 0; d < NDIR; ++d)
            if (d == dir) dcw = dchi_wl[d];
          const double a0 = 1.0 / (1.0 + geo->nz_z0[t]);
          const int2 sg0 = interp_segment_inc(a0, c->atab_chi, NCHI, logspace_guess(a0, NCHI));
          // chi(z0) from the float-pair chi table and its float tangents
          const double ida = 1.0 / (c->atab_chi[sg0.y] - c->atab_chi[sg0.x]);
          const D1 f0 = mk1((double)tb->chiF[sg0.x].x + (double)tb->chiF[sg0.x].y, (double)tb->chidF[sg0.x][dir]);
          const D1 f1 = mk1((double)tb->chiF[sg0.y].x + (double)tb->chiF[sg0.y].y, (double)tb->chidF[sg0.y][dir]);
          const D1 chi0 = xfmax(f0 + (f1 - f0) * (ida * (a0 - c->atab_chi[sg0.x])), 0.0);
          const D1 r = xfmax(chi0 - mk1((double)chi_wl, (double)dcw), 0.0) / xfmax(chi0, 1.0);
          const float rv = (float)r.v, rd = (float)r.d[0];
          const float fac = cff * zp1, m1 = 1.f + (float)geo->mult[t];
          float* dst = gi.kernf + ((size_t)t * na + n) * (NDIR + 1);
          if (dir == 0) dst[0] = fac * chi_wl * rv * m1;
          dst[1 + dir] = fac * (dlcf * chi_wl * rv + dcw * rv + chi_wl * rd) * m1;
          if (geo->bias_kind[t] == JCG_BIAS_NONE) continue;
        }
        double kv, kd;
        bias_term_d1(tb, c, geo, t, dir, AWL[n], Z[n], NZL[(size_t)t * na + n], wl, &kv, &kd);
        float* dst = gi.kernf + ((size_t)t * na + n) * (NDIR + 1);
        if (wl) {
          const float m1 = 1.f + (float)geo->mult[t];
          if (dir == 0) dst[0] += (float)kv * m1;
          // UW: the shear tangents are zero and not stored by the value kernel
          if (UW) dst[1 + dir] = (float)kd * m1;
          else dst[1 + dir] += (float)kd * m1;
        } else {
          if (dir == 0) dst[0] = (float)kv;
          dst[1 + dir] = (float)kd;
        }
      }
    }
  }
}

void launch_grad_kern32(const GradBatch& gb, const ConstTables* c, cudaStream_t st) {
  // halve the nodes per CTA (down to one per warp) until the grid has two
  // CTAs per SM
  const long target = 2L * device_sm_count();
  int npc = GK_NODES;
  while (npc > 8 && (long)((gb.na + npc - 1) / npc) * gb.n_items < target) npc /= 2;
  dim3 grid((gb.na + npc - 1) / npc, gb.n_items);
  if (gb.krev_u) {
    // uniform batch: the shear values in the lanes-over-cosmologies layout,
    // then the NumberCounts / NLA terms (if any) per cosmology
    launch_kernval32u(gb, st);
    if (!gb.kern_rest) return;
    if (gb.n_tr <= 3) grad_kern32_kernel<3, true, true><<<grid, 256, 0, st>>>(gb, c, npc);
    else if (gb.n_tr <= 5) grad_kern32_kernel<5, true, true><<<grid, 256, 0, st>>>(gb, c, npc);
    else grad_kern32_kernel<8, true, true><<<grid, 256, 0, st>>>(gb, c, npc);
  } else if (gb.vjp_rev) {
    if (gb.n_tr <= 3) grad_kern32_kernel<3, true><<<grid, 256, 0, st>>>(gb, c, npc);
    else if (gb.n_tr <= 5) grad_kern32_kernel<5, true><<<grid, 256, 0, st>>>(gb, c, npc);
    else grad_kern32_kernel<8, true><<<grid, 256, 0, st>>>(gb, c, npc);
  } else if (gb.n_tr <= 3) {
    grad_kern32_kernel<3, false><<<grid, 256, 0, st>>>(gb, c, npc);
  } else if (gb.n_tr <= 5) {
    grad_kern32_kernel<5, false><<<grid, 256, 0, st>>>(gb, c, npc);
  } else {
    grad_kern32_kernel<8, false><<<grid, 256, 0, st>>>(gb, c, npc);
  }
}

constexpr int L32_THREADS = 256;
constexpr int L32_G = 2;      // pairs per contraction unit
constexpr int L32_MAXLT = 32;

int grad_limber32_chunk(int n_cls) { return n_cls <= 64 ? 32 : 16; }

int grad_limber32_tile(int n_ell, int n_cls) {
  const int groups = (n_cls + L32_G - 1) / L32_G;
  int lt = L32_THREADS / groups;
  if (lt > L32_MAXLT) lt = L32_MAXLT;
  if (lt < 1) lt = 1;
  const int tiles = (n_ell + lt - 1) / lt;
  return (n_ell + tiles - 1) / tiles;
}

static size_t limber32_smem_floats(int n_cls, int n_tr, int LT, int TA) {
  return 128 + 128 + (size_t)TA * NROWG + (size_t)TA * n_tr * (NDIR + 1) + (size_t)TA * n_cls * (NDIR + 1) +
         (size_t)TA * LT * (NDIR + 1);
}

// One CTA per (ell tile, a split, cosmology).
//   phase K: the chunk's FP32 rows and kernels into shared memory;
//   phase M: M_p(a) = u K_i K_j and its tangents;
//   phase A: per (a, ell) P and dP/dtheta (reverse sweep + projection);
//   phase B: per (ell, pair group) the 9 sums over the chunk, Kahan-added.
// GEN: some item may use a non-default operator point (transfer type
// "eisenhu", smith2003, linear_matter_power); a separate instantiation keeps
// the default one's registers.
template <bool GEN>
__global__ void __launch_bounds__(L32_THREADS, 2)
    grad_limber32_kernel(GradBatch gb, const ConstTables* __restrict__ c, int LT, int TA) {
  const int item = blockIdx.z, split = blockIdx.y;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const GeoHeader* geo = gi.geo;
  const int n_ell = geo->n_ell, n_cls = geo->n_cls, na = geo->na, n_tr = geo->n_tr;
  const bool lin = pk_model(geo->physics) == JCG_PK_LINEAR;
  const bool nw = GEN && tf_nowiggle(geo->physics);
  const int l0 = blockIdx.x * LT;
  if (l0 >= n_ell) return;
  const int lt = min(LT, n_ell - l0);
  const int per = (na + gb.n_split - 1) / gb.n_split;
  const int a_begin = split * per, a_end = min(na, a_begin + per);
  extern __shared__ __align__(16) float sm32[];
  float* ev = sm32;                                   // EHg values (14)
  float* et = ev + 16;                                // [NET][NDIR] tangents
  float* khv = sm32 + 128;                            // [32] l + 1/2
  float* lkhv = khv + 32;                             // [32] log2(l + 1/2)
  float* ikhv = lkhv + 32;                            // [32] 1 / (l + 1/2)
  float* R = sm32 + 256;                              // [TA][NROWG]
  float* Ks = R + (size_t)TA * NROWG;                 // [TA][n_tr][NDIR + 1]
  float* Mv = Ks + (size_t)TA * n_tr * (NDIR + 1);    // [TA][n_cls]
  float* Md = Mv + (size_t)TA * n_cls;                // [TA][n_cls][NDIR]
  float* Pv = Md + (size_t)TA * n_cls * NDIR;         // [TA][LT]
  float* Pd = Pv + (size_t)TA * LT;                   // [TA][NDIR][LT]
  const int tid = threadIdx.x;
  const TabD* tb = gi.tab;
  // the Eisenstein-Hu inputs and their tangents (formed once per cosmology
  // by the table stage)
  for (int i = tid; i < 16; i += L32_THREADS) ev[i] = tb->ehv[i];
  for (int i = tid; i < NET * NDIR; i += L32_THREADS) et[i] = tb->eht[i];
  const double* ELL = geo_ptr<double>(geo, geo->off_ell);
  const double* EF = geo_ptr<double>(geo, geo->off_ellfac);
  for (int l = tid; l < lt; l += L32_THREADS) {
    const double e = ELL[l0 + l] + 0.5;
    khv[l] = (float)e;
    lkhv[l] = (float)log2(e);
    ikhv[l] = (float)(1.0 / e);
  }
  __syncthreads();
  EHg eh;
  eh.qinv = ev[0]; eh.lg2_qinv = ev[1]; eh.sh = ev[2]; eh.inv_sh = ev[3]; eh.c18bc = ev[4];
  eh.c142ac = ev[5]; eh.alpha_b = ev[6]; eh.beta_b = ev[7]; eh.beta_node = ev[8]; eh.lg2_ksilk = ev[9];
  eh.fb = ev[10]; eh.fc = ev[11]; eh.ns3 = ev[12]; eh.inv_keq = ev[13];
  eh.agam = ev[14]; eh.nwq = ev[15];
  // contraction unit of this thread: ell l_u, pairs [p0, p1)
  const int groups = (n_cls + L32_G - 1) / L32_G;
  const int l_u = tid % LT, pg = tid / LT;
  const bool unit_on = pg < groups && l_u < lt;
  const int p0 = pg * L32_G, p1 = min(n_cls, p0 + L32_G);
  float acc[L32_G][NDIR + 1], cmp[L32_G][NDIR + 1];
#pragma unroll
  for (int g = 0; g < L32_G; ++g)
#pragma unroll
    for (int s = 0; s <= NDIR; ++s) {
      acc[g][s] = 0.f;
      cmp[g][s] = 0.f;
    }
  for (int base = a_begin; base < a_end; base += TA) {
    const int tc = min(TA, a_end - base);
    // phase K
    {
      const float4* src = reinterpret_cast<const float4*>(gi.rowg + (size_t)base * NROWG);
      float4* dst = reinterpret_cast<float4*>(R);
      for (int i = tid; i < tc * (NROWG / 4); i += L32_THREADS) dst[i] = src[i];
      for (int i = tid; i < tc * n_tr * (NDIR + 1); i += L32_THREADS) {
        const int t = i / (n_tr * (NDIR + 1)), rem = i % (n_tr * (NDIR + 1));
        const int tr = rem / (NDIR + 1), s = rem % (NDIR + 1);
        Ks[i] = gi.kernf[((size_t)tr * na + base + t) * (NDIR + 1) + s];
      }
    }
    __syncthreads();
    // phase M
    for (int i = tid; i < tc * n_cls; i += L32_THREADS) {
      const int t = i / n_cls, p = i % n_cls;
      const float* Ki = Ks + ((size_t)t * n_tr + geo->pair_i[p]) * (NDIR + 1);
      const float* Kj = Ks + ((size_t)t * n_tr + geo->pair_j[p]) * (NDIR + 1);
      const float* row = R + (size_t)t * NROWG;
      const float u = row[F_U];
      const float kk = Ki[0] * Kj[0];
      Mv[i] = u * kk;
      const float* du = row + NROWV + T_U * NDIR;
#pragma unroll
      for (int d = 0; d < NDIR; ++d) Md[(size_t)i * NDIR + d] = du[d] * kk + u * (Ki[1 + d] * Kj[0] + Ki[0] * Kj[1 + d]);
    }
    // phase A
    for (int i = tid; i < tc * lt; i += L32_THREADS) {
      const int t = i / lt, l = i % lt;
      const float* row = R + (size_t)t * NROWG;
      float an[NGT], ae[NET];
      const float P = !GEN ? node32_fb_default(eh, row, khv[l], lkhv[l], ikhv[l], an, ae)
                      : nw ? node32_fb_nw(eh, row, khv[l], lkhv[l], ikhv[l], an, ae, lin)
                           : node32_fb<true>(eh, row, khv[l], lkhv[l], ikhv[l], an, ae, lin);
      float pd[NDIR];
#pragma unroll
      for (int d = 0; d < NDIR; ++d) pd[d] = 0.f;
      const float* tg = row + NROWV;
#pragma unroll
      for (int j = 0; j < T_U; ++j) {
        if (!GEN && j == T_MUN) continue;  // mu_n = 0 for takahashi2012
        const float4 a = *reinterpret_cast<const float4*>(tg + j * NDIR);
        const float4 b = *reinterpret_cast<const float4*>(tg + j * NDIR + 4);
        pd[0] = fmaf(an[j], a.x, pd[0]); pd[1] = fmaf(an[j], a.y, pd[1]);
        pd[2] = fmaf(an[j], a.z, pd[2]); pd[3] = fmaf(an[j], a.w, pd[3]);
        pd[4] = fmaf(an[j], b.x, pd[4]); pd[5] = fmaf(an[j], b.y, pd[5]);
        pd[6] = fmaf(an[j], b.z, pd[6]); pd[7] = fmaf(an[j], b.w, pd[7]);
      }
#pragma unroll
      for (int j = 0; j < NET; ++j) {
        const float4 a = *reinterpret_cast<const float4*>(et + j * NDIR);
        const float4 b = *reinterpret_cast<const float4*>(et + j * NDIR + 4);
        pd[0] = fmaf(ae[j], a.x, pd[0]); pd[1] = fmaf(ae[j], a.y, pd[1]);
        pd[2] = fmaf(ae[j], a.z, pd[2]); pd[3] = fmaf(ae[j], a.w, pd[3]);
        pd[4] = fmaf(ae[j], b.x, pd[4]); pd[5] = fmaf(ae[j], b.y, pd[5]);
        pd[6] = fmaf(ae[j], b.z, pd[6]); pd[7] = fmaf(ae[j], b.w, pd[7]);
      }
      Pv[t * LT + l] = P;
#pragma unroll
      for (int d = 0; d < NDIR; ++d) Pd[((size_t)t * NDIR + d) * LT + l] = pd[d];
    }
    __syncthreads();
    // phase B
    if (unit_on) {
      float part[L32_G][NDIR + 1];
#pragma unroll
      for (int g = 0; g < L32_G; ++g)
#pragma unroll
        for (int s = 0; s <= NDIR; ++s) part[g][s] = 0.f;
      for (int t = 0; t < tc; ++t) {
        const float pv = Pv[t * LT + l_u];
        float pd[NDIR];
#pragma unroll
        for (int d = 0; d < NDIR; ++d) pd[d] = Pd[((size_t)t * NDIR + d) * LT + l_u];
#pragma unroll
        for (int g = 0; g < L32_G; ++g) {
          const int p = p0 + g;
          if (p < p1) {
            const float mv = Mv[t * n_cls + p];
            const float4 a = *reinterpret_cast<const float4*>(Md + ((size_t)t * n_cls + p) * NDIR);
            const float4 b = *reinterpret_cast<const float4*>(Md + ((size_t)t * n_cls + p) * NDIR + 4);
            const float md[NDIR] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
            part[g][0] = fmaf(pv, mv, part[g][0]);
#pragma unroll
            for (int d = 0; d < NDIR; ++d) part[g][1 + d] = fmaf(pd[d], mv, fmaf(pv, md[d], part[g][1 + d]));
          }
        }
      }
#pragma unroll
      for (int g = 0; g < L32_G; ++g)
#pragma unroll
        for (int s = 0; s <= NDIR; ++s) {
          const float y = part[g][s] - cmp[g][s];
          const float tt = acc[g][s] + y;
          cmp[g][s] = (tt - acc[g][s]) - y;
          acc[g][s] = tt;
        }
    }
    __syncthreads();
  }
  if (unit_on) {
    const int ell = l0 + l_u;
    double* part = gi.part + (size_t)split * n_cls * n_ell * (NDIR + 1);
#pragma unroll
    for (int g = 0; g < L32_G; ++g) {
      const int p = p0 + g;
      if (p < p1) {
        const double ef = EF[(size_t)geo->pair_i[p] * n_ell + ell] * EF[(size_t)geo->pair_j[p] * n_ell + ell];
        double* dst = part + ((size_t)p * n_ell + ell) * (NDIR + 1);
#pragma unroll
        for (int s = 0; s <= NDIR; ++s) dst[s] = ((double)acc[g][s] - (double)cmp[g][s]) * ef;
      }
    }
  }
}

void launch_grad_limber32(const GradBatch& gb, const ConstTables* c, cudaStream_t st) {
  const int lt = grad_limber32_tile(gb.n_ell, gb.n_cls);
  const int ta = grad_limber32_chunk(gb.n_cls);
  const size_t smem = sizeof(float) * limber32_smem_floats(gb.n_cls, gb.n_tr, lt, ta);
  dim3 grid((gb.n_ell + lt - 1) / lt, gb.n_split, gb.n_items);
  if (gb.physics_or != 0) {
    cudaFuncSetAttribute(grad_limber32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    grad_limber32_kernel<true><<<grid, L32_THREADS, smem, st>>>(gb, c, lt, ta);
  } else {
    cudaFuncSetAttribute(grad_limber32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    grad_limber32_kernel<false><<<grid, L32_THREADS, smem, st>>>(gb, c, lt, ta);
  }
}

}  // namespace jcg
