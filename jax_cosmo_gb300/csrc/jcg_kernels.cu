// Tracer radial kernels on the Limber nodes.
//
// WeakLensing (probes.py:16-74, 188-208): for each node z,
//   q_i(z) = simps_{z' in [z, zmax], 256}[ n_i(z') clip(chi' - chi, 0) / clip(chi', 1) ]
//            * (1 + z) * chi,  times 3 H0^2 Omega_m / (2 c) and (1 + m).
// The n(z') Simpson weights and the chi-table segment of every z' node are
// cosmology-independent and come precomputed in the geometry buffer; per
// cosmology only the chi table and its segment slopes are needed, so each
// chi(z') is one multiply-add (scipy/interpolate.py:55-59 with the slope of
// the chosen segment precomputed).
// NumberCounts (probes.py:77-99, 260-272): n_i(z) * b * H(z2a(z)).
// The ell factor of WeakLensing (probes.py:73) is applied in the Limber stage.
//
// FP64 (plain): float64 throughout.  FP32 (fp32c): the lensing integrand in
// float32 (chi' from the float table, reciprocal by MUFU), the result scaled
// in float64.
#include "jcg_internal.cuh"

namespace jcg {

constexpr int TK_WARPS = 8;
constexpr int TK_NODES_PER_BLOCK = 32;

__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <bool FP32>
__global__ void __launch_bounds__(TK_WARPS * 32)
    tracer_kernels_kernel(Batch bt, const ConstTables* __restrict__ c) {
  using T = typename std::conditional<FP32, float, double>::type;
  const int item = blockIdx.y;
  if (item >= bt.n_items) return;
  const Item it = batch_item(bt, item);
  const GeoHeader* geo = it.geo;
  const int na = geo->na;
  const int n0 = blockIdx.x * TK_NODES_PER_BLOCK;
  if (n0 >= na) return;
  __shared__ T chi[NCHI];
  __shared__ T slope[NCHI];
  __shared__ double atab[NCHI];
  __shared__ double s[NSCAL];
  const CosmoTab* ct = it.ctab;
  for (int i = threadIdx.x; i < NCHI; i += blockDim.x) {
    if (FP32) {
      chi[i] = (T)ct->chi32[i];
      slope[i] = (T)ct->slope32[i];
    } else {
      chi[i] = (T)ct->chi[i];
      slope[i] = (T)ct->chi_slope[i];
    }
    atab[i] = c->atab_chi[i];
  }
  for (int i = threadIdx.x; i < NSCAL; i += blockDim.x) s[i] = ct->s[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_tr = geo->n_tr;
  const double* Z = geo_ptr<double>(geo, geo->off_z);
  const double* AWL = geo_ptr<double>(geo, geo->off_awl);
  const int64_t* SW = geo_ptr<int64_t>(geo, geo->off_seg_chiwl);
  const int32_t* QWL = geo_ptr<int32_t>(geo, geo->off_qwl32);
  const float* DXWL = geo_ptr<float>(geo, geo->off_dxwl32);
  const double* NZL = geo_ptr<double>(geo, geo->off_nzl);
  // 3 H0^2 Omega_m / 2 / c  (probes.py:71)
  const double cf = 3.0 * (H0 * H0) * s[S_OMEGA_M] / 2.0 / C_KMS;
  const int n_end = min(na, n0 + TK_NODES_PER_BLOCK);
  for (int n = n0 + warp; n < n_end; n += TK_WARPS) {
    const double awl = AWL[n];
    T chi_wl;
    if (FP32) {
      const int q = QWL[n];
      chi_wl = fmaxf((float)chi[q & 0xffff] + (float)slope[q >> 16] * DXWL[n], 0.f);
    } else {
      const int2 sg = unpack_seg(SW[n]);
      chi_wl = fmax((double)chi[sg.x] + (double)slope[min(sg.x, sg.y)] * (awl - atab[sg.x]), 0.0);
    }
    T acc[MAXTR];
#pragma unroll
    for (int t = 0; t < MAXTR; ++t) acc[t] = 0;
    for (int g = 0; g < geo->n_groups; ++g) {
      const size_t row = (size_t)n * NZP;
      const double* AP = geo_ptr<double>(geo, geo->off_ap[g]) + row;
      const int64_t* SP = geo_ptr<int64_t>(geo, geo->off_segp[g]) + row;
      const int32_t* Q32 = geo_ptr<int32_t>(geo, geo->off_q32[g]) + row;
      const float* DX32 = geo_ptr<float>(geo, geo->off_dx32[g]) + row;
      for (int j = lane; j < NZP; j += 32) {
        T ratio;
        if (FP32) {
          const int q = Q32[j];
          const float chip = fmaxf((float)chi[q & 0xffff] + (float)slope[q >> 16] * DX32[j], 0.f);
          ratio = fmaxf(chip - (float)chi_wl, 0.f) * rcp_approx(fmaxf(chip, 1.f));
        } else {
          const int2 sg = unpack_seg(SP[j]);
          const double chip =
              fmax((double)chi[sg.x] + (double)slope[min(sg.x, sg.y)] * (AP[j] - atab[sg.x]), 0.0);
          ratio = fmax(chip - (double)chi_wl, 0.0) / fmax(chip, 1.0);
        }
#pragma unroll
        for (int t = 0; t < MAXTR; ++t) {
          if (t < n_tr && geo->kind[t] == JCG_TRACER_WL && geo->group[t] == g) {
            if (FP32) {
              const float* W = geo_ptr<float>(geo, geo->off_W32[t]) + row;
              acc[t] += (T)W[j] * ratio;
            } else {
              const double* W = geo_ptr<double>(geo, geo->off_W[t]) + row;
              acc[t] += (T)W[j] * ratio;
            }
          }
        }
      }
    }
#pragma unroll
    for (int t = 0; t < MAXTR; ++t) {
      if (t < n_tr && geo->kind[t] == JCG_TRACER_WL) {
        T v = acc[t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        acc[t] = v;
      }
    }
    const double z = Z[n];
    double hz = 0.0, dz = 1.0;
    if (geo->n_nc > 0 || geo->special_bias) hz = bg_H(make_bg(s), awl);
    if (geo->special_bias) dz = growth_at(ct->g, c, awl);
    // lanes write one tracer each (acc indices stay compile-time)
#pragma unroll
    for (int t = 0; t < MAXTR; ++t) {
      if (t < n_tr && lane == (t & 31)) {
        double kv;
        if (geo->kind[t] == JCG_TRACER_WL) {
          double acc_t = (double)acc[t];
          if (geo->nz_kind[t] == JCG_NZ_DELTA) {
            // single plane (probes.py:53-64): clip(chi(z0) - chi, 0) / clip(chi(z0), 1)
            const double a0 = 1.0 / (1.0 + geo->nz_z0[t]);
            const int2 sg = interp_segment_inc(a0, c->atab_chi, NCHI, logspace_guess(a0, NCHI));
            const double chi0 = fmax(interp_eval(a0, c->atab_chi, ct->chi, sg), 0.0);
            acc_t = fmax(chi0 - (double)chi_wl, 0.0) / fmax(chi0, 1.0);
          }
          const double rk = acc_t * (1.0 + z) * (double)chi_wl;
          kv = cf * rk;
          if (geo->bias_kind[t] != JCG_BIAS_NONE) {
            // NLA intrinsic alignment (probes.py:102-129), same ell factor as the shear
            const double nla = NZL[(size_t)t * na + n] * bias_at(geo, t, z, dz) * hz;
            kv = kv + nla * (-IA_C1_RHOCRIT * s[S_OMEGA_M] / dz);
          }
          kv = kv * (1.0 + geo->mult[t]);
        } else {
          kv = NZL[(size_t)t * na + n] * bias_at(geo, t, z, dz) * hz;
        }
        if (it.kern32) it.kern32[(size_t)t * na + n] = (float)kv;  // fp32c: what the Limber kernel reads
        else it.kern[(size_t)t * na + n] = kv;
      }
    }
  }
}

// FP32 lensing kernel for a batch sharing one geometry: lanes are 32
// cosmologies, warps walk the nodes.  The cosmology-independent lensing grid of
// a node (segments, offsets, n(z') weights) is the same for every lane, so it
// is read once per 32 cosmologies, in coalesced chunks of 32 points staged as
// point records in the warp's shared memory and read back by broadcast; each
// lane reads its cosmology's chi table from shared memory ([segment][cosmology],
// conflict-free), from the first segment a point can fall in (chi_wbase) on,
// once per run of points with the same segment query.
constexpr int TU_NODES = 32;
constexpr int TU_PAD = 33;
__host__ __device__ inline size_t tu_smem(int wn, int nw) {
  return ku_rec_bytes(nw) + sizeof(float) * 2 * (size_t)wn * TU_PAD;
}

template <int NW>  // WeakLensing tracers (one lensing group)
__global__ void __launch_bounds__(256)
    tracer32_uniform_kernel(Batch bt, const ConstTables* __restrict__ c) {
  const GeoHeader* geo = bt.geo;
  const int na = geo->na;
  const int n0 = blockIdx.x * TU_NODES;
  const int c0 = blockIdx.y * 32;
  if (n0 >= na || c0 >= bt.n_items) return;
  extern __shared__ __align__(16) float tu_sm[];
  const int wbase = bt.chi_wbase, wn = NCHI - wbase;
  float4* recs = reinterpret_cast<float4*>(tu_sm);    // [8][32][N4] point records
  float* chiT = tu_sm + 4 * 8 * 32 * KuRec<NW>::N4;  // [wn][TU_PAD]
  float* slT = chiT + wn * TU_PAD;                    // [wn][TU_PAD]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int idx = tid; idx < 32 * wn; idx += blockDim.x) {
    const int cc = idx / wn, sidx = idx % wn;
    const int ci = c0 + cc;
    float cv = 0.f, sv = 0.f;
    if (ci < bt.n_items) {
      const CosmoTab* ct = bt.ctab + ci;
      cv = ct->chi32[wbase + sidx];
      sv = ct->slope32[wbase + sidx];
    }
    chiT[sidx * TU_PAD + cc] = cv;
    slT[sidx * TU_PAD + cc] = sv;
  }
  __syncthreads();
  const int ci = c0 + lane;
  const bool live = ci < bt.n_items;
  const CosmoTab* ct = bt.ctab + (live ? ci : 0);
  const double om = ct->s[S_OMEGA_M];
  const Bg bg = make_bg(ct->s);
  const double cf = 3.0 * (H0 * H0) * om / 2.0 / C_KMS;  // probes.py:71
  const float cff = (float)cf;
  const int n_tr = geo->n_tr;
  const double* Z = geo_ptr<double>(geo, geo->off_z);
  const double* AWL = geo_ptr<double>(geo, geo->off_awl);
  const int32_t* QWL = geo_ptr<int32_t>(geo, geo->off_qwl32);
  const float* DXWL = geo_ptr<float>(geo, geo->off_dxwl32);
  const double* NZL = geo_ptr<double>(geo, geo->off_nzl);
  double* kern = bt.kern + (size_t)(live ? ci : 0) * bt.max_tr * na;
  float* kern32 = bt.kern32 ? bt.kern32 + (size_t)(live ? ci : 0) * bt.max_tr * na : nullptr;
  const int n_end = min(na, n0 + TU_NODES);
  // the WeakLensing tracers in order, and their float weights
  int wl_t[NW];
  {
    int u = 0;
    for (int t = 0; t < n_tr && u < NW; ++t)
      if (geo->kind[t] == JCG_TRACER_WL) wl_t[u++] = t;
  }
  const int32_t* Q32b = geo_ptr<int32_t>(geo, geo->off_q32[0]);
  const float* DX32b = geo_ptr<float>(geo, geo->off_dx32[0]);
  float4* recw = recs + warp * 32 * KuRec<NW>::N4;
  for (int n = n0 + warp; n < n_end; n += 8) {
    const int qw = QWL[n];
    const float chi_wl = fmaxf(
        chiT[((qw & 0xffff) - wbase) * TU_PAD + lane] + slT[((qw >> 16) - wbase) * TU_PAD + lane] * DXWL[n], 0.f);
    float acc[NW];
#pragma unroll
    for (int u = 0; u < NW; ++u) acc[u] = 0.f;
    const size_t row = (size_t)n * NZP;
    const float* Wr[NW];
#pragma unroll
    for (int u = 0; u < NW; ++u) Wr[u] = geo_ptr<float>(geo, geo->off_W32[wl_t[u]]) + row;
    // the node's lensing grid in chunks of 32 z' points: one coalesced load
    // per lane, staged as records and read back point by point (same order
    // of accumulation as a plain loop over j)
    for (int j0 = 0; j0 < NZP; j0 += 32) {
      const int jl = j0 + lane;
      const bool in = jl < NZP;
      const int qv = in ? Q32b[row + jl] : 0;
      const float dxv = in ? DX32b[row + jl] : 0.f;
      float wv[NW];
#pragma unroll
      for (int u = 0; u < NW; ++u) wv[u] = in ? Wr[u][jl] : 0.f;
      const int cnt = min(32, NZP - j0);
      ku_put_rec<NW>(recw + lane * KuRec<NW>::N4, qv, dxv, wv);
      const int qp = __shfl_up_sync(0xffffffffu, qv, 1);
      const unsigned starts = __ballot_sync(0xffffffffu, lane == 0 || qp != qv);
      __syncwarp();
      float cx = 0.f, sx = 0.f;  // chi[x], slope[m] of the current run
      for (int jj = 0; jj < cnt; ++jj) {
        int q;
        float dx, w[NW];
        ku_get_rec<NW>(recw + jj * KuRec<NW>::N4, q, dx, w);
        if ((starts >> jj) & 1u) {  // warp-uniform
          cx = chiT[((q & 0xffff) - wbase) * TU_PAD + lane];
          sx = slT[((q >> 16) - wbase) * TU_PAD + lane];
        }
        const float chip = fmaxf(cx + sx * dx, 0.f);
        const float ratio = fmaxf(chip - chi_wl, 0.f) * rcp_approx(fmaxf(chip, 1.f));
#pragma unroll
        for (int u = 0; u < NW; ++u) acc[u] += w[u] * ratio;
      }
      __syncwarp();
    }
    if (live) {
      const double z = Z[n];
      const float zf1 = (float)(1.0 + z);
#pragma unroll
      for (int u = 0; u < NW; ++u) {
        const int t = wl_t[u];
        if (kern32) {  // what the Limber kernel reads: the same product in FP32
          kern32[(size_t)t * na + n] = cff * (acc[u] * zf1 * chi_wl) * (float)(1.0 + geo->mult[t]);
        } else {
          kern[(size_t)t * na + n] = cf * ((double)acc[u] * (1.0 + z) * (double)chi_wl) * (1.0 + geo->mult[t]);
        }
      }
      if (geo->n_nc > 0) {
        const double hz = bg_H(bg, AWL[n]);
        for (int t = 0; t < n_tr; ++t)
          if (geo->kind[t] != JCG_TRACER_WL) {
            const double kv = NZL[(size_t)t * na + n] * geo->bias[t] * hz;
            if (kern32) kern32[(size_t)t * na + n] = (float)kv;
            else kern[(size_t)t * na + n] = kv;
          }
      }
    }
  }
}

template <int NW>
static void launch_tu(const Batch& b, const ConstTables* c, cudaStream_t st) {
  const size_t smem = tu_smem(NCHI - b.chi_wbase, NW);
  cudaFuncSetAttribute(tracer32_uniform_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  dim3 grid((b.max_na + TU_NODES - 1) / TU_NODES, (b.n_items + 31) / 32);
  tracer32_uniform_kernel<NW><<<grid, 256, smem, st>>>(b, c);
}

void launch_tracer_kernels(const Batch& b, const ConstTables* c, cudaStream_t st) {
  if (b.precision == JCG_FP32C && !b.listed && !b.special_bias && !b.has_delta && b.n_wl_groups == 1 && b.n_wl >= 1 &&
      b.n_wl <= 8) {
    switch (b.n_wl) {
      case 1: launch_tu<1>(b, c, st); return;
      case 2: launch_tu<2>(b, c, st); return;
      case 3: launch_tu<3>(b, c, st); return;
      case 4: launch_tu<4>(b, c, st); return;
      case 5: launch_tu<5>(b, c, st); return;
      case 6: launch_tu<6>(b, c, st); return;
      case 7: launch_tu<7>(b, c, st); return;
      default: launch_tu<8>(b, c, st); return;
    }
  }
  dim3 grid((b.max_na + TK_NODES_PER_BLOCK - 1) / TK_NODES_PER_BLOCK, b.n_items);
  if (b.precision == JCG_FP32C)
    tracer_kernels_kernel<true><<<grid, TK_WARPS * 32, 0, st>>>(b, c);
  else
    tracer_kernels_kernel<false><<<grid, TK_WARPS * 32, 0, st>>>(b, c);
}

}  // namespace jcg
