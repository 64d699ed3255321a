// Tracer radial kernels on the Limber nodes (FP64).
//
// WeakLensing (probes.py:16-74, 188-208): for each node z,
//   q_i(z) = simps_{z' in [z, zmax], 256}[ n_i(z') clip(chi' - chi, 0) / clip(chi', 1) ]
//            * (1 + z) * chi,  times 3 H0^2 Omega_m / (2 c) and (1 + m).
// The n(z') weights and the chi-table segments of every z' node are
// cosmology-independent and come precomputed in the geometry buffer; only the
// chi table is per cosmology (staged in shared memory).
// NumberCounts (probes.py:77-99, 260-272): n_i(z) * b * H(z2a(z)).
// The ell factor of WeakLensing (probes.py:73) is applied in the Limber stage.
#include "jcg_internal.cuh"

namespace jcg {

constexpr int TK_WARPS = 8;
constexpr int TK_NODES_PER_BLOCK = 32;

__global__ void __launch_bounds__(TK_WARPS * 32)
    tracer_kernels_kernel(Batch bt, const ConstTables* __restrict__ c) {
  const int item = blockIdx.y;
  if (item >= bt.n_items) return;
  const Item it = batch_item(bt, item);
  const GeoHeader* geo = it.geo;
  const int na = geo->na;
  const int n0 = blockIdx.x * TK_NODES_PER_BLOCK;
  if (n0 >= na) return;
  __shared__ double chi[NCHI];
  __shared__ double atab[NCHI];
  __shared__ double s[NSCAL];
  const CosmoTab* ct = it.ctab;
  for (int i = threadIdx.x; i < NCHI; i += blockDim.x) {
    chi[i] = ct->chi[i];
    atab[i] = c->atab_chi[i];
  }
  for (int i = threadIdx.x; i < NSCAL; i += blockDim.x) s[i] = ct->s[i];
  __syncthreads();
  const Bg bg = make_bg(s);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_tr = geo->n_tr;
  const double* Z = geo_ptr<double>(geo, geo->off_z);
  const double* AWL = geo_ptr<double>(geo, geo->off_awl);
  const int64_t* SW = geo_ptr<int64_t>(geo, geo->off_seg_chiwl);
  const double* NZL = geo_ptr<double>(geo, geo->off_nzl);
  // 3 H0^2 Omega_m / 2 / c  (probes.py:71)
  const double cf = 3.0 * (H0 * H0) * s[S_OMEGA_M] / 2.0 / C_KMS;
  const int n_end = min(na, n0 + TK_NODES_PER_BLOCK);
  for (int n = n0 + warp; n < n_end; n += TK_WARPS) {
    const double awl = AWL[n];
    const double chi_wl = fmax(interp_eval(awl, atab, chi, unpack_seg(SW[n])), 0.0);
    double acc[MAXTR];
#pragma unroll
    for (int t = 0; t < MAXTR; ++t) acc[t] = 0.0;
    for (int g = 0; g < geo->n_groups; ++g) {
      const double* AP = geo_ptr<double>(geo, geo->off_ap[g]) + (size_t)n * NZP;
      const int64_t* SP = geo_ptr<int64_t>(geo, geo->off_segp[g]) + (size_t)n * NZP;
      for (int j = lane; j < NZP; j += 32) {
        const double ap = AP[j];
        const double chip = fmax(interp_eval(ap, atab, chi, unpack_seg(SP[j])), 0.0);
        const double ratio = fmax(chip - chi_wl, 0.0) / fmax(chip, 1.0);
#pragma unroll
        for (int t = 0; t < MAXTR; ++t) {
          if (t < n_tr && geo->kind[t] == JCG_TRACER_WL && geo->group[t] == g) {
            const double* W = geo_ptr<double>(geo, geo->off_W[t]) + (size_t)n * NZP;
            acc[t] += W[j] * ratio;
          }
        }
      }
    }
#pragma unroll
    for (int t = 0; t < MAXTR; ++t) {
      if (t < n_tr && geo->kind[t] == JCG_TRACER_WL) {
        double v = acc[t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        acc[t] = v;
      }
    }
    if (lane == 0) {
      const double z = Z[n];
      for (int t = 0; t < n_tr; ++t) {
        double kv;
        if (geo->kind[t] == JCG_TRACER_WL) {
          const double rk = acc[t] * (1.0 + z) * chi_wl;
          kv = cf * rk * (1.0 + geo->mult[t]);
        } else {
          kv = NZL[(size_t)t * na + n] * geo->bias[t] * bg_H(bg, awl);
        }
        it.kern[(size_t)t * na + n] = kv;
      }
    }
  }
}

void launch_tracer_kernels(const Batch& b, const ConstTables* c, cudaStream_t st) {
  dim3 grid((b.max_na + TK_NODES_PER_BLOCK - 1) / TK_NODES_PER_BLOCK, b.n_items);
  tracer_kernels_kernel<<<grid, TK_WARPS * 32, 0, st>>>(b, c);
}

}  // namespace jcg
