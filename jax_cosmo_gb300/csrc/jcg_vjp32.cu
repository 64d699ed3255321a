// Vector-Jacobian product of angular_cl in the fp32c arithmetic: for a
// cotangent vbar_p(l) of the spectra (the derivative of a likelihood with
// respect to C_ell), the gradient
//
//   g_d = sum_{p,l} vbar_p(l) dC_p(l)/dtheta_d
//
// without forming dC/dtheta (angular_cl.py:49-98 differentiated as jax.grad
// does for a scalar function of it, README.md:14-27).  With
//   C_p(l) = ef_i(l) ef_j(l) sum_a P(l, a) M_p(a),   M_p(a) = u(a) K_i(a) K_j(a)
// and v_p(l) = vbar_p(l) ef_i(l) ef_j(l):
//
//   g_d = sum_{a,l} W(a, l) dP(l, a)/dtheta_d + sum_{a,p} Q_p(a) dM_p(a)/dtheta_d
//   W(a, l) = sum_p v_p(l) M_p(a),        Q_p(a) = sum_l v_p(l) P(l, a).
//
// dP/dtheta at a node is the reverse sweep of the integrand (jcg_node32.cuh)
// contracted with the tangents of its inputs; here the adjoints are weighted
// by W and summed over ell first, so the projection on the 8 tangent
// directions runs once per a node instead of once per (a, ell) node, and the
// contraction with the spectra is two small products (W and Q) instead of
// one per spectrum and direction.
//
// One CTA per (chunk of at most VJ_TA a nodes, cosmology); 8 lanes per a
// node, iterating over ell.  The same kernel in its forward form (FWD) gives
// the chunk's partial C_ell, from which the serving loop forms the
// likelihood's cotangent before the product.
#include "jcg_node32.cuh"
#include "jcg_ff.cuh"

namespace jcg {

constexpr int VJ_THREADS = 256;
constexpr int VJ_GROUP = 8;      // lanes per a node
constexpr int VJ_LTMAX = 256;    // ell per tile at most
constexpr int VJ_VBYTES = 32 * 1024;  // the cotangent tile [n_cls][LT] in shared memory

int vjp_ltile(int n_cls, int n_ell) {
  int lt = VJ_VBYTES / (4 * (n_cls > 0 ? n_cls : 1));
  if (lt > VJ_LTMAX) lt = VJ_LTMAX;
  lt = lt / 8 * 8;
  if (lt < 8) lt = 8;
  const int need = (n_ell + 7) / 8 * 8;
  return lt < need ? lt : need;
}

// row stride of the [.][LT] tiles: >= LT, a multiple of 4 (float4 rows) and
// 8 mod 32, so that 8 consecutive columns of 4 consecutive rows fall in 32
// distinct banks
__host__ __device__ inline int vj_stride(int LT) { return LT + (40 - LT % 32) % 32; }

struct VjLayout {
  size_t ev, kh, rows, ks, mv, mt, vs, pt, ws, abar, qd, red, total;
  size_t rows_b, ks_b;  // the second buffer of each (the next chunk's copies)
  size_t cacc;
};
// C_ell summed in shared memory (float pairs, chunk order) when one CTA runs
// all of a cosmology's chunks in one ell tile and the sums fit
constexpr int VJ_CACC_MAX = 3072;  // n_cls x n_ell float pairs (24 kB)
__host__ __device__ inline int vj_cacc(int n_cls, int n_ell, int LT, int G) {
  return G == 1 && n_ell <= LT && n_cls * n_ell <= VJ_CACC_MAX ? n_cls * n_ell : 0;
}
__host__ __device__ inline VjLayout vj_layout(int n_tr, int n_cls, int LT, int ncacc = 0) {
  VjLayout L;
  size_t o = 0;
  L.ev = o;                                   // 16 values + [NET][NDIR] tangents (floats)
  o += 4 * (16 + NET * NDIR);
  o = (o + 15) & ~(size_t)15;
  L.kh = o;                                   // [3][LT] l + 1/2, log2(l + 1/2), 1 / (l + 1/2)
  o += 4 * 3 * (size_t)LT;
  o = (o + 15) & ~(size_t)15;
  L.rows = o;                                 // [VJ_TA][NROWG]
  o += 4 * (size_t)VJ_TA * NROWG;
  L.rows_b = o;
  o += 4 * (size_t)VJ_TA * NROWG;
  L.ks = o;                                   // [VJ_TA][n_tr][NDIR + 1]
  o += 4 * (size_t)VJ_TA * n_tr * (NDIR + 1);
  o = (o + 15) & ~(size_t)15;
  L.ks_b = o;
  o += 4 * (size_t)VJ_TA * n_tr * (NDIR + 1);
  o = (o + 15) & ~(size_t)15;
  L.mv = o;                                   // [VJ_TA][n_cls]
  o += 4 * (size_t)VJ_TA * n_cls;
  o = (o + 15) & ~(size_t)15;
  L.mt = o;                                   // [n_cls][VJ_TA] (M transposed)
  o += 4 * (size_t)VJ_TA * n_cls;
  L.vs = o;                                   // [n_cls][vj_stride(LT)]
  o += 4 * (size_t)n_cls * vj_stride(LT);
  L.pt = o;                                   // [VJ_TA][vj_stride(LT)] P(t, l)
  o += 4 * (size_t)VJ_TA * vj_stride(LT);
  L.ws = o;                                   // [VJ_TA][vj_stride(LT)] W(t, l)
  o += 4 * (size_t)VJ_TA * vj_stride(LT);
  L.abar = o;                                 // [VJ_TA][NGT]
  o += 4 * (size_t)VJ_TA * NGT;
  o = (o + 15) & ~(size_t)15;
  L.qd = o;                                   // [VJ_TA][n_cls] float pairs
  o += 8 * (size_t)VJ_TA * n_cls;
  L.red = o;                                  // [VJ_THREADS / 32][NET] floats, then [VJ_TA][NDIR] doubles of room
  o += 4 * (size_t)(VJ_THREADS / 32) * NET;
  o = (o + 15) & ~(size_t)15;
  o += 8 * (size_t)VJ_TA * NDIR;
  o = (o + 15) & ~(size_t)15;
  L.cacc = o;                                 // [n_cls][n_ell] float pairs (or none)
  o += 8 * (size_t)ncacc;
  L.total = o;
  return L;
}

// asynchronous global -> shared copies (no register staging; all of a
// thread's copies in flight at once), completed by cp_async_wait_all
__device__ __forceinline__ void cp_async16(void* s, const void* g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(s)), "l"(g)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* s, const void* g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(s)), "l"(g)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// wait for all committed groups but the most recent one
__device__ __forceinline__ void cp_async_wait_prior() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// GEN: some item may use a non-default operator point (as grad_limber32).
// FWD: the forward form (partial C_ell of the chunk, no cotangent).
template <bool GEN, bool FWD>
__global__ void __launch_bounds__(VJ_THREADS, 2) grad_vjp32_kernel(GradBatch gb, int LT, int G) {
  const int item = blockIdx.y;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const GeoHeader* geo = gi.geo;
  const int n_ell = geo->n_ell, n_cls = geo->n_cls, na = geo->na, n_tr = geo->n_tr;
  const int nch = vjp_chunks(na), tav = vjp_tav(na);
  if ((int)blockIdx.x >= nch) return;
  const bool lin = pk_model(geo->physics) == JCG_PK_LINEAR;
  const bool nw = GEN && tf_nowiggle(geo->physics);
  const int ncacc = (FWD || gb.vjp_cl) && !gb.listed ? vj_cacc(n_cls, n_ell, LT, G) : 0;  // as the launch
  const VjLayout L = vj_layout(n_tr, n_cls, LT, ncacc);
  extern __shared__ __align__(16) unsigned char vj_smem[];
  float2* Cacc = reinterpret_cast<float2*>(vj_smem + L.cacc);
  float* ev = reinterpret_cast<float*>(vj_smem + L.ev);
  float* et = ev + 16;
  float* khv = reinterpret_cast<float*>(vj_smem + L.kh);
  float* lkhv = khv + LT;
  float* ikhv = lkhv + LT;
  float* const R0 = reinterpret_cast<float*>(vj_smem + L.rows);
  float* const R1 = reinterpret_cast<float*>(vj_smem + L.rows_b);
  float* const K0 = reinterpret_cast<float*>(vj_smem + L.ks);
  float* const K1 = reinterpret_cast<float*>(vj_smem + L.ks_b);
  float* Mv = reinterpret_cast<float*>(vj_smem + L.mv);
  float* MT = reinterpret_cast<float*>(vj_smem + L.mt);
  float* vS = reinterpret_cast<float*>(vj_smem + L.vs);
  float* Pt = reinterpret_cast<float*>(vj_smem + L.pt);
  float* Ws = reinterpret_cast<float*>(vj_smem + L.ws);
  const int TS = vj_stride(LT);
  float* Abar = reinterpret_cast<float*>(vj_smem + L.abar);
  float2* Qd = reinterpret_cast<float2*>(vj_smem + L.qd);  // Q_p(t) as (hi, lo)
  float* Ered = reinterpret_cast<float*>(vj_smem + L.red);
  float2* gred = reinterpret_cast<float2*>(vj_smem + ((L.red + 4 * (VJ_THREADS / 32) * NET + 15) & ~(size_t)15));
  const int tid = threadIdx.x, grp = tid >> 3, sub = tid & (VJ_GROUP - 1);
  const TabD* tb = gi.tab;
  // a chunk's FP32 rows (values and tangents) and radial kernels into buffer
  // b: asynchronous copies (one commit group per chunk)
  auto copy_chunk = [&](int ch, int b) {
    const int c0 = ch * tav, cc = min(tav, na - c0);
    const float* src = gi.rowg + (size_t)c0 * NROWG;
    float* R = b ? R1 : R0;
    for (int i = tid; i < cc * (NROWG / 4); i += VJ_THREADS) cp_async16(R + 4 * i, src + 4 * i);
    // K rows [t][tracer][NDIR + 1]: consecutive threads on consecutive nodes.
    // With the shear integral in reverse over a uniform batch, a WeakLensing
    // kernel without NLA term has zero tangents, which the value kernel does
    // not store: they are set here.
    float* K = b ? K1 : K0;
    for (int i = tid; i < cc * n_tr; i += VJ_THREADS) {
      const int tr = i / cc, t = i - tr * cc;
      const float* ks = gi.kernf + ((size_t)tr * na + c0 + t) * (NDIR + 1);
      float* kd = K + ((size_t)t * n_tr + tr) * (NDIR + 1);
      if (gb.krev_u && geo->kind[tr] == JCG_TRACER_WL && geo->bias_kind[tr] == JCG_BIAS_NONE) {
        cp_async4(kd, ks);
#pragma unroll
        for (int k = 1; k < NDIR + 1; ++k) kd[k] = 0.f;
      } else {
#pragma unroll
        for (int k = 0; k < NDIR + 1; ++k) cp_async4(kd + k, ks + k);
      }
    }
  };
  // the Eisenstein-Hu inputs and their tangents (formed once per cosmology
  // by the table stage) and the first chunk's rows
  for (int i = tid; i < 16; i += VJ_THREADS) cp_async4(ev + i, tb->ehv + i);
  if (!FWD)
    for (int i = tid; i < NET * NDIR; i += VJ_THREADS) cp_async4(et + i, tb->eht + i);
  copy_chunk(blockIdx.x, 0);
  cp_async_commit();
  const float4* KH4 = geo_ptr<float4>(geo, geo->off_kh4);
  const float* EF32 = geo_ptr<float>(geo, geo->off_ef32);
  // an ell tile's (l + 1/2) factors and, for the product, its cotangents
  // v_p(l) = vbar_p(l) ef_i(l) ef_j(l); with one tile, once per CTA while the
  // first copies fly (read-only loads, free to move past the shared-memory
  // stores)
  auto fill_tile = [&](int l0, int lt) {
    for (int l = tid; l < lt; l += VJ_THREADS) {
      const float4 k4 = __ldg(KH4 + l0 + l);
      khv[l] = k4.x;
      lkhv[l] = k4.y;
      ikhv[l] = k4.z;
    }
    if (!FWD)
      for (int w = tid; w < lt * n_tr; w += VJ_THREADS) {
        // one thread per (ell, first tracer i); the pairs in the geometry's
        // order: (i, j >= i) row by row
        const int i = w / lt, l = w - i * lt;
        const int ell = l0 + l;
        const float efi = __ldg(EF32 + (size_t)i * n_ell + ell);
        int p = i * n_tr - (i * (i - 1)) / 2;
        for (int j = i; j < n_tr; ++j, ++p)
          vS[p * TS + l] =
              (float)__ldg(gi.vbar + (size_t)p * n_ell + ell) * (efi * __ldg(EF32 + (size_t)j * n_ell + ell));
      }
  };
  const bool one_tile = n_ell <= LT;
  if (one_tile) fill_tile(0, n_ell);
  for (int i = tid; i < ncacc; i += VJ_THREADS) Cacc[i] = make_float2(0.f, 0.f);
  // the CTA's chunks blockIdx.x, blockIdx.x + G, ...: the next chunk's rows
  // are copied while this one runs
  for (int chunk = blockIdx.x, it = 0; chunk < nch; chunk += G, ++it) {
    const int buf = it & 1;
    float* R = buf ? R1 : R0;
    float* Ks = buf ? K1 : K0;
    if (chunk + G < nch) copy_chunk(chunk + G, buf ^ 1);
    cp_async_commit();
    cp_async_wait_prior();  // every group but the one just committed
    if (!one_tile) fill_tile(0, min(LT, n_ell));
    const int a0 = chunk * tav, tc = min(tav, na - a0);
    if (!FWD)
      for (int i = tid; i < tc * n_cls; i += VJ_THREADS) Qd[i] = make_float2(0.f, 0.f);
    __syncthreads();
    // M_p(a) = u K_i K_j, the operation order of grad_limber32
    // (one thread per (a node, first tracer i); pair p = (i, j >= i))
    for (int q = tid; q < tc * n_tr; q += VJ_THREADS) {
      const int t = q / n_tr, i = q - t * n_tr;
      const float* Kt = Ks + (size_t)t * n_tr * (NDIR + 1);
      const float u = R[(size_t)t * NROWG + F_U], ki = Kt[i * (NDIR + 1)];
      int p = i * n_tr - (i * (i - 1)) / 2;
      for (int j = i; j < n_tr; ++j, ++p) {
        const float m = u * (ki * Kt[j * (NDIR + 1)]);
        Mv[t * n_cls + p] = m;
        MT[p * VJ_TA + t] = m;
      }
    }
    EHg eh;
    eh.qinv = ev[0]; eh.lg2_qinv = ev[1]; eh.sh = ev[2]; eh.inv_sh = ev[3]; eh.c18bc = ev[4];
    eh.c142ac = ev[5]; eh.alpha_b = ev[6]; eh.beta_b = ev[7]; eh.beta_node = ev[8]; eh.lg2_ksilk = ev[9];
    eh.fb = ev[10]; eh.fc = ev[11]; eh.ns3 = ev[12]; eh.inv_keq = ev[13];
    eh.agam = ev[14]; eh.nwq = ev[15];
    float accA[T_U], accE[NET];
#pragma unroll
    for (int j = 0; j < T_U; ++j) accA[j] = 0.f;
#pragma unroll
    for (int j = 0; j < NET; ++j) accE[j] = 0.f;
    for (int l0 = 0; l0 < n_ell; l0 += LT) {
      const int lt = min(LT, n_ell - l0);
      if (l0 > 0) {
        __syncthreads();  // the previous tile's Pt / vS are consumed
        fill_tile(l0, lt);
      }
      __syncthreads();  // the tile's factors and cotangents (first tile: and M)
      const int L4 = (lt + 3) >> 2;
      if (!FWD) {
        // W(t, l) = sum_p M_p(t) v_p(l) in 4 x 4 blocks (rows past tc and
        // columns past lt are not read)
        for (int w = tid; w < (VJ_TA / 4) * L4; w += VJ_THREADS) {
          const int tb = w / L4, lq = (w - tb * L4) * 4, t0 = tb * 4;
          float4 a[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) a[i] = make_float4(0.f, 0.f, 0.f, 0.f);
          for (int p = 0; p < n_cls; ++p) {
            const float4 m = *reinterpret_cast<const float4*>(MT + p * VJ_TA + t0);
            const float4 v = *reinterpret_cast<const float4*>(vS + p * TS + lq);
            const float mm[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              a[i].x = fmaf(mm[i], v.x, a[i].x);
              a[i].y = fmaf(mm[i], v.y, a[i].y);
              a[i].z = fmaf(mm[i], v.z, a[i].z);
              a[i].w = fmaf(mm[i], v.w, a[i].w);
            }
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) *reinterpret_cast<float4*>(Ws + (t0 + i) * TS + lq) = a[i];
        }
        __syncthreads();
      }
      if (grp < tc) {
        const int t = grp;
        const float* row = R + (size_t)t * NROWG;
        for (int l = sub; l < lt; l += VJ_GROUP) {
          float an[NGT], ae[NET];
          const float P = !GEN ? node32_fb_default(eh, row, khv[l], lkhv[l], ikhv[l], an, ae)
                          : nw ? node32_fb_nw(eh, row, khv[l], lkhv[l], ikhv[l], an, ae, lin)
                               : node32_fb<true>(eh, row, khv[l], lkhv[l], ikhv[l], an, ae, lin);
          Pt[t * TS + l] = P;
          if (!FWD) {
            const float W = Ws[t * TS + l];
#pragma unroll
            for (int j = 0; j < T_U; ++j) {
              if (!GEN && j == T_MUN) continue;  // mu_n = 0 for takahashi2012
              accA[j] = fmaf(W, an[j], accA[j]);
            }
#pragma unroll
            for (int j = 0; j < NET; ++j) accE[j] = fmaf(W, ae[j], accE[j]);
          }
        }
      }
      __syncthreads();
      if (FWD || gb.vjp_cl) {
        // partial C_p(l) of the chunk: sum_t M_p(t) P(t, l), t in order, in
        // blocks of 2 spectra x 4 ell
        float* cp = gi.cpart + (size_t)chunk * n_cls * n_ell;
        const int P2 = (n_cls + 1) >> 1;
        for (int w = tid; w < P2 * L4; w += VJ_THREADS) {
          const int pb = w / L4, lq = (w - pb * L4) * 4, p0 = pb * 2;
          const bool two = p0 + 1 < n_cls;
          float4 c0 = make_float4(0.f, 0.f, 0.f, 0.f), c1 = c0;
          for (int t = 0; t < tc; ++t) {
            const float4 pt = *reinterpret_cast<const float4*>(Pt + t * TS + lq);
            const float m0 = Mv[t * n_cls + p0], m1 = two ? Mv[t * n_cls + p0 + 1] : 0.f;
            c0.x = fmaf(pt.x, m0, c0.x), c0.y = fmaf(pt.y, m0, c0.y), c0.z = fmaf(pt.z, m0, c0.z), c0.w = fmaf(pt.w, m0, c0.w);
            c1.x = fmaf(pt.x, m1, c1.x), c1.y = fmaf(pt.y, m1, c1.y), c1.z = fmaf(pt.z, m1, c1.z), c1.w = fmaf(pt.w, m1, c1.w);
          }
          const float r0[4] = {c0.x, c0.y, c0.z, c0.w}, r1[4] = {c1.x, c1.y, c1.z, c1.w};
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (lq + k >= lt) break;
            if (ncacc) {  // the chunks in order, as the global sum below
              float2* c0p = Cacc + p0 * n_ell + lq + k;
              const FF s0 = FF{c0p->x, c0p->y} + r0[k];
              *c0p = make_float2(s0.hi, s0.lo);
              if (two) {
                float2* c1p = c0p + n_ell;
                const FF s1 = FF{c1p->x, c1p->y} + r1[k];
                *c1p = make_float2(s1.hi, s1.lo);
              }
            } else {
              cp[(size_t)p0 * n_ell + l0 + lq + k] = r0[k];
              if (two) cp[(size_t)(p0 + 1) * n_ell + l0 + lq + k] = r1[k];
            }
          }
        }
      }
      if (!FWD) {
        // Q_p(t) += sum_l v_p(l) P(t, l): blocks of 4 a nodes x 4 spectra
        // (p = 16 g + b + 4 k), each summed over 8 ell slices in FP32 and the
        // slices added by shuffles, then added to Q in float-pair arithmetic
        const int NPG = (n_cls + 15) >> 4;
        for (int w = tid; w < (VJ_THREADS) * NPG; w += VJ_THREADS) {
          const int pg = w / VJ_THREADS, r = w - pg * VJ_THREADS;
          const int slice = r & 7, blk = r >> 3, t0 = (blk >> 2) * 4, pb = blk & 3;
          int pk[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) pk[k] = pg * 16 + pb + 4 * k;
          float acc[4][4];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][k] = 0.f;
          for (int l = slice; l < lt; l += 8) {
            float pt[4], v[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) pt[i] = Pt[(t0 + i) * TS + l];
#pragma unroll
            for (int k = 0; k < 4; ++k) v[k] = pk[k] < n_cls ? vS[pk[k] * TS + l] : 0.f;
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int k = 0; k < 4; ++k) acc[i][k] = fmaf(pt[i], v[k], acc[i][k]);
          }
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              float x = acc[i][k];
              x += __shfl_xor_sync(0xffffffffu, x, 4);
              x += __shfl_xor_sync(0xffffffffu, x, 2);
              x += __shfl_xor_sync(0xffffffffu, x, 1);
              acc[i][k] = x;
            }
          if (slice == 0) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int k = 0; k < 4; ++k) {
                const int t = t0 + i, p = pk[k];
                if (t < tc && p < n_cls) {
                  const int q = t * n_cls + p;
                  const FF sq = FF{Qd[q].x, Qd[q].y} + acc[i][k];
                  Qd[q] = make_float2(sq.hi, sq.lo);
                }
              }
          }
        }
      }
    }
    if ((FWD || gb.vjp_cl) && !ncacc) {
      // C_ell of the item once all its chunks are in: the last chunk CTA to
      // finish adds the partials in chunk order (the same sum whichever CTA
      // it is), times the ell factors, and resets the count
      __shared__ int s_last;
      __threadfence();
      __syncthreads();
      if (tid == 0) s_last = atomicAdd(&gb.cl_count[item], 1u) == (unsigned)(nch - 1);
      __syncthreads();
      if (s_last && gi.cl) {
        __threadfence();
        const double* EF = geo_ptr<double>(geo, geo->off_ellfac);
        const size_t per = (size_t)n_cls * n_ell;
        for (int idx = tid; idx < (int)per; idx += VJ_THREADS) {
          const int p = idx / n_ell, l = idx - p * n_ell;
          // chunks added in order, in float pairs; loads issued eight at a time
          FF s{0.f, 0.f};
          int c = 0;
          for (; c + 8 <= nch; c += 8) {
            float v[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) v[k] = __ldcg(gi.cpart + (size_t)(c + k) * per + idx);
#pragma unroll
            for (int k = 0; k < 8; ++k) s = s + v[k];
          }
          for (; c < nch; ++c) s = s + __ldcg(gi.cpart + (size_t)c * per + idx);
          gi.cl[idx] = ffd(s) * EF[(size_t)geo->pair_i[p] * n_ell + l] * EF[(size_t)geo->pair_j[p] * n_ell + l];
        }
      }
      if (s_last && tid == 0) gb.cl_count[item] = 0;
    }
    if (FWD) {
      __syncthreads();  // this chunk's buffers and scratch are free
      continue;
    }
    // adjoints of the node inputs: summed over the a node's 8 lanes; those of
    // the cosmology's Eisenstein-Hu inputs over the CTA
#pragma unroll
    for (int j = 0; j < T_U; ++j) {
      float v = accA[j];
      v += __shfl_xor_sync(0xffffffffu, v, 4);
      v += __shfl_xor_sync(0xffffffffu, v, 2);
      v += __shfl_xor_sync(0xffffffffu, v, 1);
      if (sub == 0 && grp < tc) Abar[grp * NGT + j] = v;
    }
    const int warp = tid >> 5, lane = tid & 31;
#pragma unroll
    for (int j = 0; j < NET; ++j) {
      float v = accE[j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) Ered[warp * NET + j] = v;
    }
    __syncthreads();
    // the Eisenstein-Hu adjoints over the warps, one thread per input (float
    // pairs), into the first row of Ered
    FF ej{0.f, 0.f};
    if (tid < NET)
      for (int w = 0; w < VJ_THREADS / 32; ++w) ej = ej + Ered[w * NET + tid];
    // reverse lensing: the cotangents of the WeakLensing shear kernels,
    // Kbar_i(t) = u(t) sum_p Q_p(t) dK_i K_j / dK_i (both factors of an auto pair)
    if (gb.vjp_rev)
      for (int q = tid; q < tc * n_tr; q += VJ_THREADS) {
        const int t = q / n_tr, i = q - t * n_tr;
        if (geo->kind[i] != JCG_TRACER_WL || geo->nz_kind[i] == JCG_NZ_DELTA) continue;
        const float2* qv = Qd + (size_t)t * n_cls;
        const float* K = Ks + (size_t)t * n_tr * (NDIR + 1);
        FF kb{0.f, 0.f};
        for (int j = 0; j < n_tr; ++j) {
          const int lo = min(i, j), hi = max(i, j);
          const int p = lo * n_tr - (lo * (lo - 1)) / 2 + (hi - lo);
          const FF qp{qv[p].x, qv[p].y};
          const float kj = K[j * (NDIR + 1)];
          kb = kb + qp * kj;
          if (j == i) kb = kb + qp * kj;  // both factors of the auto pair
        }
        gi.kbar[(size_t)i * na + a0 + t] = R[(size_t)t * NROWG + F_U] * kb.hi;
      }
    __syncthreads();  // every read of Ered is done
    if (tid < NET) {
      Ered[2 * tid] = ej.hi;
      Ered[2 * tid + 1] = ej.lo;
    }
    __syncthreads();
    // projection on the tangents: thread (a node t, direction d), in float
    // pairs; the sum over t by shuffles within the warp (4 nodes), then over
    // the 8 warps in order
    {
      const int t = tid >> 3, d = tid & 7;
      FF gd{0.f, 0.f};
      if (t < tc) {
        const float* row = R + (size_t)t * NROWG;
        const float* tg = row + NROWV;
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < T_U; ++j) {
          if (!GEN && j == T_MUN) continue;
          s = fmaf(Abar[t * NGT + j], tg[j * NDIR + d], s);
        }
        // sum_p Q_p (du K_i K_j + u (dK_i K_j + K_i dK_j)), in float pairs
        const float u = row[F_U], du = tg[T_U * NDIR + d];
        const float2* q = Qd + (size_t)t * n_cls;
        FF sm{0.f, 0.f};
        int p = 0;
        for (int i = 0; i < n_tr; ++i) {
          const float* Ki = Ks + ((size_t)t * n_tr + i) * (NDIR + 1);
          const float ki0 = Ki[0], kid = Ki[1 + d];
          for (int j = i; j < n_tr; ++j, ++p) {
            const float* Kj = Ks + ((size_t)t * n_tr + j) * (NDIR + 1);
            const float dm = fmaf(du, ki0 * Kj[0], u * fmaf(kid, Kj[0], ki0 * Kj[1 + d]));
            sm = sm + FF{q[p].x, q[p].y} * dm;
          }
        }
        gd = sm + s;
      }
      if (t == 0) {
        // the cosmology's Eisenstein-Hu inputs, once per CTA
        FF se{0.f, 0.f};
        for (int j = 0; j < NET; ++j) se = se + FF{Ered[2 * j], Ered[2 * j + 1]} * et[j * NDIR + d];
        gd = gd + se;
      }
#pragma unroll
      for (int o = 8; o < 32; o <<= 1)
        gd = gd + FF{__shfl_xor_sync(0xffffffffu, gd.hi, o), __shfl_xor_sync(0xffffffffu, gd.lo, o)};
      if (lane < NDIR) gred[warp * NDIR + lane] = make_float2(gd.hi, gd.lo);
    }
    __syncthreads();
    if (tid < NDIR) {
      FF g{0.f, 0.f};
      for (int w = 0; w < VJ_THREADS / 32; ++w) g = g + FF{gred[w * NDIR + tid].x, gred[w * NDIR + tid].y};
      gi.gpart[(size_t)chunk * NDIR + tid] = ffd(g);
    }
    __syncthreads();  // this chunk's buffers and scratch are free
  }
  if (ncacc && gi.cl) {
    // every chunk of the cosmology ran here: C_ell from the sums
    const double* EF = geo_ptr<double>(geo, geo->off_ellfac);
    for (int idx = tid; idx < ncacc; idx += VJ_THREADS) {
      const int p = idx / n_ell, l = idx - p * n_ell;
      gi.cl[idx] = ffd(FF{Cacc[idx].x, Cacc[idx].y}) * EF[(size_t)geo->pair_i[p] * n_ell + l] *
                   EF[(size_t)geo->pair_j[p] * n_ell + l];
    }
  }
}

// Reverse form of the WeakLensing shear kernel (probes.py:44-51, 71-73)
//   K_i(a) = (1 + m_i) cf (1 + z) chi_w acc_i,  acc_i = sum_j W_ij r_j,
//   r_j = max(chi'_j - chi_w, 0) / max(chi'_j, 1),  cf = 3 H0^2 Omega_m / 2c
// given the cotangents Kbar_i(a) of the product kernel: the gradient
//   sum_{a,i} Kbar_i(a) dK_i(a)/dtheta
//   = dlncf L + sum_a cw(a) dchi_w(a) + sum_{a,j} c_j(a) dchi'_j(a)
// with L = sum Kbar_i K_i, cw = fac sum_i Kbar_i (1 + m_i) (acc_i - chi_w at_i)
// (at_i = sum_j W_ij / max(chi'_j, 1) over chi'_j > chi_w) and c_j = fac chi_w
// h_j sum_i Kbar_i (1 + m_i) W_ij, h_j = (1 - r_j [chi'_j > 1]) / max(chi'_j, 1).
// chi' and chi_w are interpolations chi[x] + slope[m] dx of the chi table, so
// their cotangents gather on the table's nodes and segment slopes and meet
// the table's 8 tangents once per CTA, instead of the 8 tangents meeting
// every lensing point.  One CTA per KV_NODES Limber nodes of one cosmology,
// one warp per node, lanes over the 257 z' points, the WeakLensing tracers
// of one lensing group per pass.  The gather is deterministic: the table
// index of consecutive z' points is monotone, so a segmented warp scan sums
// each index's run and the run's last lane adds it to the warp's own copy
// of the table cotangents; the 8 copies are added in a fixed order (the
// same result alone and in any batch, bit for bit).
template <int TP>
__global__ void __launch_bounds__(256) grad_kernrev32_kernel(GradBatch gb) {
  const int item = blockIdx.y, chunk = blockIdx.x;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const GeoHeader* geo = gi.geo;
  const int na = geo->na, n_tr = geo->n_tr;
  const int n0 = chunk * KV_NODES;
  if (n0 >= na) return;
  __shared__ int ptr_t[JCG_MAX_TRACERS * TP];
  __shared__ int pgroup[JCG_MAX_TRACERS];
  __shared__ int npass_s;
  __shared__ float chi[NCHI], slope[NCHI];
  __shared__ float cbw[8][NCHI], sbw[8][NCHI];  // per-warp table cotangents
  __shared__ float lsum[8];
  __shared__ double red[8][NDIR];
  const TabD* tb = gi.tab;
  if (threadIdx.x == 0) {
    int np = 0;
    for (int g = 0; g < geo->n_groups; ++g) {
      int u = TP;
      for (int t = 0; t < n_tr; ++t) {
        if (geo->kind[t] != JCG_TRACER_WL || geo->group[t] != g || geo->nz_kind[t] == JCG_NZ_DELTA) continue;
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
  for (int i = threadIdx.x; i < NCHI; i += blockDim.x) {
    chi[i] = tb->c32[0][i];
    slope[i] = tb->s32[0][i];
  }
  for (int i = threadIdx.x; i < 8 * NCHI; i += blockDim.x) {
    (&cbw[0][0])[i] = 0.f;
    (&sbw[0][0])[i] = 0.f;
  }
  __syncthreads();
  const int npass = npass_s;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double* Z = geo_ptr<double>(geo, geo->off_z);
  const int32_t* QWL = geo_ptr<int32_t>(geo, geo->off_qwl32);
  const float* DXWL = geo_ptr<float>(geo, geo->off_dxwl32);
  const float cff = (float)(3.0 * (H0 * H0) * tb->sv[S_OMEGA_M] / 2.0 / C_KMS);  // probes.py:71
  float lacc = 0.f;  // sum Kbar K over this lane's nodes (lane 0)
  const int n_end = min(na, n0 + KV_NODES);
  for (int n = n0 + warp; n < n_end; n += 8) {
    const int qw = QWL[n];
    const int xw = qw & 0xffff, mw = qw >> 16;
    const float dxw = DXWL[n];
    const float craw_w = chi[xw] + slope[mw] * dxw;
    const float chi_wl = fmaxf(craw_w, 0.f);
    const float fac = cff * (float)(1.0 + Z[n]);
    const size_t row = (size_t)n * NZP;
    for (int pass = 0; pass < npass; ++pass) {
      const int g = pgroup[pass];
      float kb[TP], av[TP], at[TP];
      const float* W[TP];
      bool any = false;
#pragma unroll
      for (int u = 0; u < TP; ++u) {
        const int t = ptr_t[pass * TP + u];
        kb[u] = t >= 0 ? gi.kbar[(size_t)t * na + n] * (1.f + (float)geo->mult[t]) : 0.f;
        W[u] = t >= 0 ? geo_ptr<float>(geo, geo->off_W32[t]) + row : nullptr;
        any |= kb[u] != 0.f;
        av[u] = 0.f;
        at[u] = 0.f;
      }
      if (!any) continue;  // the same on every lane of the warp
      const int32_t* Q32 = geo_ptr<int32_t>(geo, geo->off_q32[g]) + row;
      const float* DX32 = geo_ptr<float>(geo, geo->off_dx32[g]) + row;
      const float cj_fac = fac * chi_wl;
      float* cb = cbw[warp];
      float* sb = sbw[warp];
      for (int jb = 0; jb < NZP; jb += 32) {
        const int j = jb + lane;
        int x = -1, m = -1;
        float cj = 0.f, cjdx = 0.f;
        if (j < NZP) {
          const int q = Q32[j];
          x = q & 0xffff, m = q >> 16;
          const float dx = DX32[j];
          const float craw = chi[x] + slope[m] * dx;
          const float chip = fmaxf(craw, 0.f);
          const float diff = chip - chi_wl;
          if (diff > 0.f) {  // then craw > 0 too
            const float ic = rcpf(fmaxf(chip, 1.f));
            const float r = diff * ic;
            const float h = chip > 1.f ? ic * (1.f - r) : ic;
            float sw = 0.f;
#pragma unroll
            for (int u = 0; u < TP; ++u) {
              if (W[u]) {
                const float w = W[u][j];
                av[u] = fmaf(w, r, av[u]);
                at[u] = fmaf(w, ic, at[u]);
                sw = fmaf(kb[u], w, sw);
              }
            }
            cj = cj_fac * h * sw;
            cjdx = cj * dx;
          }
        }
        // segmented inclusive scans over runs of equal x and of equal m
        // (both monotone in j), then the run's last lane adds the run
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const float vc = __shfl_up_sync(0xffffffffu, cj, o), vs = __shfl_up_sync(0xffffffffu, cjdx, o);
          const int kx = __shfl_up_sync(0xffffffffu, x, o), km = __shfl_up_sync(0xffffffffu, m, o);
          if (lane >= o && kx == x) cj += vc;
          if (lane >= o && km == m) cjdx += vs;
        }
        const int nx = __shfl_down_sync(0xffffffffu, x, 1), nm = __shfl_down_sync(0xffffffffu, m, 1);
        if (x >= 0 && (lane == 31 || nx != x)) cb[x] += cj;
        if (m >= 0 && (lane == 31 || nm != m)) sb[m] += cjdx;
        __syncwarp();
      }
      float cw = 0.f, lk = 0.f;
#pragma unroll
      for (int u = 0; u < TP; ++u) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          av[u] += __shfl_xor_sync(0xffffffffu, av[u], o);
          at[u] += __shfl_xor_sync(0xffffffffu, at[u], o);
        }
        cw = fmaf(kb[u], av[u] - chi_wl * at[u], cw);
        lk = fmaf(kb[u], av[u], lk);
      }
      if (lane == 0) {
        lacc = fmaf(fac * chi_wl, lk, lacc);
        if (craw_w > 0.f) {
          cb[xw] += fac * cw;
          sb[mw] += fac * cw * dxw;
        }
      }
      __syncwarp();
    }
  }
  if (lane == 0) lsum[warp] = lacc;
  __syncthreads();
  // meet the chi table's tangents: sum_x cbar dchi_d[x] + sbar dslope_d[x]
  double acc[NDIR];
#pragma unroll
  for (int d = 0; d < NDIR; ++d) acc[d] = 0.0;
  {
    float s[NDIR];
#pragma unroll
    for (int d = 0; d < NDIR; ++d) s[d] = 0.f;
    for (int x = threadIdx.x; x < NCHI; x += blockDim.x) {
      float cb = 0.f, sb = 0.f;
      for (int w = 0; w < 8; ++w) cb += cbw[w][x], sb += sbw[w][x];
#pragma unroll
      for (int d = 0; d < NDIR; ++d) s[d] = fmaf(cb, tb->c32[1 + d][x], fmaf(sb, tb->s32[1 + d][x], s[d]));
    }
#pragma unroll
    for (int d = 0; d < NDIR; ++d) {
      float v = s[d];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][d] = (double)v;
    }
  }
  __syncthreads();
  if (threadIdx.x < NDIR) {
    const int d = threadIdx.x;
    double g = 0.0, L = 0.0;
    for (int w = 0; w < 8; ++w) {
      g += red[w][d];
      L += (double)lsum[w];
    }
    // d ln cf / dtheta = d Omega_m / Omega_m
    g += L * (tb->sd[d][S_OMEGA_M] / tb->sv[S_OMEGA_M]);
    gi.kpart[(size_t)chunk * NDIR + d] = g;
  }
}

// ------------------------------------------------ uniform reverse lensing --
// A batch sharing one geometry (one lensing group, no single-plane n(z)):
// lanes are 32 cosmologies, as in the forward tracer32_uniform_kernel, so the
// lensing grid of a node (segments, offsets, n(z') weights) is read once per
// 32 cosmologies, every branch on it is warp-uniform, and each lane reads its
// cosmology's chi table from shared memory ([segment][cosmology]).  Only the
// table segments from krev_wbase up can hold a Limber node or lensing point
// (a >= z2a(max(zmax, probe zmax))), so the shared tables start there.
constexpr int KU_PAD = 33;
constexpr int KU_NODES = 32;  // nodes per CTA of the value kernel

__host__ __device__ inline size_t ku_val_smem(int wn, int nw) {
  return ku_rec_bytes(nw) + sizeof(float) * 2 * (size_t)wn * KU_PAD;
}
__host__ __device__ inline size_t ku_rev_smem(int wn, int nw) {
  return ku_rec_bytes(nw) + sizeof(float) * ((size_t)4 * wn * KU_PAD + (size_t)8 * KV_NODES * KU_PAD + 16 * KU_PAD);
}
bool krev_uniform_ok(const GeoHeader& h) {
  return !h.custom_nodes && h.n_wl >= 1 && h.n_wl <= 8 && h.n_groups == 1 && !h.has_delta;
}

// first chi table segment (atab_chi = logspace(-3, 0, NCHI)) that a Limber
// node or a lensing point can fall in, two segments of margin
int krev_wbase(const GeoHeader& h) {
  if (h.custom_nodes) return 0;  // nodes at the caller's redshifts: the whole table
  double zm = h.zmax;
  for (int g = 0; g < h.n_groups; ++g) zm = fmax(zm, h.group_zmax[g]);
  const double t = (log10(1.0 / (1.0 + zm)) + 3.0) * (NCHI - 1) / 3.0;
  int w = (int)floor(t) - 2;
  if (!(t > 2.0)) w = 0;
  return w > NCHI - 2 ? NCHI - 2 : w;
}

// K_t(a) of the WeakLensing tracers (probes.py:44-51, 71-73) with no shear
// tangents (the reverse kernel below takes the integral's cotangents):
//   K = cf (1 + z) chi_w sum_j W_tj r_j (1 + m_t),
// the per-cosmology grad_kern32_kernel's values in the lanes-over-cosmologies
// layout.  Writes the value and 8 zero tangents of each (tracer, node); the
// kernel stage adds NLA terms to them afterwards.
template <int NW>
__global__ void __launch_bounds__(256) grad_kernval32u_kernel(GradBatch gb) {
  const GeoHeader* geo = gb.geo;
  const int na = geo->na, n_tr = geo->n_tr;
  const int n0 = blockIdx.x * KU_NODES, c0 = blockIdx.y * 32;
  if (n0 >= na || c0 >= gb.n_items) return;
  const int wbase = gb.krev_wbase, wn = NCHI - wbase;
  extern __shared__ __align__(16) float kv_smem[];
  float4* recs = reinterpret_cast<float4*>(kv_smem);  // [8][32][N4] point records
  float* chiT = kv_smem + 4 * 8 * 32 * KuRec<NW>::N4;  // [wn][KU_PAD]
  float* slT = chiT + wn * KU_PAD;   // [wn][KU_PAD]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int idx = tid; idx < 32 * wn; idx += blockDim.x) {
    const int cc = idx / wn, i = idx % wn;
    const int ci = c0 + cc;
    float cv = 0.f, sv = 0.f;
    if (ci < gb.n_items) {
      cv = gb.tab[ci].c32[0][wbase + i];
      sv = gb.tab[ci].s32[0][wbase + i];
    }
    chiT[i * KU_PAD + cc] = cv;
    slT[i * KU_PAD + cc] = sv;
  }
  __syncthreads();
  const int ci = c0 + lane;
  const bool live = ci < gb.n_items;
  const TabD* tb = gb.tab + (live ? ci : c0);
  const float cff = (float)(3.0 * (H0 * H0) * tb->sv[S_OMEGA_M] / 2.0 / C_KMS);  // probes.py:71
  int wl_t[NW];
  float m1[NW];
  {
    int u = 0;
    for (int t = 0; t < n_tr && u < NW; ++t)
      if (geo->kind[t] == JCG_TRACER_WL) wl_t[u++] = t;
#pragma unroll
    for (int v = 0; v < NW; ++v) m1[v] = 1.f + (float)geo->mult[wl_t[v]];
  }
  const double* Z = geo_ptr<double>(geo, geo->off_z);
  const int32_t* QWL = geo_ptr<int32_t>(geo, geo->off_qwl32);
  const float* DXWL = geo_ptr<float>(geo, geo->off_dxwl32);
  const int32_t* Q32b = geo_ptr<int32_t>(geo, geo->off_q32[0]);
  const float* DX32b = geo_ptr<float>(geo, geo->off_dx32[0]);
  const float* Wb[NW];
#pragma unroll
  for (int u = 0; u < NW; ++u) Wb[u] = geo_ptr<float>(geo, geo->off_W32[wl_t[u]]);
  float* kf = gb.kernf + (size_t)(live ? ci : c0) * n_tr * na * (NDIR + 1);
  const int n_end = min(na, n0 + KU_NODES);
  for (int n = n0 + warp; n < n_end; n += 8) {
    const int qw = QWL[n];
    const float craw_w = chiT[((qw & 0xffff) - wbase) * KU_PAD + lane] + slT[((qw >> 16) - wbase) * KU_PAD + lane] * DXWL[n];
    const float chi_wl = fmaxf(craw_w, 0.f);
    float acc[NW];
#pragma unroll
    for (int u = 0; u < NW; ++u) acc[u] = 0.f;
    const size_t row = (size_t)n * NZP;
    for (int j0 = 0; j0 < NZP; j0 += 32) {
      const int jl = j0 + lane;
      const bool in = jl < NZP;
      const int qv = in ? Q32b[row + jl] : 0;
      const float dxv = in ? DX32b[row + jl] : 0.f;
      float wv[NW];
#pragma unroll
      for (int u = 0; u < NW; ++u) wv[u] = in ? Wb[u][row + jl] : 0.f;
      const int cnt = min(32, NZP - j0);
      float4* recw = recs + warp * 32 * KuRec<NW>::N4;
      ku_put_rec<NW>(recw + lane * KuRec<NW>::N4, qv, dxv, wv);
      __syncwarp();
      for (int jj = 0; jj < cnt; ++jj) {
        int q;
        float dx, w[NW];
        ku_get_rec<NW>(recw + jj * KuRec<NW>::N4, q, dx, w);
        const float chip =
            fmaxf(chiT[((q & 0xffff) - wbase) * KU_PAD + lane] + slT[((q >> 16) - wbase) * KU_PAD + lane] * dx, 0.f);
        const float diff = chip - chi_wl;
        const float r = diff > 0.f ? diff * rcpf(fmaxf(chip, 1.f)) : 0.f;
#pragma unroll
        for (int u = 0; u < NW; ++u) acc[u] = fmaf(w[u], r, acc[u]);
      }
      __syncwarp();
    }
    if (live) {
      const float fac = cff * (float)(1.0 + Z[n]);
#pragma unroll
      for (int u = 0; u < NW; ++u) {
        // the value only: the shear integral's tangents are zero (taken in
        // reverse), and the product kernel fills them in shared memory
        kf[((size_t)wl_t[u] * na + n) * (NDIR + 1)] = fac * chi_wl * acc[u] * m1[u];
      }
    }
  }
}

// Segment ownership of the 8 warps of grad_kernrev32u_kernel per chunk of
// KV_NODES nodes: warp w takes the chunk's lensing points whose chi table
// segment m lies in [b_w, b_{w+1}); the boundaries split the chunk's points
// into near-equal eighths.  (Integer histogram: the same bounds every run.)
// Also each warp's range of points [jlo, jhi) on every node of the chunk
// (contiguous: the segment is monotone along a node's z' grid), packed
// jlo | jhi << 16 into ranges[node][warp].
__global__ void __launch_bounds__(256) kernrev_owner_kernel(const GeoHeader* geo, int* bounds, int* ranges) {
  const int chunk = blockIdx.x, na = geo->na;
  const int n0 = chunk * KV_NODES, n_end = min(na, n0 + KV_NODES);
  __shared__ int hist[NCHI];
  for (int i = threadIdx.x; i < NCHI; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  const int32_t* Q32 = geo_ptr<int32_t>(geo, geo->off_q32[0]) + (size_t)n0 * NZP;
  const int cnt = (n_end - n0) * NZP;
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) atomicAdd(&hist[Q32[i] >> 16], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int* b = bounds + (size_t)chunk * 9;
    b[0] = 0;
    int below = 0, w = 1;  // below: points with a segment < m
    for (int m = 0; m < NCHI; ++m) {
      while (w < 8 && (long long)below * 8 >= (long long)w * cnt) b[w++] = m;
      below += hist[m];
    }
    while (w < 8) b[w++] = NCHI;
    b[8] = NCHI;
  }
  __syncthreads();
  // thread (node, warp): the warp's points on the node
  const int* b = bounds + (size_t)chunk * 9;
  for (int q = threadIdx.x; q < (n_end - n0) * 8; q += blockDim.x) {
    const int nl = q >> 3, w = q & 7;
    const int blo = b[w], bhi = b[w + 1];
    const int32_t* row = Q32 + (size_t)nl * NZP;
    int jlo = NZP, jhi = 0;
    for (int j = 0; j < NZP; ++j) {
      const int m = row[j] >> 16;
      if (m >= blo && m < bhi) {
        jlo = min(jlo, j);
        jhi = j + 1;
      }
    }
    if (jhi <= jlo) jlo = jhi = 0;
    ranges[(size_t)(n0 + nl) * 8 + w] = jlo | (jhi << 16);
  }
}

// Reverse form of the shear integral (the same sums as grad_kernrev32_kernel,
// whose header derives them), lanes over 32 cosmologies.  The warps share a
// chunk of KV_NODES nodes and split its lensing points by segment
// (kernrev_owner_kernel), so the cotangents of a lane's chi table nodes
// cN[x] and segment slopes sB[m] are written by one warp only, in a fixed
// order: warp w owns the slopes of [b_w, b_{w+1}) and the nodes
// [b_w, b_{w+1} - 1]; what its top segment gives node b_{w+1} it keeps in a
// register (bS in shared memory at the end).    The segment of
// consecutive points changes every few points: the current run's sums stay
// in registers and go to shared memory when it changes.  The chi_w
// cotangents (one per node and warp) and the sums for d ln cf wait in shared
// memory; at the end warp d meets them all with tangent d of each lane's
// chi table.  One partial gradient per (cosmology, node chunk) in kpart.
template <int NW>
__global__ void __launch_bounds__(256) grad_kernrev32u_kernel(GradBatch gb) {
  const GeoHeader* geo = gb.geo;
  const int na = geo->na, n_tr = geo->n_tr;
  const int chunk = blockIdx.x, c0 = blockIdx.y * 32;
  const int n0 = chunk * KV_NODES;
  if (n0 >= na || c0 >= gb.n_items) return;
  const int n_end = min(na, n0 + KV_NODES);
  const int wbase = gb.krev_wbase, wn = NCHI - wbase;
  extern __shared__ __align__(16) float kr_smem[];
  float4* recs = reinterpret_cast<float4*>(kr_smem);  // [8][32][N4] point records
  float* chiT = kr_smem + 4 * 8 * 32 * KuRec<NW>::N4;  // [wn][KU_PAD]
  float* slT = chiT + wn * KU_PAD;              // [wn][KU_PAD]
  float* cN = slT + wn * KU_PAD;                // [wn][KU_PAD]
  float* sB = cN + wn * KU_PAD;                 // [wn][KU_PAD]
  float* cwS = sB + wn * KU_PAD;                // [8][KV_NODES][KU_PAD]
  float* lS = cwS + 8 * KV_NODES * KU_PAD;      // [8][KU_PAD]
  float* bS = lS + 8 * KU_PAD;                  // [8][KU_PAD]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int idx = tid; idx < 32 * wn; idx += blockDim.x) {
    const int cc = idx / wn, i = idx % wn;
    const int ci = c0 + cc;
    float cv = 0.f, sv = 0.f;
    if (ci < gb.n_items) {
      cv = gb.tab[ci].c32[0][wbase + i];
      sv = gb.tab[ci].s32[0][wbase + i];
    }
    chiT[i * KU_PAD + cc] = cv;
    slT[i * KU_PAD + cc] = sv;
    cN[i * KU_PAD + cc] = 0.f;
    sB[i * KU_PAD + cc] = 0.f;
  }
  for (int idx = tid; idx < 8 * KV_NODES * KU_PAD; idx += blockDim.x) cwS[idx] = 0.f;
  __syncthreads();
  const int ci = c0 + lane;
  const bool live = ci < gb.n_items;
  const TabD* tb = gb.tab + (live ? ci : c0);
  const float cff = (float)(3.0 * (H0 * H0) * tb->sv[S_OMEGA_M] / 2.0 / C_KMS);  // probes.py:71
  const float* kbar = gb.kbar + (size_t)(live ? ci : c0) * n_tr * na;
  int wl_t[NW];
  float m1[NW];
  {
    int u = 0;
    for (int t = 0; t < n_tr && u < NW; ++t)
      if (geo->kind[t] == JCG_TRACER_WL) wl_t[u++] = t;
#pragma unroll
    for (int v = 0; v < NW; ++v) m1[v] = 1.f + (float)geo->mult[wl_t[v]];
  }
  const double* Z = geo_ptr<double>(geo, geo->off_z);
  const int32_t* QWL = geo_ptr<int32_t>(geo, geo->off_qwl32);
  const float* DXWL = geo_ptr<float>(geo, geo->off_dxwl32);
  const int32_t* Q32b = geo_ptr<int32_t>(geo, geo->off_q32[0]);
  const float* DX32b = geo_ptr<float>(geo, geo->off_dx32[0]);
  const float* Wb[NW];
#pragma unroll
  for (int u = 0; u < NW; ++u) Wb[u] = geo_ptr<float>(geo, geo->off_W32[wl_t[u]]);
  const int bhi = gb.krev_owner[chunk * 9 + warp + 1];
  float rc = 0.f, rcd = 0.f;  // the current run's chi' cotangent, and times dx
  float lacc = 0.f;       // sum_n fac chi_w sum_j sw r  (the d ln cf sum)
  float bacc = 0.f;       // node bhi's cotangent from segment bhi - 1
  // a run (consecutive points of one segment query, nearest | segment << 16)
  // ends: its sums go to the table cotangents
  auto flush = [&](int q) {
    const int m = q >> 16, i = (m - wbase) * KU_PAD + lane;
    if ((q & 0xffff) == m) cN[i] += rc;
    else if (m + 1 < bhi) cN[i + KU_PAD] += rc;
    else bacc += rc;
    sB[i] += rcd;
    rc = 0.f;
    rcd = 0.f;
  };
  for (int n = n0; n < n_end; ++n) {
    const int qw = QWL[n];
    const float craw_w =
        chiT[((qw & 0xffff) - wbase) * KU_PAD + lane] + slT[((qw >> 16) - wbase) * KU_PAD + lane] * DXWL[n];
    const float chi_wl = fmaxf(craw_w, 0.f);
    const float fac = cff * (float)(1.0 + Z[n]);
    const float cjf = fac * chi_wl;
    float kb[NW];
#pragma unroll
    for (int u = 0; u < NW; ++u) kb[u] = kbar[(size_t)wl_t[u] * na + n] * m1[u];
    const size_t row = (size_t)n * NZP;
    float lk = 0.f, cwa = 0.f;
    const int jr = gb.krev_ranges[(size_t)n * 8 + warp];
    const int jlo = jr & 0xffff, jhi = jr >> 16;
    for (int j0 = jlo; j0 < jhi; j0 += 32) {
      const int jl = j0 + lane;
      const bool own = jl < jhi;
      const int cnt = min(32, jhi - j0), jf = 0;
      const int qv = own ? Q32b[row + jl] : -1;
      const float dxv = own ? DX32b[row + jl] : 0.f;
      float wv[NW];
#pragma unroll
      for (int u = 0; u < NW; ++u) wv[u] = own ? Wb[u][row + jl] : 0.f;
      const int qn = __shfl_down_sync(0xffffffffu, qv, 1);
      const unsigned ends = __ballot_sync(0xffffffffu, own && (lane == jf + cnt - 1 || qn != qv));
      float4* recw = recs + warp * 32 * KuRec<NW>::N4;
      if (own) ku_put_rec<NW>(recw + lane * KuRec<NW>::N4, qv, dxv, wv);
      __syncwarp();
      for (int k = 0; k < cnt; ++k) {
        const int jj = jf + k;
        int q;
        float dx, w[NW];
        ku_get_rec<NW>(recw + jj * KuRec<NW>::N4, q, dx, w);
        float sw = 0.f;  // sum_t Kbar_t (1 + m_t) W_tj
#pragma unroll
        for (int u = 0; u < NW; ++u) sw = fmaf(kb[u], w[u], sw);
        const float chip =
            fmaxf(chiT[((q & 0xffff) - wbase) * KU_PAD + lane] + slT[((q >> 16) - wbase) * KU_PAD + lane] * dx, 0.f);
        const float diff = chip - chi_wl;
        if (diff > 0.f) {  // then the chi' clip is inactive too
          const float ic = rcpf(fmaxf(chip, 1.f));
          const float r = diff * ic;
          const float h = chip > 1.f ? ic * (1.f - r) : ic;  // dr / dchi'
          lk = fmaf(sw, r, lk);
          cwa = fmaf(sw, fmaf(-chi_wl, ic, r), cwa);  // dr / dchi_w = -ic
          const float ch = cjf * h * sw;
          rc += ch;
          rcd = fmaf(ch, dx, rcd);
        }
        if ((ends >> jj) & 1u) flush(q);  // warp-uniform
      }
      __syncwarp();
    }
    lacc = fmaf(cjf, lk, lacc);
    cwS[(warp * KV_NODES + (n - n0)) * KU_PAD + lane] = craw_w > 0.f ? fac * cwa : 0.f;
  }
  lS[warp * KU_PAD + lane] = lacc;
  bS[warp * KU_PAD + lane] = bacc;
  __syncthreads();
  if (!live) return;
  // warp d: the table cotangents against tangent d of the lane's chi table
  const int d = warp;
  const float* dc = tb->c32[1 + d];
  const float* ds = tb->s32[1 + d];
  float g = 0.f;
  for (int i = 0; i < wn; ++i) g = fmaf(cN[i * KU_PAD + lane], dc[wbase + i], fmaf(sB[i * KU_PAD + lane], ds[wbase + i], g));
#pragma unroll
  for (int w = 0; w < 7; ++w) {
    const int x = gb.krev_owner[chunk * 9 + w + 1];
    if (x < NCHI) g = fmaf(bS[w * KU_PAD + lane], dc[x], g);
  }
  for (int n = n0; n < n_end; ++n) {
    float cw = 0.f;
#pragma unroll
    for (int w = 0; w < 8; ++w) cw += cwS[(w * KV_NODES + (n - n0)) * KU_PAD + lane];
    const int qw = QWL[n];
    g = fmaf(cw, fmaf(ds[qw >> 16], DXWL[n], dc[qw & 0xffff]), g);
  }
  float L = 0.f;
#pragma unroll
  for (int w = 0; w < 8; ++w) L += lS[w * KU_PAD + lane];
  // d ln cf / dtheta = d Omega_m / Omega_m
  gb.kpart[((size_t)ci * kv_chunks(na) + chunk) * NDIR + d] =
      (double)g + (double)L * (tb->sd[d][S_OMEGA_M] / tb->sv[S_OMEGA_M]);
}

template <int NW>
static void launch_ku(const GradBatch& gb, cudaStream_t st, bool rev) {
  const int wn = NCHI - gb.krev_wbase;
  if (rev) {
    const size_t smem = ku_rev_smem(wn, NW);
    cudaFuncSetAttribute(grad_kernrev32u_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(kv_chunks(gb.na), (gb.n_items + 31) / 32);
    grad_kernrev32u_kernel<NW><<<grid, 256, smem, st>>>(gb);
  } else {
    const size_t smem = ku_val_smem(wn, NW);
    cudaFuncSetAttribute(grad_kernval32u_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((gb.na + KU_NODES - 1) / KU_NODES, (gb.n_items + 31) / 32);
    grad_kernval32u_kernel<NW><<<grid, 256, smem, st>>>(gb);
  }
}

static void launch_ku_nw(const GradBatch& gb, cudaStream_t st, bool rev) {
  switch (gb.n_wl) {
    case 1: launch_ku<1>(gb, st, rev); return;
    case 2: launch_ku<2>(gb, st, rev); return;
    case 3: launch_ku<3>(gb, st, rev); return;
    case 4: launch_ku<4>(gb, st, rev); return;
    case 5: launch_ku<5>(gb, st, rev); return;
    case 6: launch_ku<6>(gb, st, rev); return;
    case 7: launch_ku<7>(gb, st, rev); return;
    default: launch_ku<8>(gb, st, rev); return;
  }
}

void launch_kernval32u(const GradBatch& gb, cudaStream_t st) { launch_ku_nw(gb, st, false); }

// the gradient from the chunks' partials (fixed order)
__global__ void vjp_grad_reduce_kernel(GradBatch gb) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int item = idx / NDIR, d = idx % NDIR;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const int nch = vjp_chunks(gi.geo->na);
  double g = 0.0;
  for (int c = 0; c < nch; ++c) g += gi.gpart[(size_t)c * NDIR + d];
  if (gb.vjp_rev) {
    const int nk = kv_chunks(gi.geo->na);
    for (int c = 0; c < nk; ++c) g += gi.kpart[(size_t)c * NDIR + d];
  }
  gi.grad[d] = g;
}

template <bool GEN, bool FWD>
static void launch_vjp_t(const GradBatch& gb, cudaStream_t st) {
  const int LT = vjp_ltile(gb.n_cls, gb.n_ell);
  // chunks per cosmology spread over G CTAs (each loops over its chunks),
  // G as small as keeps about 4 CTAs per SM in the grid
  const int nch = vjp_chunks(gb.na);
  int G = (4 * device_sm_count() + gb.n_items - 1) / gb.n_items;
  G = G < 1 ? 1 : (G > nch ? nch : G);
  // (a listed batch's sizes are maxima: its items take the global sums)
  const int ncacc = (FWD || gb.vjp_cl) && !gb.listed ? vj_cacc(gb.n_cls, gb.n_ell, LT, G) : 0;
  const size_t smem = vj_layout(gb.n_tr, gb.n_cls, LT, ncacc).total;
  cudaFuncSetAttribute(grad_vjp32_kernel<GEN, FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if ((FWD || gb.vjp_cl) && !ncacc) cudaMemsetAsync(gb.cl_count, 0, sizeof(unsigned) * (size_t)gb.n_items, st);
  dim3 grid(G, gb.n_items);
  grad_vjp32_kernel<GEN, FWD><<<grid, VJ_THREADS, smem, st>>>(gb, LT, G);
}

// forward: C_ell into the items' cl (uniform batch: gb.cl)
void launch_vjp32_cl(const GradBatch& gb, cudaStream_t st) {
  if (gb.physics_or != 0) launch_vjp_t<true, true>(gb, st);
  else launch_vjp_t<false, true>(gb, st);
}

// the product with the items' cotangents vbar into their grad
void launch_vjp32_grad(const GradBatch& gb, cudaStream_t st, unsigned stages) {
  if (stages & GS_PRODUCT) {
    if (gb.physics_or != 0) launch_vjp_t<true, false>(gb, st);
    else launch_vjp_t<false, false>(gb, st);
  }
  if (!(stages & GS_REVERSE)) return;
  if (gb.vjp_rev && gb.krev_u) {
    kernrev_owner_kernel<<<kv_chunks(gb.na), 256, 0, st>>>(gb.geo, gb.krev_owner, gb.krev_ranges);
    launch_ku_nw(gb, st, true);
  } else if (gb.vjp_rev) {
    dim3 grid(kv_chunks(gb.na), gb.n_items);
    if (gb.n_tr <= 3) grad_kernrev32_kernel<3><<<grid, 256, 0, st>>>(gb);
    else if (gb.n_tr <= 5) grad_kernrev32_kernel<5><<<grid, 256, 0, st>>>(gb);
    else grad_kernrev32_kernel<8><<<grid, 256, 0, st>>>(gb);
  }
  vjp_grad_reduce_kernel<<<(gb.n_items * NDIR + 127) / 128, 128, 0, st>>>(gb);
}

}  // namespace jcg
