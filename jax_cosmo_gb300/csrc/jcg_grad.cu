// Derivatives of C_ell with respect to the 8 Cosmology leaves (core.py:98-108):
// the Jacobian dC_ij(l)/dtheta of angular_cl (angular_cl.py:49-98), FP64.
//
// Tables (background ODEs, sigma8, sigma^2(R), P(k) k^3), per-node halofit
// parameters and radial kernels are differentiated forward: value + 8
// tangents.  Scalar chains run with one tangent direction per lane (lanes 0-7
// of a warp each carry Dual<1>), per-term loops with Dual<8>.  The Limber
// integrand, evaluated n_ell x Na times, is differentiated backward by a
// hand-written reverse sweep (node_fb) that returns dP/d(inputs); contracting
// with the inputs' tangents gives dP/dtheta, and
//   dC_ij(l)/dtheta = ef_ij(l) sum_a [dP(l,a)/dtheta M_ij(a) + P(l,a) dM_ij(a)/dtheta].
// The tables are recomputed here from the parameters, not taken from a
// forward pass.  Derivative conventions are JAX's for the reference's
// operations (max/min pass the tangent of the selected branch; the
// interpolation segment is locally constant).
#include <string.h>

#include <vector>

#include "jcg_fp32.cuh"
#include "jcg_grad.cuh"
#include "jcg_dualff.cuh"

namespace jcg {

// value as a float pair, 8 FP32 tangents: the fp32c table stages (jcg_dualff.cuh)
typedef DualFF<NDIR> FF8;

// Tables of one cosmology with tangents.  Lanes: dir = tid & 7, item = tid >> 3.
// F32T (fp32c Jacobian): the per-node evaluations (ODE right-hand sides,
// Eisenstein-Hu at the Romberg and halofit k nodes) run one node per thread in
// DualF<8> -- value in FP64, tangents in FP32 -- instead of one direction per
// lane; the sigma^2(R) tangents are FP32 sums; float copies of the chi and
// P(k) k^3 tangent tables are written for the FP32 stages.  The sequential
// scans (chi prefix sum, growth RK4, Romberg) stay FP64 Dual<1>.
// fp32c node arrays, packed: [n] float-pair values (float2), then
// [NDIR][n] float tangents (5 n doubles of storage); written by
// grad_nodes_kernel, read by grad_tables_kernel, no float64 conversion on
// either side.
__device__ __forceinline__ void put_packed(double* arr, int n, int e, const FF8& x) {
  reinterpret_cast<float2*>(arr)[e] = make_float2(x.v.hi, x.v.lo);
  float* tg = reinterpret_cast<float*>(arr + n);
#pragma unroll
  for (int d = 0; d < NDIR; ++d) tg[d * n + e] = x.d[d];
}
__device__ __forceinline__ FF packed_v(const double* arr, int e) {
  const float2 v = reinterpret_cast<const float2*>(arr)[e];
  return FF{v.x, v.y};
}
__device__ __forceinline__ float packed_t(const double* arr, int n, int d, int e) {
  return reinterpret_cast<const float*>(arr + n)[d * n + e];
}
__device__ __forceinline__ FF8 ff8_packed(const double* arr, int n, int e) {
  FF8 r;
  r.v = packed_v(arr, e);
#pragma unroll
  for (int d = 0; d < NDIR; ++d) r.d[d] = packed_t(arr, n, d, e);
  return r;
}

// The chi table (background.py:227-233) of one component for one warp, in
// float pairs from the packed arrays: prefix sums of the RK4 increments
// h/6 (f_{i-1} + 2 fm_i + 2 fm_i + f_i) in ln a (scipy/ode.py:21, the first
// step has h = 0), then chi_i = Y[-1] - Y_i.  Lane l holds nodes
// 8l .. 8l + 7 (returned in v).  The value (comp 0) forms its increments in
// float pairs; a tangent in FP32 (its inputs are FP32).
__device__ __forceinline__ void chi_scan_ff(const double* fnode, const double* fmid, const float2* h6, int comp,
                                            int lane, FF* v) {
  const bool value = comp == 0;
  const int d = comp - 1;
  FF loc[8];
  FF s{0.f, 0.f};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int i = lane * 8 + k;
    if (i > 0) {
      if (value) {
        const FF fmv = packed_v(fmid, i);
        s = s + (((packed_v(fnode, i - 1) + ff_scale2(fmv, 2.f)) + ff_scale2(fmv, 2.f)) + packed_v(fnode, i)) *
                    f2ff(h6[i]);
      } else {
        const float fmv = packed_t(fmid, NCHI, d, i);
        s = s + h6[i].x * (((packed_t(fnode, NCHI, d, i - 1) + 2.f * fmv) + 2.f * fmv) + packed_t(fnode, NCHI, d, i));
      }
    }
    loc[k] = s;
  }
  FF x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const FF u{__shfl_up_sync(0xffffffffu, x.hi, o), __shfl_up_sync(0xffffffffu, x.lo, o)};
    if (lane >= o) x = u + x;
  }
  FF off{__shfl_up_sync(0xffffffffu, x.hi, 1), __shfl_up_sync(0xffffffffu, x.lo, 1)};
  if (lane == 0) off = FF{0.f, 0.f};
  const FF tot{__shfl_sync(0xffffffffu, x.hi, 31), __shfl_sync(0xffffffffu, x.lo, 31)};
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = tot - (off + loc[k]);
}

// NW: some item may use the transfer type "eisenhu"
template <bool F32T, bool NW>
__global__ void __launch_bounds__(F32T ? 128 : 256, F32T ? 4 : 1) grad_tables_kernel(GradBatch gb, const ConstTables* __restrict__ c) {
  const int item = blockIdx.x;
  if (item >= gb.n_items) return;
  extern __shared__ __align__(16) double sm[];
  double* sv = sm;                      // NSCAL
  double* sd = sv + NSCAL;              // [NDIR][NSCAL]
  // FP64: [NDIR+1][n] doubles per array; fp32c: the packed layout of
  // grad_nodes_kernel (GNODE_* offsets)
  double* fn = sd + NDIR * NSCAL;       // f at the chi nodes
  double* fm = fn + (F32T ? GNODE_FM : (NDIR + 1) * NCHI);  // f at the chi midpoints
  double* qr = fn + (F32T ? GNODE_QR : 2 * (NDIR + 1) * NCHI);  // qa, ra, qm, rm
  double* fr = fn + (F32T ? GNODE_FR : 2 * (NDIR + 1) * NCHI + 4 * (NDIR + 1) * NGROW);  // Romberg integrand
  double* g1s = F32T ? fn + GNODE_U : fr + (NDIR + 1) * NROMB;  // [NDIR+1]
  double* pq = qr;                            // FP64: [NDIR+1][NKH], after the growth RK4
  const int t = threadIdx.x, dir = t & 7, it = t >> 3;
  const GradItem gi = grad_item(gb, item);
  TabD* out = gi.tab;
  // the chi and growth tables go straight to the output (read back after a barrier)
  // scalars and their tangents (from grad_scalars_kernel)
  for (int i = t; i < NSCAL; i += blockDim.x) sv[i] = out->sv[i];
  for (int i = t; i < NDIR * NSCAL; i += blockDim.x) sd[i] = out->sd[i / NSCAL][i % NSCAL];
  __syncthreads();
  D1 sD[NSCAL];
  for (int i = 0; i < NSCAL; ++i) sD[i] = mk1(sv[i], sd[dir * NSCAL + i]);
  const BgT<D1> bg = make_bgT(sD);
  auto put = [&](double* arr, int stride, int e, const D1& x) {
    if (dir == 0) arr[e] = x.v;
    arr[(1 + dir) * stride + e] = x.d[0];
  };
  auto putf = [&](double* arr, int stride, int e, const auto& x) {
    arr[e] = val(x);
#pragma unroll
    for (int d = 0; d < NDIR; ++d) arr[(1 + d) * stride + e] = x.d[d];
  };
  if (!F32T) {
    // chi RK4 right-hand side at nodes and midpoints (background.py:227-231)
    for (int e = it; e < 2 * NCHI; e += 32) {
      if (e < NCHI) {
        put(fn, NCHI, e, dchi_dlnaT(bg, c->lna_chi[e]));
      } else if (e > NCHI) {
        const int i = e - NCHI;
        const double t0 = c->lna_chi[i - 1], t1 = c->lna_chi[i];
        put(fm, NCHI, i, dchi_dlnaT(bg, t0 + (t1 - t0) / 2));
      }
    }
    // growth ODE coefficients (background.py:96-106)
    for (int e = it; e < 2 * NGROW; e += 32) {
      D1 q, r;
      if (e < NGROW) {
        growth_qrT(bg, c->atab_grow[e], q, r);
        put(qr + 0 * (NDIR + 1) * NGROW, NGROW, e, q);
        put(qr + 1 * (NDIR + 1) * NGROW, NGROW, e, r);
      } else if (e > NGROW) {
        const int i = e - NGROW;
        const double x = c->atab_grow[i], xp = c->atab_grow[i - 1];
        growth_qrT(bg, xp + (x - xp) / 2, q, r);
        put(qr + 2 * (NDIR + 1) * NGROW, NGROW, i, q);
        put(qr + 3 * (NDIR + 1) * NGROW, NGROW, i, r);
      }
    }
    // sigmasqr(8) integrand at the romb nodes (power.py:70-75)
    for (int e = it; e < NROMB; e += 32) {
      const double logk = c->romb_logk[e];
      const double k = exp(logk);
      const double x = k * 8.0;
      const double wf = 3.0 * (sin(x) - x * cos(x)) / (x * x * x);
      const D1 T = eh_transferT<NW>(sD, k, logk);
      const D1 pk = (T * T) * xexp(sD[S_NS] * logk);
      const double kw = k * wf;
      put(fr, NROMB, e, k * (kw * kw) * pk);
    }
  } else {
    // node values from grad_nodes_kernel: the same packed layout as fn .. fr here;
    // 16-byte copies, eight in flight per thread
    static_assert((9 * NSCAL) % 2 == 0 && GNODE_STRIDE % 2 == 0, "16-byte aligned node copy");
    static_assert(GNODE_U % 2 == 0, "whole 16-byte node copies");
    const double2* src = reinterpret_cast<const double2*>(gb.gnode + (size_t)item * GNODE_STRIDE);
    double2* dst = reinterpret_cast<double2*>(fn);
    constexpr int NV = GNODE_U / 2;
    for (int i0 = t; i0 < NV; i0 += 8 * blockDim.x) {
      double2 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = i0 + u * blockDim.x;
        if (i < NV) v[u] = src[i];
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = i0 + u * blockDim.x;
        if (i < NV) dst[i] = v[u];
      }
    }
  }
  __syncthreads();
  const int warp = t >> 5, lane = t & 31;
  if (F32T) {
    // fp32c: the three sequential scans as parallel scans (128 threads).
    // Growth: one RK4 step is linear in y = (D, dD/da), y_i = M_i y_{i-1};
    // thread i forms M_i (FP64) and its tangents dM_i (FP32) by running the
    // step on the unit vectors in DualF<8>.
    double m4[4] = {1.0, 0.0, 0.0, 1.0};
    float dm4[4][NDIR];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int d = 0; d < NDIR; ++d) dm4[q][d] = 0.f;
    if (t >= 1 && t < NGROW) {
      const double* QA = qr;
      const double* RA = qr + 5 * NGROW;
      const double* QM = qr + 10 * NGROW;
      const double* RM = qr + 15 * NGROW;
      auto g8 = [&](const double* arr, int e) { return ff8_packed(arr, NGROW, e); };
      const FF8 qa0 = g8(QA, t - 1), ra0 = g8(RA, t - 1), qm = g8(QM, t), rm = g8(RM, t);
      const FF8 qa1 = g8(QA, t), ra1 = g8(RA, t);
      const double hh = c->atab_grow[t] - c->atab_grow[t - 1];
      const FF8 one = ffd_const<NDIR>(1.0), zero = ffd_const<NDIR>(0.0);
      FF8 o0, o1;
      growth_rk4_step(one, zero, qa0, ra0, qm, rm, qa1, ra1, hh, o0, o1);  // column 0
      m4[0] = val(o0), m4[2] = val(o1);
#pragma unroll
      for (int d = 0; d < NDIR; ++d) dm4[0][d] = o0.d[d], dm4[2][d] = o1.d[d];
      growth_rk4_step(zero, one, qa0, ra0, qm, rm, qa1, ra1, hh, o0, o1);  // column 1
      m4[1] = val(o0), m4[3] = val(o1);
#pragma unroll
      for (int d = 0; d < NDIR; ++d) dm4[1][d] = o0.d[d], dm4[3][d] = o1.d[d];
    }
    __syncthreads();  // every read of the growth coefficients is done
    double* Mv = qr;                                          // [NGROW][4]
    float* dMv = reinterpret_cast<float*>(qr + 4 * NGROW);    // [NGROW][4][NDIR]
    double* Yv = qr + 4 * NGROW + 2 * NDIR * NGROW;           // [NGROW][2] y_i
    float* Mvf = reinterpret_cast<float*>(Yv + 2 * NGROW);   // [NGROW][4] float copies
    float* Yvf = Mvf + 4 * NGROW;                             // [NGROW][2] float copies
    static_assert(4 * NGROW + 2 * NDIR * NGROW + 2 * NGROW + 3 * NGROW <= GNODE_QR_SPAN, "growth scratch span");
    if (t < NGROW) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        Mv[t * 4 + q] = m4[q];
        Mvf[t * 4 + q] = (float)m4[q];
#pragma unroll
        for (int d = 0; d < NDIR; ++d) dMv[(t * 4 + q) * NDIR + d] = dm4[q][d];
      }
    }
    __syncthreads();
    if (warp == 0) {
      double ys[4];
      const double yf = growth_scan_warp(Mv, c->atab_grow[0], 1.0, lane, ys, Yv);
      const double iyf = 1.0 / yf;
      for (int k = 0; k < 4; ++k) {
        const int i = lane * 4 + k;
        const double gvv = ys[k] * iyf;
        out->gv[i] = gvv;
        const FF gf = ff_of(gvv);
        out->gF[i] = make_float2(gf.hi, gf.lo);  // the row stage's copy
        Yvf[i * 2] = (float)Yv[i * 2];
        Yvf[i * 2 + 1] = (float)Yv[i * 2 + 1];
      }
    } else {
      // chi for the value and the 8 tangents, in float pairs; the FP32 tables
      // (values, segment slopes) and the row stage's copies straight from
      // the sums
      for (int comp = warp - 1; comp < NDIR + 1; comp += 3) {
        FF v[8];
        chi_scan_ff(fn, fm, c->chi_h6_ff, comp, lane, v);
        const FF vn{__shfl_down_sync(0xffffffffu, v[0].hi, 1), __shfl_down_sync(0xffffffffu, v[0].lo, 1)};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int i = lane * 8 + k;
          const FF nxt = k < 7 ? v[k + 1] : vn;
          out->c32[comp][i] = v[k].hi;
          out->s32[comp][i] = i + 1 < NCHI ? ((nxt - v[k]) * f2ff(c->chi_ida_ff[i])).hi : 0.f;
          if (comp == 0) out->chiF[i] = make_float2(v[k].hi, v[k].lo);
          else out->chidF[i][comp - 1] = v[k].hi;
        }
      }
      // sigmasqr(8) (power.py:70-78): romb is linear in the integrand values,
      // sum_e w_e f_e with the weights of the Richardson combination (the
      // value in float pairs, a tangent in FP32)
      for (int comp = warp - 1; comp < NDIR + 1; comp += 3) {
        if (comp == 0) {
          FF sf{0.f, 0.f};
          for (int e = lane; e < NROMB; e += 32) sf = sf + f2ff(c->romb_w_ff[e]) * packed_v(fr, e);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1)
            sf = sf + FF{__shfl_xor_sync(0xffffffffu, sf.hi, o), __shfl_xor_sync(0xffffffffu, sf.lo, o)};
          if (lane == 0) sv[S_SIGMASQR8] = ffd(sf * ffc(1.0 / (2.0 * (PI * PI))));
        } else {
          float sf = 0.f;
          for (int e = lane; e < NROMB; e += 32) sf = fmaf(c->romb_w_ff[e].x, packed_t(fr, NROMB, comp - 1, e), sf);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) sf += __shfl_xor_sync(0xffffffffu, sf, o);
          if (lane == 0) sd[(comp - 1) * NSCAL + S_SIGMASQR8] = (double)(sf * (float)(1.0 / (2.0 * (PI * PI))));
        }
      }
    }
    __syncthreads();
    // growth tangents: dy_i = M_i dy_{i-1} + dM_i y_{i-1}, dy_0 = 0, as an
    // FP32 scan of affine maps (A, b), one direction per warp and pass
    const float iyf = 1.f / Yvf[(NGROW - 1) * 2];
    for (int d = warp; d < NDIR; d += 4) {
      float A[4] = {1.f, 0.f, 0.f, 1.f}, b[2] = {0.f, 0.f};
      float Mf[4][4], bf[4][2];
      for (int k = 0; k < 4; ++k) {
        const int i = lane * 4 + k;
#pragma unroll
        for (int q = 0; q < 4; ++q) Mf[k][q] = Mvf[i * 4 + q];
        const float yp0 = i > 0 ? Yvf[(i - 1) * 2] : 0.f, yp1 = i > 0 ? Yvf[(i - 1) * 2 + 1] : 0.f;
        const float* dM = dMv + i * 4 * NDIR + d;
        bf[k][0] = dM[0] * yp0 + dM[NDIR] * yp1;
        bf[k][1] = dM[2 * NDIR] * yp0 + dM[3 * NDIR] * yp1;
        const float a0 = Mf[k][0] * A[0] + Mf[k][1] * A[2], a1 = Mf[k][0] * A[1] + Mf[k][1] * A[3];
        const float a2 = Mf[k][2] * A[0] + Mf[k][3] * A[2], a3 = Mf[k][2] * A[1] + Mf[k][3] * A[3];
        const float b0 = Mf[k][0] * b[0] + Mf[k][1] * b[1] + bf[k][0];
        const float b1 = Mf[k][2] * b[0] + Mf[k][3] * b[1] + bf[k][1];
        A[0] = a0, A[1] = a1, A[2] = a2, A[3] = a3, b[0] = b0, b[1] = b1;
      }
      for (int o = 1; o < 32; o <<= 1) {
        float P[4], p[2];
#pragma unroll
        for (int q = 0; q < 4; ++q) P[q] = __shfl_up_sync(0xffffffffu, A[q], o);
        p[0] = __shfl_up_sync(0xffffffffu, b[0], o);
        p[1] = __shfl_up_sync(0xffffffffu, b[1], o);
        if (lane >= o) {
          // (A, b) after (P, p): x -> A (P x + p) + b
          const float b0 = A[0] * p[0] + A[1] * p[1] + b[0], b1 = A[2] * p[0] + A[3] * p[1] + b[1];
          const float a0 = A[0] * P[0] + A[1] * P[2], a1 = A[0] * P[1] + A[1] * P[3];
          const float a2 = A[2] * P[0] + A[3] * P[2], a3 = A[2] * P[1] + A[3] * P[3];
          A[0] = a0, A[1] = a1, A[2] = a2, A[3] = a3, b[0] = b0, b[1] = b1;
        }
      }
      float x0 = __shfl_up_sync(0xffffffffu, b[0], 1), x1 = __shfl_up_sync(0xffffffffu, b[1], 1);
      if (lane == 0) x0 = 0.f, x1 = 0.f;
      float dy[4];
      for (int k = 0; k < 4; ++k) {
        const float v0 = Mf[k][0] * x0 + Mf[k][1] * x1 + bf[k][0];
        const float v1 = Mf[k][2] * x0 + Mf[k][3] * x1 + bf[k][1];
        x0 = v0, x1 = v1;
        dy[k] = x0;
      }
      const float dyf = __shfl_sync(0xffffffffu, x0, 31);
      for (int k = 0; k < 4; ++k) {
        const int i = lane * 4 + k;
        const float D = Yvf[i * 2] * iyf;
        const float gdv = (dy[k] - D * dyf) * iyf;
        out->gd[d][i] = (double)gdv;
        out->gdF[i][d] = gdv;  // the row stage's copy
      }
    }
  } else if (lane < NDIR) {
    const int d = lane;
    auto gv = [&](const double* arr, int stride, int e) { return mk1(arr[e], arr[(1 + d) * stride + e]); };
    if (warp == 0) {
      // chi prefix sum (scipy/ode.py:21 first step h = 0), then chi[-1] - chi
      D1 y = mk1(0.0, 0.0);
      D1 ys[NCHI];
      ys[0] = y;
      for (int i = 1; i < NCHI; ++i) {
        const double hh = c->lna_chi[i] - c->lna_chi[i - 1];
        const D1 fmv = gv(fm, NCHI, i);
        y = y + 1.0 / 6.0 * hh * (gv(fn, NCHI, i - 1) + 2 * fmv + 2 * fmv + gv(fn, NCHI, i));
        ys[i] = y;
      }
      for (int i = 0; i < NCHI; ++i) {
        const D1 v = ys[NCHI - 1] - ys[i];
        if (d == 0) out->chiv[i] = v.v;
        out->chid[d][i] = v.d[0];
      }
    } else if (warp == 1) {
      // growth RK4 in a (background.py:108-111)
      const double* QA = qr;
      const double* RA = qr + (NDIR + 1) * NGROW;
      const double* QM = qr + 2 * (NDIR + 1) * NGROW;
      const double* RM = qr + 3 * (NDIR + 1) * NGROW;
      D1 y0 = mk1(c->atab_grow[0], 0.0), y1 = mk1(1.0, 0.0);
      D1 ys[NGROW];
      ys[0] = y0;
      for (int i = 1; i < NGROW; ++i) {
        const double hh = c->atab_grow[i] - c->atab_grow[i - 1];
        const D1 qa0 = gv(QA, NGROW, i - 1), ra0 = gv(RA, NGROW, i - 1);
        const D1 qm = gv(QM, NGROW, i), rm = gv(RM, NGROW, i);
        const D1 qa1 = gv(QA, NGROW, i), ra1 = gv(RA, NGROW, i);
        const D1 k1a = y1, k1b = -qa0 * y1 + ra0 * y0;
        const D1 y0b = y0 + hh * k1a / 2, y1b = y1 + hh * k1b / 2;
        const D1 k2a = y1b, k2b = -qm * y1b + rm * y0b;
        const D1 y0c = y0 + hh * k2a / 2, y1c = y1 + hh * k2b / 2;
        const D1 k3a = y1c, k3b = -qm * y1c + rm * y0c;
        const D1 y0d = y0 + hh * k3a, y1d = y1 + hh * k3b;
        const D1 k4a = y1d, k4b = -qa1 * y1d + ra1 * y0d;
        y0 = y0 + 1.0 / 6.0 * hh * (k1a + 2 * k2a + 2 * k3a + k4a);
        y1 = y1 + 1.0 / 6.0 * hh * (k1b + 2 * k2b + 2 * k3b + k4b);
        ys[i] = y0;
      }
      for (int i = 0; i < NGROW; ++i) {
        const D1 v = ys[i] / y0;
        if (d == 0) out->gv[i] = v.v;
        out->gd[d][i] = v.d[0];
      }
    } else if (warp == 2) {
      // romb combination (scipy/integrate.py:131-159), divmax = 7
      const double a = -4.0, b = 3.0, intrange = b - a;
      D1 ordsum = 0.5 * (gv(fr, NROMB, 0) + gv(fr, NROMB, 1));
      D1 state[8];
      for (int i = 0; i < 8; ++i) state[i] = intrange * ordsum;
      int pos = 2;
      for (int lev = 1; lev <= 7; ++lev) {
        const int n = 1 << lev, numtosum = n / 2;
        D1 sum = mk1(0.0, 0.0);
        for (int m = 0; m < numtosum; ++m) sum = sum + gv(fr, NROMB, pos + m);
        pos += numtosum;
        ordsum = ordsum + sum;
        D1 x = intrange * ordsum / (double)n;
        D1 ns[8];
        ns[0] = x;
        for (int kk = 0; kk < 7; ++kk) {
          const double tmp = ldexp(1.0, 2 * (kk + 1));
          x = (tmp * x - state[kk]) / (tmp - 1.0);
          ns[kk + 1] = x;
        }
        for (int i = 0; i < 8; ++i) state[i] = ns[i];
      }
      const D1 sig8 = 1.0 / (2.0 * (PI * PI)) * state[7];
      const D1 s8 = mk1(sv[S_SIGMA8], sd[d * NSCAL + S_SIGMA8]);
      const D1 pkn = (s8 * s8) / sig8;
      if (d == 0) {
        sv[S_SIGMASQR8] = sig8.v;
        sv[S_PKNORM] = pkn.v;
      }
      sd[d * NSCAL + S_SIGMASQR8] = sig8.d[0];
      sd[d * NSCAL + S_PKNORM] = pkn.d[0];
    }
  }
  __syncthreads();
  if (F32T && t < NDIR) {
    // P(k) normalisation sigma8^2 / sigmasqr(8) (power.py:47)
    const D1 s8 = mk1(sv[S_SIGMA8], sd[dir * NSCAL + S_SIGMA8]);
    const D1 pkn = (s8 * s8) / mk1(sv[S_SIGMASQR8], sd[dir * NSCAL + S_SIGMASQR8]);
    __syncwarp(0xffu);
    if (dir == 0) sv[S_PKNORM] = pkn.v;
    sd[dir * NSCAL + S_PKNORM] = pkn.d[0];
  }
  if (t < NDIR) {
    // growth_factor(1.0)
    const int2 sg = interp_segment_inc(1.0, c->atab_grow, NGROW, NGROW - 1);
    D1 g1 = interp_d1(1.0, c->atab_grow, out->gv, out->gd[dir], sg);
    g1 = xfmin(xfmax(g1, 0.0), 1.0);
    if (dir == 0) g1s[0] = g1.v;
    g1s[1 + dir] = g1.d[0];
  }
  __syncthreads();
  for (int i = 0; i < NSCAL; ++i) sD[i] = mk1(sv[i], sd[dir * NSCAL + i]);
  const D1 g1 = mk1(g1s[0], g1s[1 + dir]);
  // P(k_i, a = 1) k_i^3 and pk3 / (2 pi^2) on the halofit grid
  if (!F32T) {
    for (int e = it; e < NKH; e += 32) {
      const double k = c->kh[e];
      const D1 p3 = pk_linearT<NW>(sD, k, c->logk[e], g1) * c->kh3[e];
      if (dir == 0) out->pk3v[e] = p3.v;
      out->pk3d[dir][e] = p3.d[0];
      put(pq, NKH, e, p3 / (2.0 * (PI * PI)));
    }
  } else {
    // the node values exp(n_s ln k) T(k)^2 from grad_nodes_kernel, in
    // pk_linearT's order: ((u g^2) pknorm), then k^3
    const FF8 g1f = ff8_of(g1s[0], g1s + 1, 1);
    const FF8 g1sq = g1f * g1f;
    const FF8 pkn = ff8_of(sv[S_PKNORM], sd + S_PKNORM, NSCAL);
    const double* gu = gb.gnode + (size_t)item * GNODE_STRIDE + GNODE_U;
    for (int e = t; e < NKH; e += blockDim.x) {
      const FF8 u = ff8_packed(gu, NKH, e);
      const FF8 p3 = ((u * g1sq) * pkn) * c->kh3[e];
      out->pk3v[e] = val(p3);
      float4* pd = reinterpret_cast<float4*>(&out->pk3df[e][0]);
      pd[0] = make_float4(p3.d[0], p3.d[1], p3.d[2], p3.d[3]);
      pd[1] = make_float4(p3.d[4], p3.d[5], p3.d[6], p3.d[7]);
    }
  }
  if (F32T && t < NDIR + 1) {
    // the Limber kernels' FP32 Eisenstein-Hu inputs and their tangents,
    // once per cosmology: t 0 the values, t 1..8 direction t - 1
    const int d = t - 1;
    const double keq = sv[S_K_EQ], sh = sv[S_SH_D], bc = sv[S_BETA_C], ac = sv[S_ALPHA_C];
    const double ks = sv[S_K_SILK];
    if (t == 0) {
      const double qinv = 1.0 / (13.41 * keq);
      float* ev = out->ehv;
      ev[0] = (float)qinv;
      ev[1] = (float)log2(qinv);
      ev[2] = (float)sh;
      ev[3] = (float)(1.0 / sh);
      ev[4] = (float)(1.8 * bc);
      ev[5] = (float)(14.2 / ac);
      ev[6] = (float)sv[S_ALPHA_B];
      ev[7] = (float)sv[S_BETA_B];
      ev[8] = (float)sv[S_BETA_NODE];
      ev[9] = (float)log2(ks);
      ev[10] = (float)sv[S_FB];
      ev[11] = (float)sv[S_FC];
      ev[12] = (float)(sv[S_NS] + 3.0);
      ev[13] = (float)(1.0 / keq);
      ev[14] = (float)sv[S_AGAM];
      ev[15] = (float)sv[S_NWQ];
    } else {
      const double* sdd = sd + d * NSCAL;
      float* et = out->eht;
      for (int j = 0; j < NET; ++j) et[j * NDIR + d] = 0.f;
      et[E_KEQ * NDIR + d] = (float)sdd[S_K_EQ];
      et[E_SH * NDIR + d] = (float)sdd[S_SH_D];
      et[E_C18BC * NDIR + d] = (float)(1.8 * sdd[S_BETA_C]);
      et[E_C142AC * NDIR + d] = (float)(-14.2 * sdd[S_ALPHA_C] / (ac * ac));
      et[E_ALPHAB * NDIR + d] = (float)sdd[S_ALPHA_B];
      et[E_BETAB * NDIR + d] = (float)sdd[S_BETA_B];
      et[E_BETANODE * NDIR + d] = (float)sdd[S_BETA_NODE];
      et[E_LG2KSILK * NDIR + d] = (float)(sdd[S_K_SILK] / (ks * 0.6931471805599453));
      et[E_FB * NDIR + d] = (float)sdd[S_FB];
      et[E_FC * NDIR + d] = (float)sdd[S_FC];
      et[E_NS3 * NDIR + d] = (float)sdd[S_NS];
      if (sv[S_TFNW] != 0.0) {  // type "eisenhu": its two inputs in the slots of k_eq and 1.8 beta_c
        et[E_AGAM * NDIR + d] = (float)sdd[S_AGAM];
        et[E_NWQ * NDIR + d] = (float)sdd[S_NWQ];
      }
    }
  }
  __syncthreads();
  // fp32c: the Taylor tables and sigma^2(R) follow in grad_moments32_kernel
  const double dx = (c->logk[NKH - 1] - c->logk[0]) / 256;
  for (int e = F32T ? (NDIR + 1) * NRT : t; e < (NDIR + 1) * NRT; e += blockDim.x) {
    const int comp = e / NRT, j = e % NRT;
    const double* w = pq + comp * NKH;
    double acc = 0.0;
    for (int m = 0; m < 128; ++m) {
      const double y0 = w[2 * m] * c->E[(2 * m) * NRT + j];
      const double y1 = w[2 * m + 1] * c->E[(2 * m + 1) * NRT + j];
      const double y2 = w[2 * m + 2] * c->E[(2 * m + 2) * NRT + j];
      acc += y0 + 4 * y1 + y2;
    }
    if (comp == 0) out->sigv[j] = dx / 3 * acc;
    else out->sigd[comp - 1][j] = dx / 3 * acc;
  }
  for (int i = t; i < NSCAL; i += blockDim.x) {
    out->sv[i] = sv[i];
    for (int d = 0; d < NDIR; ++d) out->sd[d][i] = sd[d * NSCAL + i];
  }
  if (F32T) {
    // float-pair copies for the row stage
    for (int i = t; i < NSCAL; i += blockDim.x) {
      const FF v = ff_of(sv[i]);
      out->svF[i] = make_float2(v.hi, v.lo);
      for (int d = 0; d < NDIR; ++d) out->sdF[i][d] = (float)sd[d * NSCAL + i];
    }
    // (the FP32 chi tables, slopes and the row stage's copies come from the scans)
  }
}

// fp32c: the tables of the moments that grad_rows32_kernel reads, from the
// P(k) k^3 table grad_tables_kernel wrote (pk3v, pk3df), one CTA of NRT
// threads per cosmology, at full occupancy (the serial recurrences of one
// cosmology overlap with other cosmologies' work):
//   Taylor tables, scaled to the table row so that no power of k overflows.
//   Values: float pairs R_m[i] = c_m Q_m[i], c_m = (-1)^m / m!,
//   Q_m[i] = sum_{k < i} w_k q3_k (kh_k / kh_i)^(2(m+1)) (one lane per m);
//   tangents (FP32, one thread per (m, d)): sum_{k < i} w_k dq3_k
//   (kh_k / kh_i)^(2(m+1)).  Both by the contracting recurrence
//   Q_m[i+1] = (Q_m[i] + w_i q3_i) (kh_i / kh_{i+1})^(2(m+1)),
//   kh_i = exp(ln 1e-4 + i dlnk);
//   sigma^2(R_j) without g^2 (power.py:98-111): value in float-pair
//   arithmetic (as cosmo_tables' fp32c sums), tangents FP32, one thread per j.
// q3 = P(k) k^3 / (2 pi^2), w the Simpson weights.
static_assert(NRT == 256, "one thread per sigma^2(R) node");
__global__ void __launch_bounds__(NRT) grad_moments32_kernel(GradBatch gb, const ConstTables* __restrict__ c) {
  const int item = blockIdx.x;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  TabD* out = gi.tab;
  __shared__ __align__(16) float2 wq[NKH];          // w q3 as float pairs
  __shared__ __align__(16) float wqd[NKH][NDIR];    // w dq3 (rows read as float4)
  const int t = threadIdx.x;
  constexpr double INV2PI2 = 1.0 / (2.0 * (PI * PI));
  for (int i = t; i < NKH + 15; i += blockDim.x) {
    float hi = 0.f;
    if (i < NKH) {
      const double sw = c->simpson_kh[i] * INV2PI2;
      const FF w = ff_of(sw * out->pk3v[i]);
      wq[i] = make_float2(w.hi, w.lo);
      hi = w.hi;
      const float swf = (float)sw;
#pragma unroll
      for (int d = 0; d < NDIR; ++d) wqd[i][d] = swf * out->pk3df[i][d];
    }
    out->wq3f[i] = hi;
  }
  __syncthreads();
  if (gi.ptt) {
    float2* pv = reinterpret_cast<float2*>(gi.ptt);  // [NKH + 1][NTAYLOR]
    float* pdv = ptt_tangents(gi.ptt);
    if (t < NTAYLOR) {
      const int m = t;
      FF rho, cm, q;
      rho.hi = c->tay_rho[m][0], rho.lo = c->tay_rho[m][1];
      cm.hi = c->tay_c[m][0], cm.lo = c->tay_c[m][1];
      q.hi = 0.f, q.lo = 0.f;
      pv[m] = make_float2(0.f, 0.f);
      for (int i = 0; i < NKH; ++i) {
        FF w;
        w.hi = wq[i].x, w.lo = wq[i].y;
        q = ff_mul(ff_add(q, w), rho);
        const FF r = ff_mul(cm, q);
        pv[(size_t)(i + 1) * NTAYLOR + m] = make_float2(r.hi, r.lo);
      }
    } else if (t >= 32 && t < 32 + NTAYLOR * NDIR) {
      const int job = t - 32, m = job / NDIR, d = job % NDIR;
      const float rho = c->tay_rho[m][0];
      float acc = 0.f;
      pdv[(size_t)m * NDIR + d] = 0.f;
      for (int i = 0; i < NKH; ++i) {
        acc = (acc + wqd[i][d]) * rho;
        pdv[((size_t)(i + 1) * NTAYLOR + m) * NDIR + d] = acc;
      }
    }
  }
  {
    const int j = t;
    float ah = 0.f, al = 0.f;
    float ad[NDIR];
#pragma unroll
    for (int d = 0; d < NDIR; ++d) ad[d] = 0.f;
#pragma unroll 4
    for (int i = 0; i < NKH; ++i) {
      const float2 e = c->Eff[i * NRT + j];
      ff_acc_prod(ah, al, wq[i], e);
      const float4 q0 = *reinterpret_cast<const float4*>(&wqd[i][0]);
      const float4 q1 = *reinterpret_cast<const float4*>(&wqd[i][4]);
      ad[0] = fmaf(q0.x, e.x, ad[0]);
      ad[1] = fmaf(q0.y, e.x, ad[1]);
      ad[2] = fmaf(q0.z, e.x, ad[2]);
      ad[3] = fmaf(q0.w, e.x, ad[3]);
      ad[4] = fmaf(q1.x, e.x, ad[4]);
      ad[5] = fmaf(q1.y, e.x, ad[5]);
      ad[6] = fmaf(q1.z, e.x, ad[6]);
      ad[7] = fmaf(q1.w, e.x, ad[7]);
    }
    out->sigv[j] = (double)ah + (double)al;
    const FF sv = ff_two_sum(ah, al);
    out->sigF[j] = make_float2(sv.hi, sv.lo);
#pragma unroll
    for (int d = 0; d < NDIR; ++d) {
      out->sigd[d][j] = (double)ad[d];
      out->sigdF[j][d] = ad[d];
    }
  }
}

size_t grad_tables_smem(bool f32t) {
  static_assert(4 * NGROW >= NKH, "P(k) k^3 staging aliases the growth coefficients");
  if (f32t) return sizeof(double) * (NSCAL * (1 + NDIR) + GNODE_U + NDIR + 1);
  return sizeof(double) * (NSCAL * (1 + NDIR) + (NDIR + 1) * (2 * NCHI + 4 * NGROW + NROMB + 1));
}

// ----------------------------------------------------------- dual rows -----
// FP64 Jacobian rows.  One warp per 4 Limber nodes: lane = 8 * node slot +
// tangent direction.
//   prelude (per lane, Dual<1>): growth, chi, the root find (index from the
//     values with the forward's arithmetic, tangent through the interpolation
//     formula), R = 1 / k_nl;
//   moments (power.py:121-139), node by node over all 32 lanes, as scalar sums
//     with their R-derivatives and their P(k) k^3 tangents:
//       S1 = sum w q3 2 y^2 e^{-y^2},  S2 = sum w q3 4 (y^2 - y^4) e^{-y^2},
//       y = k R, q3 = P(k) k^3 / (2 pi^2);  dS = S_q3[d] + dS/dR dR[d];
//     every term with y^2 <= 60 (the rest is below 1e-20 of the sums);
//   epilogue (per lane, Dual<1>): n_eff, C, takahashi2012 coefficients, the
//     Limber weight; rows out.
__global__ void __launch_bounds__(256) grad_rows_kernel(GradBatch gb, const ConstTables* __restrict__ c) {
  const int item = blockIdx.y;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const GeoHeader* geo = gi.geo;
  const int na = geo->na;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = lane >> 3, dir = lane & 7;
  const int n_first = (blockIdx.x * 8 + warp) * 4;
  if (n_first >= na) return;
  const int n_raw = n_first + slot;
  const bool live = n_raw < na;
  const int n = live ? n_raw : na - 1;  // dead slots evaluate a valid node, write nothing
  const TabD* tb = gi.tab;
  const double* A = geo_ptr<double>(geo, geo->off_a);
  const double* WS = geo_ptr<double>(geo, geo->off_wsimp);
  const int64_t* SC = geo_ptr<int64_t>(geo, geo->off_seg_chi);
  const int64_t* SG = geo_ptr<int64_t>(geo, geo->off_seg_grow);
  const double a = A[n];
  D1 g = interp_d1(a, c->atab_grow, tb->gv, tb->gd[dir], unpack_seg(SG[n]));
  g = xfmin(xfmax(g, 0.0), 1.0);
  D1 chi = interp_d1(a, c->atab_chi, tb->chiv, tb->chid[dir], unpack_seg(SC[n]));
  chi = xfmax(chi, 0.0);
  const D1 g2 = g * g;
  int ind, j2;
  if (gb.seg_in) {
    // the segment of another parameter point: differentiate on its branch
    const int pk = gb.seg_in[(size_t)item * na + n];
    ind = min(max(pk & 0xffff, 1), NRT - 2);
    j2 = ind + ((pk >> 16) ? 1 : -1);
  } else {
    int best;
    int lo = 0, hi = NRT;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (tb->sigv[mid] * g2.v > 1.0) lo = mid + 1;
      else hi = mid;
    }
    const int cc = lo;
    best = cc < NRT ? cc : NRT - 1;
    if (cc >= 1) {
      const double dlo = 1.0 - tb->sigv[cc - 1] * g2.v;
      if (cc < NRT) {
        const double dhi = 1.0 - tb->sigv[cc] * g2.v;
        best = (dlo * dlo <= dhi * dhi) ? cc - 1 : cc;
      } else {
        best = cc - 1;
      }
    }
    ind = best < 1 ? 1 : (best > NRT - 2 ? NRT - 2 : best);
    const double xpi = tb->sigv[ind] * g2.v;
    const double xc = fmin(fmax(1.0, tb->sigv[1] * g2.v), tb->sigv[NRT - 2] * g2.v);
    j2 = ind + ((xc - xpi >= 0.0) ? 1 : -1);
  }
  if (gb.seg_out && live && dir == 0) gb.seg_out[(size_t)item * na + n] = ind | ((j2 > ind ? 1 : 0) << 16);
  const D1 xp0 = mk1(tb->sigv[ind], tb->sigd[dir][ind]) * g2;
  const D1 xp1 = mk1(tb->sigv[j2], tb->sigd[dir][j2]) * g2;
  const D1 slope = (c->logr[j2] - c->logr[ind]) / (xp1 - xp0);
  const D1 bb = c->logr[ind] - slope * xp0;
  const D1 root = slope * 1.0 + bb;
  const D1 R = xfmax(xexp(root), 1e-6);
  const D1 knl = 1.0 / R;
  const D1 inv = 1.0 / knl;
  const int ilo = 0, ihi = NKH - 1;
  // explicit terms, node by node over the warp
  double m_s1 = 0, m_s2 = 0, m_s1r = 0, m_s2r = 0, m_s1d = 0, m_s2d = 0;
  const double q3s = 1.0 / TWO_PI2_G;
  for (int q = 0; q < 4; ++q) {
    const double Rq = __shfl_sync(0xffffffffu, inv.v, q * 8);
    const int lo = __shfl_sync(0xffffffffu, ilo, q * 8), hi = __shfl_sync(0xffffffffu, ihi, q * 8);
    const double iRq = 1.0 / Rq;
    double s1 = 0, s2 = 0, s1r = 0, s2r = 0, s1d[NDIR], s2d[NDIR];
#pragma unroll
    for (int d = 0; d < NDIR; ++d) s1d[d] = s2d[d] = 0.0;
    for (int i = lo + lane; i <= hi; i += 32) {
      const double y = c->kh[i] * Rq;
      const double y2 = y * y;
      if (y2 > Y2_SKIP) continue;
      const double E = exp(-y2);
      const double wq = c->simpson_kh[i] * E * q3s;
      const double Av = wq * tb->pk3v[i];
      const double c1 = 2.0 * y2, c2 = 4.0 * (y2 - y2 * y2);
      s1 += Av * c1;
      s2 += Av * c2;
      s1r += 4.0 * Av * y2 * (1.0 - y2) * iRq;
      s2r += 8.0 * Av * y2 * (1.0 - 3.0 * y2 + y2 * y2) * iRq;
      const double w1 = wq * c1, w2 = wq * c2;
#pragma unroll
      for (int d = 0; d < NDIR; ++d) {
        const double p = tb->pk3d[d][i];
        s1d[d] += w1 * p;
        s2d[d] += w2 * p;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      s1r += __shfl_xor_sync(0xffffffffu, s1r, o);
      s2r += __shfl_xor_sync(0xffffffffu, s2r, o);
#pragma unroll
      for (int d = 0; d < NDIR; ++d) {
        s1d[d] += __shfl_xor_sync(0xffffffffu, s1d[d], o);
        s2d[d] += __shfl_xor_sync(0xffffffffu, s2d[d], o);
      }
    }
    if (slot == q) {
      m_s1 = s1;
      m_s2 = s2;
      m_s1r = s1r;
      m_s2r = s2r;
#pragma unroll
      for (int d = 0; d < NDIR; ++d)
        if (d == dir) {
          m_s1d = s1d[d];
          m_s2d = s2d[d];
        }
    }
  }
  // moments with their tangents in this lane's direction, times g^2
  const D1 S1 = mk1(m_s1, m_s1d + m_s1r * inv.d[0]);
  const D1 S2 = mk1(m_s2, m_s2d + m_s2r * inv.d[0]);
  const D1 I1 = S1 * g2, I2 = S2 * g2;

  const D1 neff = I1 - 3.0;
  const D1 C = I1 * I1 + I2;
  // coefficients (power.py:177-238)
  D1 sD[NSCAL];
  for (int i = 0; i < NSCAL; ++i) sD[i] = mk1(tb->sv[i], tb->sd[dir][i]);
  const BgT<D1> bg = make_bgT(sD);
  const double lna = log(a);
  D1 om_m, om_de;
  omT(bg, a, lna, om_m, om_de);
  const D1 w = wT(bg, a);
  const HfCoef<D1> hc = hf_coefs<D1>(pk_model(gi.geo->physics), neff, C, om_m, om_de, w);
  D1 outv[NA_IN];
  outv[A_CHIC] = xfmax(chi, 1.0);
  outv[A_G] = g;
  outv[A_KNL] = knl;
  outv[A_BETA] = hc.beta;
  outv[A_ALPHA] = hc.alpha;
  outv[A_AN] = hc.an;
  outv[A_BN] = hc.bn;
  outv[A_LCF3] = hc.lcf3;
  outv[A_F1] = hc.f1;
  outv[A_F2] = hc.f2;
  outv[A_GAM] = hc.gam;
  outv[A_NU] = hc.nu;
  outv[A_MU] = hc.mu;
  const D1 dchi = dchioverdaT(bg, a, lna);
  outv[A_U] = WS[n] * dchi / xfmax(chi * chi, 1.0) / C2_G;
  if (live) {
    if (gb.precision == JCG_FP64) {
      double* row = gi.rowd + (size_t)n * NROWD;
      for (int i = 0; i < NA_IN; ++i) {
        if (dir == 0) row[i] = outv[i].v;
        row[NA_IN * (1 + dir) + i] = outv[i].d[0];
      }
    } else {
      // FP32 row: values in the forward row's units, tangents of the inputs
      constexpr double LOG2E = 1.4426950408889634;
      float* row = gi.rowg + (size_t)n * NROWG;
      const D1 chic = outv[A_CHIC], kn = outv[A_KNL];
      const D1 d2fac = outv[A_G] * outv[A_G] * sD[S_PKNORM] / TWO_PI2_G;
      if (dir == 0) {
        row[F_INVCHI] = (float)(1.0 / chic.v);
        row[F_LG2INVCHI] = (float)(-log2(chic.v));
        row[F_CHIC] = (float)chic.v;
        row[F_LG2KNL] = (float)log2(kn.v);
        row[F_INVKNL] = (float)(1.0 / kn.v);
        row[F_D2FAC] = (float)d2fac.v;
        row[F_BETAN] = (float)outv[A_BETA].v;
        row[F_ALPHAN] = (float)outv[A_ALPHA].v;
        row[F_AN] = (float)outv[A_AN].v;
        row[F_3F1] = (float)(3.0 * outv[A_F1].v);
        row[F_F2] = (float)outv[A_F2].v;
        row[F_BN] = (float)outv[A_BN].v;
        row[F_LG2CF3] = (float)(LOG2E * outv[A_LCF3].v);
        row[F_3MGAMMA] = (float)(3.0 - outv[A_GAM].v);
        row[F_NUN] = (float)outv[A_NU].v;
        row[F_MUN] = (float)outv[A_MU].v;
        row[F_U] = (float)outv[A_U].v;
      }
      float* tg = row + NROWV;
      tg[T_CHIC * NDIR + dir] = (float)chic.d[0];
      tg[T_D2FAC * NDIR + dir] = (float)d2fac.d[0];
      tg[T_KNL * NDIR + dir] = (float)kn.d[0];
      tg[T_BETAN * NDIR + dir] = (float)outv[A_BETA].d[0];
      tg[T_ALPHAN * NDIR + dir] = (float)outv[A_ALPHA].d[0];
      tg[T_AN * NDIR + dir] = (float)outv[A_AN].d[0];
      tg[T_3F1 * NDIR + dir] = (float)(3.0 * outv[A_F1].d[0]);
      tg[T_F2 * NDIR + dir] = (float)outv[A_F2].d[0];
      tg[T_BN * NDIR + dir] = (float)outv[A_BN].d[0];
      tg[T_LG2CF3 * NDIR + dir] = (float)(LOG2E * outv[A_LCF3].d[0]);
      tg[T_3MG * NDIR + dir] = (float)(-outv[A_GAM].d[0]);
      tg[T_NUN * NDIR + dir] = (float)outv[A_NU].d[0];
      tg[T_MUN * NDIR + dir] = (float)outv[A_MU].d[0];
      tg[T_U * NDIR + dir] = (float)outv[A_U].d[0];
    }
  }
}

// ------------------------------------------------------- fp32c rows -------
__device__ __forceinline__ F8 interp_f8(double x, const double* xp, const double* fv, const double* fd,
                                        int stride, int2 sg) {
  const F8 f0 = f8_of(fv[sg.x], fd + sg.x, stride), f1 = f8_of(fv[sg.y], fd + sg.y, stride);
  const F8 a = (f1 - f0) / (xp[sg.y] - xp[sg.x]);
  const F8 b = f0 - a * xp[sg.x];
  return a * x + b;
}

// fp32c Jacobian rows: one node per thread in DualF<8> (value FP64, the 8
// tangents FP32), the same operations as grad_rows_kernel's FP32C path: root
// find, moments (exp terms for y^2 in [1, 60], Taylor prefix tables below),
// takahashi2012 coefficients, Limber weight; the row is written as computed.
// interpolation on the segment sg of a table with tangents, by the segment's
// node-spacing reciprocal ida (no float64 division)
// float value with 8 float tangents (the row stage's halofit coefficients,
// which the Limber integrand consumes as float)
struct S8 {
  float v;
  float d[NDIR];
};
__device__ __forceinline__ S8 s8_of(const FF8& x) {
  S8 r;
  r.v = x.v.hi;
#pragma unroll
  for (int d = 0; d < NDIR; ++d) r.d[d] = x.d[d];
  return r;
}
__device__ __forceinline__ S8 s8_scale(const S8& x, float c) {
  S8 r;
  r.v = c * x.v;
#pragma unroll
  for (int d = 0; d < NDIR; ++d) r.d[d] = c * x.d[d];
  return r;
}
__device__ __forceinline__ S8 s8_ex2(const S8& x) {  // 2^x
  S8 r;
  r.v = ex2f(x.v);
  const float s = r.v * LN2_F;
#pragma unroll
  for (int d = 0; d < NDIR; ++d) r.d[d] = s * x.d[d];
  return r;
}
__device__ __forceinline__ S8 s8_lg2(const S8& x) {  // log2 x
  S8 r;
  r.v = lg2f(x.v);
  const float s = LOG2E_F * rcpf(x.v);
#pragma unroll
  for (int d = 0; d < NDIR; ++d) r.d[d] = s * x.d[d];
  return r;
}
__device__ __forceinline__ void put_s8(float* tg, int slot, const S8& x, float sc) {
#pragma unroll
  for (int d = 0; d < NDIR; ++d) tg[slot * NDIR + d] = x.d[d] * sc;
}

__device__ __forceinline__ FF8 interp_ff8(FF x, const float2* xp, const float2* ida, const float2* fv,
                                         const float (*fd)[NDIR], int2 sg) {
  const FF8 f0 = ff8_of(fv[sg.x], fd[sg.x]), f1 = ff8_of(fv[sg.y], fd[sg.y]);
  const FF iv = f2ff(ida[min(sg.x, sg.y)]);
  const FF inv = sg.y > sg.x ? iv : -iv;
  return f0 + (f1 - f0) * (inv * (x - f2ff(xp[sg.x])));
}

constexpr int GR32_THREADS = 256;  // nodes of one cosmology per CTA (its tables shared in L1)

// Uniform batches: one flat index over (cosmology, node), so that no CTA is
// left with a node or two of a cosmology (na = 2^k + 1); listed: a 2-D grid.
__global__ void __launch_bounds__(GR32_THREADS, 2) grad_rows32_kernel(GradBatch gb, const ConstTables* __restrict__ c) {
  int item, n;
  if (!gb.listed) {
    const long long idx = (long long)blockIdx.x * GR32_THREADS + threadIdx.x;
    item = (int)(idx / gb.na);
    n = (int)(idx - (long long)item * gb.na);
  } else {
    item = blockIdx.y;
    n = blockIdx.x * GR32_THREADS + threadIdx.x;
  }
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const GeoHeader* geo = gi.geo;
  const int na = geo->na;
  if (n >= na) return;
  const TabD* tb = gi.tab;
  const double* A = geo_ptr<double>(geo, geo->off_a);
  const double* WS = geo_ptr<double>(geo, geo->off_wsimp);
  const int64_t* SC = geo_ptr<int64_t>(geo, geo->off_seg_chi);
  const int64_t* SG = geo_ptr<int64_t>(geo, geo->off_seg_grow);
  const double a = A[n];
  const FF aF = ff_of(a);
  float* row = gi.rowg + (size_t)n * NROWG;
  float* tg = row + NROWV;
  auto put_t = [&](int slot, const FF8& x, float sc) {
#pragma unroll
    for (int d = 0; d < NDIR; ++d) tg[slot * NDIR + d] = x.d[d] * sc;
  };
  FF8 g = interp_ff8(aF, c->grow_a_ff, c->grow_ida_ff, tb->gF, tb->gdF, unpack_seg(SG[n]));
  g = xfmin(xfmax(g, 0.0), 1.0);
  FF8 chi = interp_ff8(aF, c->atab_chi_ff, c->chi_ida_ff, tb->chiF, tb->chidF, unpack_seg(SC[n]));
  chi = xfmax(chi, 0.0);
  const FF8 g2 = g * g;
  const double g2v = val(g2);
  int best;
  {
    int lo = 0, hi = NRT;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (tb->sigv[mid] * g2v > 1.0) lo = mid + 1;
      else hi = mid;
    }
    const int cc = lo;
    best = cc < NRT ? cc : NRT - 1;
    if (cc >= 1) {
      const double dlo = 1.0 - tb->sigv[cc - 1] * g2v;
      if (cc < NRT) {
        const double dhi = 1.0 - tb->sigv[cc] * g2v;
        best = (dlo * dlo <= dhi * dhi) ? cc - 1 : cc;
      } else {
        best = cc - 1;
      }
    }
  }
  const int ind = best < 1 ? 1 : (best > NRT - 2 ? NRT - 2 : best);
  const double xpi = tb->sigv[ind] * g2v;
  const double xc = fmin(fmax(1.0, tb->sigv[1] * g2v), tb->sigv[NRT - 2] * g2v);
  const int j2 = ind + ((xc - xpi >= 0.0) ? 1 : -1);
  const FF8 xp0 = ff8_of(tb->sigF[ind], tb->sigdF[ind]) * g2;
  const FF8 xp1 = ff8_of(tb->sigF[j2], tb->sigdF[j2]) * g2;
  const FF8 slope = (f2ff(c->logr_ff[j2]) - f2ff(c->logr_ff[ind])) / (xp1 - xp0);
  const FF8 bb = f2ff(c->logr_ff[ind]) - slope * xp0;
  const FF8 root = slope * 1.0 + bb;
  const FF8 R = xfmax(xexp(root), 1e-6);
  const FF8 knl = 1.0 / R;
  const FF8 inv = 1.0 / knl;
  row[F_LG2KNL] = (ff_log(knl.v) * ffc(1.4426950408889634)).hi;
  row[F_INVKNL] = inv.v.hi;
  put_t(T_KNL, knl, 1.f);
  // moments: the exp terms for y^2 in [Y2_TAYLOR, Y2_SKIP] in FP32 from a
  // float-pair y^2 (values summed in float pairs), below Y2_TAYLOR the Taylor
  // series from the float-pair tables (Horner with derivatives); the
  // derivatives with respect to R and the tangents in FP32
  const float iR = knl.v.hi;
  const float linv = LN2_F * lg2f(inv.v.hi);
  constexpr float HLY2T = 0.0f, HLY2S = 2.0471425f;  // 0.5 log(Y2_TAYLOR), 0.5 log(Y2_SKIP)
  int ilo = (int)floorf((HLY2T - linv - (float)LOG_KMIN) * (float)(1.0 / DLOGK));
  int ihi = (int)ceilf((HLY2S - linv - (float)LOG_KMIN) * (float)(1.0 / DLOGK));
  ilo = max(0, min(ilo, NKH));
  ihi = max(ilo - 1, min(ihi, NKH - 1));
  const FF R2 = ff_sqr(inv.v);
  constexpr float Q3S = (float)(1.0 / TWO_PI2_G);
  FF s1p, s2p;
  s1p.hi = s1p.lo = s2p.hi = s2p.lo = 0.f;
  float s1r = 0.f, s2r = 0.f;
  float s1d[NDIR], s2d[NDIR];
#pragma unroll
  for (int d = 0; d < NDIR; ++d) s1d[d] = s2d[d] = 0.f;
#pragma unroll 2
  for (int i = ilo; i <= ihi; ++i) {
    const float kh = c->kh2_hi[i];
    const float pp = kh * R2.hi;
    float ee = fmaf(kh, R2.hi, -pp);
    ee = fmaf(kh, R2.lo, ee);
    ee = fmaf(c->kh2_lo[i], R2.hi, ee);
    const float ex = exp_neg_pair(pp, ee);
    const float y2 = pp + ee, om = (1.f - pp) - ee;  // y^2, 1 - y^2
    const float Av = tb->wq3f[i] * ex;
    const float c1 = 2.f * y2, c2 = 4.f * y2 * om;
    FF t;
    t.hi = Av * c1, t.lo = 0.f;
    s1p = ff_add(s1p, t);
    t.hi = Av * c2;
    s2p = ff_add(s2p, t);
    s1r = fmaf(4.f * Av * y2 * om, iR, s1r);
    s2r = fmaf(8.f * Av * y2 * (om - 2.f * y2 + y2 * y2), iR, s2r);
    const float wq = c->simpson_f[i] * Q3S * ex;
    const float w1 = wq * c1, w2 = wq * c2;
    const float4 pa = *reinterpret_cast<const float4*>(&tb->pk3df[i][0]);
    const float4 pb = *reinterpret_cast<const float4*>(&tb->pk3df[i][4]);
    const float p[NDIR] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w};
#pragma unroll
    for (int d = 0; d < NDIR; ++d) {
      s1d[d] = fmaf(w1, p[d], s1d[d]);
      s2d[d] = fmaf(w2, p[d], s2d[d]);
    }
  }
  FF s1 = s1p, s2 = s2p;
  float t1d[NDIR], t2d[NDIR];
#pragma unroll
  for (int d = 0; d < NDIR; ++d) t1d[d] = t2d[d] = 0.f;
  if (ilo > 0) {
    // x = y_ilo^2 = (kh_ilo R)^2, F(x) = sum_m R_m[ilo] x^m: t1 = x F,
    // t2 = t1 + x^2 F', d/dR through dx/dR = 2 x / R
    const float2* T = reinterpret_cast<const float2*>(gi.ptt) + (size_t)ilo * NTAYLOR;
    const float* TD = ptt_tangents(gi.ptt) + (size_t)ilo * NTAYLOR * NDIR;
    FF kk;
    kk.hi = c->kh2_hi[ilo], kk.lo = c->kh2_lo[ilo];
    const FF x = ff_mul(kk, R2);
    FF P, D;
    P.hi = T[NTAYLOR - 1].x, P.lo = T[NTAYLOR - 1].y;
    D.hi = D.lo = 0.f;
    float pf = P.hi, df = 0.f, ddf = 0.f;
    for (int m = NTAYLOR - 2; m >= 0; --m) {
      D = ff_add(ff_mul(D, x), P);
      FF r;
      r.hi = T[m].x, r.lo = T[m].y;
      P = ff_add(ff_mul(P, x), r);
      ddf = fmaf(ddf, x.hi, df);
      df = fmaf(df, x.hi, pf);
      pf = fmaf(pf, x.hi, r.hi);
    }
    const FF t1 = ff_mul(x, P);
    const FF t2 = t1 + ff_mul(ff_mul(x, x), D);
    const float xs = x.hi, dxr = 2.f * xs * iR;
    const float t1r = (pf + xs * df) * dxr;
    const float t2r = (pf + 3.f * xs * df + xs * xs * (2.f * ddf)) * dxr;
    // tangent tables are scaled by kh_ilo^-(2(m+1)): powers of x
    float ps = xs;
    for (int m = 0; m < NTAYLOR - 1; ++m) {
      const float sg = c->tay_c[m][0];
      const float ps1 = ps * xs;
      const float a1 = sg * ps, a2 = sg * ps1;
      ps = ps1;
      const float4 u0 = *reinterpret_cast<const float4*>(TD + m * NDIR);
      const float4 u1 = *reinterpret_cast<const float4*>(TD + m * NDIR + 4);
      const float4 v0 = *reinterpret_cast<const float4*>(TD + (m + 1) * NDIR);
      const float4 v1 = *reinterpret_cast<const float4*>(TD + (m + 1) * NDIR + 4);
      const float dm[NDIR] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
      const float dm1[NDIR] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
#pragma unroll
      for (int d = 0; d < NDIR; ++d) {
        t1d[d] = fmaf(a1, dm[d], t1d[d]);
        t2d[d] = fmaf(a1, dm[d], fmaf(-a2, dm1[d], t2d[d]));
      }
    }
    s1 = s1 + ff_scale2(t1, 2.f);
    s2 = s2 + ff_scale2(t2, 4.f);
    s1r += 2.f * t1r;
    s2r += 4.f * t2r;
  }
  FF8 S1, S2;
  S1.v = s1;
  S2.v = s2;
  const float f1r = s1r, f2r = s2r;
#pragma unroll
  for (int d = 0; d < NDIR; ++d) {
    S1.d[d] = s1d[d] + 2.f * t1d[d] + f1r * inv.d[d];
    S2.d[d] = s2d[d] + 4.f * t2d[d] + f2r * inv.d[d];
  }
  const FF8 I1 = S1 * g2, I2 = S2 * g2;
  const FF8 neff = I1 - 3.0;
  const FF8 C = I1 * I1 + I2;
  // coefficients (power.py:177-238)
  BgT<FF8> bg;
  bg.Om = ff8_of(tb->svF[S_OMEGA_M], tb->sdF[S_OMEGA_M]);
  bg.Ok = ff8_of(tb->svF[S_OMEGA_K], tb->sdF[S_OMEGA_K]);
  bg.Ode = ff8_of(tb->svF[S_OMEGA_DE], tb->sdF[S_OMEGA_DE]);
  bg.w0 = ff8_of(tb->svF[S_W0], tb->sdF[S_W0]);
  bg.wa = ff8_of(tb->svF[S_WA], tb->sdF[S_WA]);
  // E^2(a) and its dark-energy factor once (esqrT, background.py:47-66), in
  // float pairs from ln a and 1 / a; Omega_m(a), Omega_de(a) (omT) and
  // dchi/da (dchioverdaT) from them
  const FF lna = ff_log(aF), ia = ff_rcp(aF), ia2 = ia * ia;
  const FF8 fde = -3.0 * (1.0 + bg.w0 + bg.wa) * lna + 3.0 * bg.wa * (aF - ffc(1.0));
  const FF8 efde = xexp(fde);
  const FF8 esq = bg.Om * (ia2 * ia) + bg.Ok * ia2 + bg.Ode * efde;
  const FF8 om_m = bg.Om * (ia2 * ia) / esq;
  const FF8 om_de = bg.Ode * efde / esq;
  // halofit coefficients (power.py:177-244) in float values with float
  // tangents (S8), the forward fp32c rows' arithmetic (halofit_coefs_fast:
  // the same float expressions, MUFU ex2 / lg2), each stored as soon as it is
  // formed
  const S8 nS = s8_of(neff), Cs = s8_of(C), omm = s8_of(om_m), omde = s8_of(om_de);
  const float nv = nS.v, n2 = nv * nv, n3 = n2 * nv, n4 = n2 * n2, Cv = Cs.v;
  // d/dn of c1 n + c2 n^2 + c3 n^3 + c4 n^4
  auto dpoly = [&](float c1, float c2, float c3, float c4) { return c1 + nv * (2.f * c2 + nv * (3.f * c3 + nv * 4.f * c4)); };
  auto lin = [&](float v, float dn, float dC) {  // value v, tangent dn dneff + dC dC
    S8 r;
    r.v = v;
#pragma unroll
    for (int d = 0; d < NDIR; ++d) r.d[d] = fmaf(dn, nS.d[d], dC * Cs.d[d]);
    return r;
  };
  constexpr float LOG2_10 = 3.321928094887362f, LN10_F = 2.302585092994046f;
  const S8 l2om = s8_lg2(omm);
  if (pk_model(gi.geo->physics) == JCG_PK_SMITH2003) {
    // power.py:182-198, 239-242
    {
      const S8 beta = lin(0.8291f + 0.9854f * nv + 0.3401f * n2, dpoly(0.9854f, 0.3401f, 0.f, 0.f), 0.f);
      row[F_BETAN] = beta.v;
      put_s8(tg, T_BETAN, beta, 1.f);
      const S8 alpha = lin(1.3884f + 0.3700f * nv - 0.1452f * n2, dpoly(0.3700f, -0.1452f, 0.f, 0.f), 0.f);
      row[F_ALPHAN] = alpha.v;
      put_s8(tg, T_ALPHAN, alpha, 1.f);
    }
    {
      const S8 e_an = lin(1.4861f + 1.8369f * nv + 1.6762f * n2 + 0.7940f * n3 + 0.1670f * n4 - 0.6206f * Cv,
                          dpoly(1.8369f, 1.6762f, 0.7940f, 0.1670f), -0.6206f);
      const S8 an = s8_ex2(s8_scale(e_an, LOG2_10));
      row[F_AN] = an.v;
      put_s8(tg, T_AN, an, 1.f);
      const S8 e_bn = lin(0.9463f + 0.9466f * nv + 0.3084f * n2 - 0.9400f * Cv, dpoly(0.9466f, 0.3084f, 0.f, 0.f), -0.9400f);
      const S8 bn = s8_ex2(s8_scale(e_bn, LOG2_10));
      row[F_BN] = bn.v;
      put_s8(tg, T_BN, bn, 1.f);
    }
    {
      // frac = Omega_de / (1 - Omega_m) (power.py:180)
      const float ir = rcpf(1.f - omm.v);
      S8 frac;
      frac.v = omde.v * ir;
#pragma unroll
      for (int d = 0; d < NDIR; ++d) frac.d[d] = (omde.d[d] + frac.v * omm.d[d]) * ir;
      auto mix = [&](float p1, float p2) {  // frac om^p1 + (1 - frac) om^p2
        const S8 x1 = s8_ex2(s8_scale(l2om, p1)), x2 = s8_ex2(s8_scale(l2om, p2));
        S8 r;
        r.v = frac.v * x1.v + (1.f - frac.v) * x2.v;
#pragma unroll
        for (int d = 0; d < NDIR; ++d)
          r.d[d] = fmaf(frac.d[d], x1.v - x2.v, fmaf(frac.v, x1.d[d], (1.f - frac.v) * x2.d[d]));
        return r;
      };
      const S8 f1 = mix(-0.0307f, -0.0732f);
      row[F_3F1] = 3.f * f1.v;
      put_s8(tg, T_3F1, f1, 3.f);
      const S8 f2 = mix(-0.0585f, -0.1423f);
      row[F_F2] = f2.v;
      put_s8(tg, T_F2, f2, 1.f);
      const S8 f3 = mix(0.0743f, 0.0725f);
      const S8 e_cn = lin(-0.2807f + 0.6669f * nv + 0.3214f * n2 - 0.0793f * Cv, dpoly(0.6669f, 0.3214f, 0.f, 0.f),
                          -0.0793f);
      const S8 lg2f3 = s8_lg2(f3);
      S8 lg2cf3;
      lg2cf3.v = LOG2_10 * e_cn.v + lg2f3.v;
#pragma unroll
      for (int d = 0; d < NDIR; ++d) lg2cf3.d[d] = fmaf(LOG2_10, e_cn.d[d], lg2f3.d[d]);
      row[F_LG2CF3] = lg2cf3.v;
      put_s8(tg, T_LG2CF3, lg2cf3, 1.f);
    }
    {
      const S8 gam = lin(0.8649f + 0.2989f * nv + 0.1631f * Cv, 0.2989f, 0.1631f);
      row[F_3MGAMMA] = 3.f - gam.v;
      put_s8(tg, T_3MG, gam, -1.f);
      const S8 nu = s8_ex2(s8_scale(lin(0.9585f + 1.2857f * nv, 1.2857f, 0.f), LOG2_10));
      row[F_NUN] = nu.v;
      put_s8(tg, T_NUN, nu, 1.f);
      const S8 mu = s8_ex2(s8_scale(lin(-3.5442f + 0.1908f * nv, 0.1908f, 0.f), LOG2_10));
      row[F_MUN] = mu.v;
      put_s8(tg, T_MUN, mu, 1.f);
    }
  } else {
    // opw = Omega_de(a) (1 + w(a)), w = w0 + (1 - a) wa (background.py:53)
    const S8 w = s8_of(bg.w0 + (ffc(1.0) - aF) * bg.wa);
    S8 opw;
    opw.v = omde.v * (1.f + w.v);
#pragma unroll
    for (int d = 0; d < NDIR; ++d) opw.d[d] = fmaf(omde.d[d], 1.f + w.v, omde.v * w.d[d]);
    auto with_opw = [&](S8 x, float c) {
      x.v = x.v + c * opw.v;
#pragma unroll
      for (int d = 0; d < NDIR; ++d) x.d[d] = fmaf(c, opw.d[d], x.d[d]);
      return x;
    };
    {
      const S8 beta = lin(2.0379f - 0.7354f * nv + 0.3157f * n2 + 1.2490f * n3 + 0.3980f * n4 - 0.1682f * Cv,
                          dpoly(-0.7354f, 0.3157f, 1.2490f, 0.3980f), -0.1682f);
      row[F_BETAN] = beta.v;
      put_s8(tg, T_BETAN, beta, 1.f);
      S8 alpha = lin(6.0835f + 1.3373f * nv - 0.1959f * n2 - 5.5274f * Cv, dpoly(1.3373f, -0.1959f, 0.f, 0.f), -5.5274f);
      if (alpha.v < 0.f) alpha = s8_scale(alpha, -1.f);  // fabs, the selected branch's tangent
      row[F_ALPHAN] = alpha.v;
      put_s8(tg, T_ALPHAN, alpha, 1.f);
    }
    {
      const S8 e_an = with_opw(lin(1.5222f + 2.8553f * nv + 2.3706f * n2 + 0.9903f * n3 + 0.2250f * n4 - 0.6038f * Cv,
                                   dpoly(2.8553f, 2.3706f, 0.9903f, 0.2250f), -0.6038f), 0.1749f);
      const S8 an = s8_ex2(s8_scale(e_an, LOG2_10));
      row[F_AN] = an.v;
      put_s8(tg, T_AN, an, 1.f);
      const S8 e_bn = with_opw(lin(-0.5642f + 0.5864f * nv + 0.5716f * n2 - 1.5474f * Cv,
                                   dpoly(0.5864f, 0.5716f, 0.f, 0.f), -1.5474f), 0.2279f);
      const S8 bn = s8_ex2(s8_scale(e_bn, LOG2_10));
      row[F_BN] = bn.v;
      put_s8(tg, T_BN, bn, 1.f);
    }
    {
      const S8 e_cn = lin(0.3698f + 2.0404f * nv + 0.8161f * n2 + 0.5869f * Cv, dpoly(2.0404f, 0.8161f, 0.f, 0.f), 0.5869f);
      S8 lg2cf3;
      lg2cf3.v = LOG2_10 * e_cn.v + 0.0743f * l2om.v;
#pragma unroll
      for (int d = 0; d < NDIR; ++d) lg2cf3.d[d] = fmaf(LOG2_10, e_cn.d[d], 0.0743f * l2om.d[d]);
      row[F_LG2CF3] = lg2cf3.v;
      put_s8(tg, T_LG2CF3, lg2cf3, 1.f);
      const S8 f1 = s8_ex2(s8_scale(l2om, -0.0307f));
      row[F_3F1] = 3.f * f1.v;
      put_s8(tg, T_3F1, f1, 3.f);
      const S8 f2 = s8_ex2(s8_scale(l2om, -0.0585f));
      row[F_F2] = f2.v;
      put_s8(tg, T_F2, f2, 1.f);
    }
    {
      const S8 gam = lin(0.1971f - 0.0843f * nv + 0.8460f * Cv, -0.0843f, 0.8460f);
      row[F_3MGAMMA] = 3.f - gam.v;
      put_s8(tg, T_3MG, gam, -1.f);
      const S8 nu = s8_ex2(s8_scale(lin(5.2105f + 3.6902f * nv, 3.6902f, 0.f), LOG2_10));
      row[F_NUN] = nu.v;
      put_s8(tg, T_NUN, nu, 1.f);
      row[F_MUN] = 0.f;
      put_s8(tg, T_MUN, s8_scale(nu, 0.f), 0.f);
    }
  }
  (void)LN10_F;
  constexpr double LOG2E = 1.4426950408889634;
  {
    const FF8 chic = xfmax(chi, 1.0);
    row[F_INVCHI] = ff_rcp(chic.v).hi;
    row[F_LG2INVCHI] = -(ff_log(chic.v) * ffc(LOG2E)).hi;
    row[F_CHIC] = chic.v.hi;
    put_t(T_CHIC, chic, 1.f);
    const FF8 pkn = ff8_of(tb->svF[S_PKNORM], tb->sdF[S_PKNORM]);
    const FF8 d2fac = g * g * pkn / TWO_PI2_G;
    row[F_D2FAC] = d2fac.v.hi;
    put_t(T_D2FAC, d2fac, 1.f);
    const FF8 dchi = (ffc(RH) * ia2) / xsqrt(esq);
    const FF8 u = WS[n] * dchi / xfmax(chi * chi, 1.0) / C2_G;
    row[F_U] = u.v.hi;
    put_t(T_U, u, 1.f);
  }
}

// ------------------------------------------------------ dual radial kernels -
// One warp per node: chi_wl and H on lanes 0-7, the lensing integrand over 32
// lanes in Dual<8> (probes.py:44-51), four tracers per pass.
__global__ void __launch_bounds__(256) grad_kern_kernel(GradBatch gb, const ConstTables* __restrict__ c) {
  const int item = blockIdx.y;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const GeoHeader* geo = gi.geo;
  const int na = geo->na, n_tr = geo->n_tr;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = blockIdx.x * 8 + warp;
  if (n >= na) return;
  const TabD* tb = gi.tab;
  const int dir = lane & 7;
  const double* Z = geo_ptr<double>(geo, geo->off_z);
  const double* AWL = geo_ptr<double>(geo, geo->off_awl);
  const int64_t* SW = geo_ptr<int64_t>(geo, geo->off_seg_chiwl);
  const double* NZL = geo_ptr<double>(geo, geo->off_nzl);
  const double awl = AWL[n], z = Z[n];
  D1 sD[NSCAL];
  for (int i = 0; i < NSCAL; ++i) sD[i] = mk1(tb->sv[i], tb->sd[dir][i]);
  const D1 chi_wl = xfmax(interp_d1(awl, c->atab_chi, tb->chiv, tb->chid[dir], unpack_seg(SW[n])), 0.0);
  const D1 cf = 3.0 * (H0 * H0) * sD[S_OMEGA_M] / 2.0 / C_KMS;  // probes.py:71
  const D8 chiwl8 = gather8(chi_wl);
  double* kd = gi.kernd;
  for (int t0 = 0; t0 < n_tr; t0 += 4) {
    int tl[4];
    int cnt = 0;
    for (int t = t0; t < min(t0 + 4, n_tr); ++t) tl[cnt++] = t;
    D8 acc[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] = dconst<NDIR>(0.0);
    bool any_wl = false;
    for (int u = 0; u < cnt; ++u) any_wl |= geo->kind[tl[u]] == JCG_TRACER_WL;
    if (any_wl) {
      for (int g = 0; g < geo->n_groups; ++g) {
        const size_t row = (size_t)n * NZP;
        const double* AP = geo_ptr<double>(geo, geo->off_ap[g]) + row;
        const int64_t* SP = geo_ptr<int64_t>(geo, geo->off_segp[g]) + row;
        for (int j = lane; j < NZP; j += 32) {
          const double ap = AP[j];
          const int2 sg = unpack_seg(SP[j]);
          const double ixp = 1.0 / (c->atab_chi[sg.y] - c->atab_chi[sg.x]);
          D8 chip;
          {
            const double a_s = (tb->chiv[sg.y] - tb->chiv[sg.x]) * ixp;
            const double b_s = tb->chiv[sg.x] - a_s * c->atab_chi[sg.x];
            chip.v = a_s * ap + b_s;
#pragma unroll
            for (int d = 0; d < NDIR; ++d) {
              const double ad = (tb->chid[d][sg.y] - tb->chid[d][sg.x]) * ixp;
              chip.d[d] = tb->chid[d][sg.x] + ad * (ap - c->atab_chi[sg.x]);
            }
          }
          chip = xfmax(chip, 0.0);
          const D8 ratio = xfmax(chip - chiwl8, 0.0) / xfmax(chip, 1.0);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            if (u < cnt && geo->kind[tl[u]] == JCG_TRACER_WL && geo->group[tl[u]] == g) {
              const double Wv = geo_ptr<double>(geo, geo->off_W[tl[u]])[row + j];
              acc[u] = acc[u] + Wv * ratio;
            }
          }
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          acc[u].v += __shfl_xor_sync(0xffffffffu, acc[u].v, o);
#pragma unroll
          for (int d = 0; d < NDIR; ++d) acc[u].d[d] += __shfl_xor_sync(0xffffffffu, acc[u].d[d], o);
        }
      }
    }
    if (lane < NDIR) {
      for (int u = 0; u < cnt; ++u) {
        const int t = tl[u];
        D1 kv;
        if (geo->kind[t] == JCG_TRACER_WL) {
          double ad = 0.0;
#pragma unroll
          for (int d = 0; d < NDIR; ++d)
            if (d == dir) ad = acc[u].d[d];
          D1 racc = mk1(acc[u].v, ad);
          if (geo->nz_kind[t] == JCG_NZ_DELTA) {
            // single plane (probes.py:53-64): clip(chi(z0) - chi, 0) / clip(chi(z0), 1)
            const double a0 = 1.0 / (1.0 + geo->nz_z0[t]);
            const int2 sg0 = interp_segment_inc(a0, c->atab_chi, NCHI, logspace_guess(a0, NCHI));
            const D1 chi0 = xfmax(interp_d1(a0, c->atab_chi, tb->chiv, tb->chid[dir], sg0), 0.0);
            racc = xfmax(chi0 - chi_wl, 0.0) / xfmax(chi0, 1.0);
          }
          const D1 rk = racc * (1.0 + z) * chi_wl;
          kv = cf * rk;
          if (geo->bias_kind[t] != JCG_BIAS_NONE) {
            double iv, id;
            bias_term_d1(tb, c, geo, t, dir, awl, z, NZL[(size_t)t * na + n], true, &iv, &id);
            kv = kv + mk1(iv, id);
          }
          kv = kv * (1.0 + geo->mult[t]);
        } else {
          double iv, id;
          bias_term_d1(tb, c, geo, t, dir, awl, z, NZL[(size_t)t * na + n], false, &iv, &id);
          kv = mk1(iv, id);
        }
        double* dst = kd + ((size_t)t * na + n) * (NDIR + 1);
        if (dir == 0) dst[0] = kv.v;
        dst[1 + dir] = kv.d[0];
      }
    }
  }
}

// ------------------------------------------------ Limber integrand adjoint --
struct NodeX {
  double chic, g, knl, beta, alpha, an, bn, lcf3, f1, f2, gam, nu, mu;
};
struct NodeK {
  double keq, sh, betac, alphac, alphab, betab, betanode, ksilk, fb, fc, ns, pknorm;
  double agam, nwq;  // transfer type "eisenhu"
  bool nw;
};

// P(k = kh / chic, a) of halofit_node_lk (Eisenstein-Hu x primordial x
// takahashi2012, transfer.py:107-153, power.py:42-53, 246-260) and its
// partial derivatives: ga[NodeA] (per-node inputs) and gc[NodeC]
// (per-cosmology inputs) receive dP/d(input).  Hand-written reverse sweep.
__device__ double node_fb(double kh, double lkh, const NodeX& x, const NodeK& c, double* ga, double* gc,
                          bool lin) {
  // forward
  const double k = kh / x.chic;
  const double lk = lkh - log(x.chic);
  const double q13 = 13.41 * c.keq;
  const double q = k / q13;
  const double u1 = exp(1.08 * (lk - log(q13)));
  const double den_c = 1.0 + 69.9 * u1;
  const double Cb = 386.0 / den_c;
  const double qq = q * q;
  const double A1 = EULER_E + 1.8 * c.betac * q, L1 = log(A1);
  const double A2 = EULER_E + 1.8 * q, L2 = log(A2);
  const double cA = 14.2 + Cb, cB = 14.2 / c.alphac + Cb;
  const double Da = L1 + cA * qq, Db = L1 + cB * qq, Dn = L2 + cA * qq;
  const double Ta = L1 / Da, Tb = L1 / Db, Tn = L2 / Dn;
  const double ksh = k * c.sh;
  const double x54 = ksh / 5.4, x2 = x54 * x54;
  const double f = 1.0 / (1.0 + x2 * x2);
  const double Tc = f * Ta + (1.0 - f) * Tb;
  const double bn = c.betanode / ksh;
  const double B3 = 1.0 + bn * bn * bn;
  const double cb = cbrt(B3);
  const double ts = c.sh / cb;
  const double x52 = ksh / 5.2, E52 = 1.0 + x52 * x52;
  const double bb = c.betab / ksh, Bb = 1.0 + bb * bb * bb;
  const double ex1 = exp(1.4 * (lk - log(c.ksilk)));
  const double silk = exp(-ex1);
  const double arg = k * ts;
  double sn, cs;
  sincos(arg, &sn, &cs);
  const double sinc = sn / arg;
  const double Tbr0 = Tn / E52 + c.alphab / Bb * silk;
  const double Tbar = Tbr0 * sinc;
  // type "eisenhu" (transfer.py:88-105); the oscillating fit above is then
  // evaluated too but gets a zero adjoint
  const double xn = 0.43 * k * c.sh, xn2 = xn * xn;
  const double un = 1.0 / (1.0 + xn2 * xn2);
  const double gen = c.agam + (1.0 - c.agam) * un;
  const double qn = k * c.nwq / gen;
  const double An = 2.0 * EULER_E + 1.8 * qn;
  const double Ln = log(An);
  const double rcn = 1.0 / (1.0 + 62.5 * qn);
  const double Cn = 14.2 + 731.0 * rcn;
  const double Dtn = Ln + Cn * qn * qn;
  const double T = c.nw ? Ln / Dtn : c.fb * Tbar + c.fc * Tc;
  const double eP = exp(c.ns * lk);
  const double gg = x.g * x.g;
  const double pklin = eP * (T * T) * gg * c.pknorm;
  const double k3 = k * k * k;
  const double d2l = k3 * pklin / TWO_PI2_G;
  const double y = k / x.knl;
  const double ly = lk - log(x.knl);
  const double fy = y / 4.0 + (y * y) / 8.0;
  const double efy = exp(-fy);
  const double ld = log(1.0 + d2l);
  const double pb = exp(x.beta * ld);
  const double den_a = 1.0 + x.alpha * d2l;
  const double Q = pb / den_a * efy;
  const double d2q = d2l * Q;
  const double H1 = exp(3.0 * x.f1 * ly);
  const double H2 = exp(x.f2 * ly);
  const double E3a = 3.0 - x.gam, E3b = x.lcf3 + ly;
  const double H3 = exp(E3a * E3b);
  const double D = 1.0 + x.bn * H2 + H3;
  const double d2hp = x.an * H1 / D;
  const double y2 = y * y, yn = (y2 + x.mu * y) + x.nu;
  const double Rr = y2 / yn;
  const double d2h = d2hp * Rr;
  const double S = lin ? d2l : d2q + d2h;  // lin: linear_matter_power
  const double P = TWO_PI2_G / k3 * S;
  // reverse, seed dP/dP = 1
  const double Sb = TWO_PI2_G / k3;
  double k3b = -P / k3;
  const double d2qb = lin ? 0.0 : Sb, d2hb = d2qb;
  const double d2hpb = d2hb * Rr;
  const double Rb = d2hb * d2hp;
  ga[A_NU] += -Rb * y2 / (yn * yn);
  ga[A_MU] += -Rb * y2 * y / (yn * yn);
  double yb = Rb * y * (x.mu * y + 2.0 * x.nu) / (yn * yn);
  ga[A_AN] += d2hpb * H1 / D;
  const double H1b = d2hpb * x.an / D;
  const double Dbar = -d2hpb * d2hp / D;
  ga[A_BN] += Dbar * H2;
  const double H2b = Dbar * x.bn;
  const double E3 = Dbar * H3;  // adjoint of the exponent of H3
  double lyb = H1b * H1 * 3.0 * x.f1 + H2b * H2 * x.f2 + E3 * E3a;
  ga[A_F1] += H1b * H1 * 3.0 * ly;
  ga[A_F2] += H2b * H2 * ly;
  ga[A_GAM] += -E3 * E3b;
  ga[A_LCF3] += E3 * E3a;
  double d2lb = lin ? Sb : d2qb * Q;
  const double Qb = d2qb * d2l;
  const double pbb = Qb * efy / den_a;
  const double denab = -Qb * Q / den_a;
  const double efyb = Qb * pb / den_a;
  ga[A_ALPHA] += denab * d2l;
  d2lb += denab * x.alpha;
  ga[A_BETA] += pbb * pb * ld;
  d2lb += pbb * pb * x.beta / (1.0 + d2l);
  yb += -efyb * efy * (0.25 + y / 4.0);
  double lkb = lyb;
  double knlb = -lyb / x.knl - yb * y / x.knl;
  double kb = yb / x.knl;
  k3b += d2lb * pklin / TWO_PI2_G;
  const double pklinb = d2lb * k3 / TWO_PI2_G;
  kb += k3b * 3.0 * k * k;
  const double ePb = pklinb * (T * T) * gg * c.pknorm;
  const double Tbn = pklinb * eP * 2.0 * T * gg * c.pknorm;  // adjoint of T
  if (c.nw) {
    const double Tv = Ln / Dtn;
    const double Lnb = Tbn * (1.0 - Tv) / Dtn;
    const double Dtnb = -Tbn * Tv / Dtn;
    const double qnb = Dtnb * (Cn * 2.0 * qn - qn * qn * 731.0 * 62.5 * rcn * rcn) + Lnb * 1.8 / An;
    kb += qnb * c.nwq / gen;
    gc[C_NWQ] += qnb * k / gen;
    const double genb = -qnb * qn / gen;
    gc[C_AGAM] += genb * (1.0 - un);
    const double xnb = -genb * (1.0 - c.agam) * 4.0 * xn2 * xn * un * un;
    kb += xnb * 0.43 * c.sh;
    gc[C_SH] += xnb * 0.43 * k;
  }
  const double Tbarr = c.nw ? 0.0 : Tbn;
  ga[A_G] += pklinb * eP * (T * T) * 2.0 * x.g * c.pknorm;
  gc[C_PKNORM] += pklinb * eP * (T * T) * gg;
  gc[C_NS] += ePb * eP * lk;
  lkb += ePb * eP * c.ns;
  gc[C_FB] += Tbarr * Tbar;
  gc[C_FC] += Tbarr * Tc;
  const double Tbarb = Tbarr * c.fb;
  const double Tcb = Tbarr * c.fc;
  const double Tbr0b = Tbarb * sinc;
  const double sincb = Tbarb * Tbr0;
  const double argb = sincb * (cs - sinc) / arg;
  kb += argb * ts;
  const double tsb = argb * k;
  const double Tnb = Tbr0b / E52;
  const double E52b = -Tbr0b * Tn / (E52 * E52);
  gc[C_ALPHAB] += Tbr0b * silk / Bb;
  const double silkb = Tbr0b * c.alphab / Bb;
  const double Bbb = -Tbr0b * c.alphab * silk / (Bb * Bb);
  const double ex1b = -silkb * silk;
  lkb += ex1b * ex1 * 1.4;
  gc[C_KSILK] += -ex1b * ex1 * 1.4 / c.ksilk;
  const double bbb = Bbb * 3.0 * bb * bb;
  gc[C_BETAB] += bbb / ksh;
  double kshb = -bbb * bb / ksh + E52b * 2.0 * x52 / 5.2;
  gc[C_SH] += tsb / cb;
  const double cbb = -tsb * ts / cb;
  const double bnb = cbb * cb / (3.0 * B3) * 3.0 * bn * bn;
  gc[C_BETANODE] += bnb / ksh;
  kshb += -bnb * bn / ksh;
  const double fbar = Tcb * (Ta - Tb);
  const double Tab = Tcb * f, Tbb = Tcb * (1.0 - f);
  kshb += (-fbar * f * f * 2.0 * x2) * 2.0 * x54 / 5.4;
  kb += kshb * c.sh;
  gc[C_SH] += kshb * k;
  const double Dab = -Tab * Ta / Da, Dbb = -Tbb * Tb / Db, Dnb = -Tnb * Tn / Dn;
  const double L1b = Tab / Da + Tbb / Db + Dab + Dbb;
  const double L2b = Tnb / Dn + Dnb;
  const double Cbb = (Dab + Dbb + Dnb) * qq;
  gc[C_ALPHAC] += Dbb * qq * (-14.2 / (c.alphac * c.alphac));
  double qb = (Dab * cA + Dbb * cB + Dnb * cA) * 2.0 * q;
  const double A1b = L1b / A1;
  gc[C_BETAC] += A1b * 1.8 * q;
  qb += A1b * 1.8 * c.betac + L2b / A2 * 1.8;
  const double u1b = -Cbb * Cb * 69.9 / den_c;
  lkb += u1b * u1 * 1.08;
  gc[C_KEQ] += -u1b * u1 * 1.08 / c.keq - qb * q / c.keq;
  kb += qb / q13;
  ga[A_CHIC] += -lkb / x.chic - kb * k / x.chic;
  ga[A_KNL] += knlb;
  return P;
}

constexpr int GL_TA = 16;     // a nodes per chunk
constexpr int GL_THREADS = 256;
constexpr int GL_MAXO = 17;   // accumulators per thread

// One CTA per (l tile, a split, cosmology): C_ell and dC_ell/dtheta partial sums.
__global__ void __launch_bounds__(GL_THREADS)
    grad_limber_kernel(GradBatch gb, const ConstTables* __restrict__ c, int LT) {
  const int item = blockIdx.z, split = blockIdx.y;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const GeoHeader* geo = gi.geo;
  const int n_ell = geo->n_ell, n_cls = geo->n_cls, na = geo->na;
  const bool lin = pk_model(geo->physics) == JCG_PK_LINEAR;
  const int l0 = blockIdx.x * LT;
  if (l0 >= n_ell) return;
  const int lt = min(LT, n_ell - l0);
  const int per = (na + gb.n_split - 1) / gb.n_split;
  const int a_begin = split * per, a_end = min(na, a_begin + per);
  extern __shared__ double sm[];
  double* cvs = sm;                                   // [NC_IN] values
  double* cds = cvs + NC_IN;                          // [NC_IN][NDIR]
  double* khs = cds + NC_IN * NDIR;                   // [LT]
  double* lkhs = khs + 32;                            // [LT]
  double* rv = lkhs + 32;                             // [GL_TA][NA_IN]
  double* rd = rv + GL_TA * NA_IN;                    // [GL_TA][NA_IN][NDIR]
  double* Mv = rd + GL_TA * NA_IN * NDIR;             // [GL_TA][n_cls]
  double* Md = Mv + GL_TA * n_cls;                    // [GL_TA][n_cls][NDIR]
  double* Pv = Md + GL_TA * n_cls * NDIR;             // [GL_TA][LT]
  double* Pd = Pv + GL_TA * LT;                       // [GL_TA][LT][NDIR]
  const int tid = threadIdx.x;
  const TabD* tb = gi.tab;
  for (int i = tid; i < NC_IN; i += GL_THREADS) {
    const int si = kNodeCScalar[i];
    cvs[i] = tb->sv[si];
    for (int d = 0; d < NDIR; ++d) cds[i * NDIR + d] = tb->sd[d][si];
  }
  const double* ELL = geo_ptr<double>(geo, geo->off_ell);
  const double* EF = geo_ptr<double>(geo, geo->off_ellfac);
  for (int l = tid; l < lt; l += GL_THREADS) {
    khs[l] = ELL[l0 + l] + 0.5;
    lkhs[l] = log(khs[l]);
  }
  __syncthreads();
  NodeK ck;
  ck.keq = cvs[C_KEQ]; ck.sh = cvs[C_SH]; ck.betac = cvs[C_BETAC]; ck.alphac = cvs[C_ALPHAC];
  ck.alphab = cvs[C_ALPHAB]; ck.betab = cvs[C_BETAB]; ck.betanode = cvs[C_BETANODE];
  ck.ksilk = cvs[C_KSILK]; ck.fb = cvs[C_FB]; ck.fc = cvs[C_FC]; ck.ns = cvs[C_NS];
  ck.pknorm = cvs[C_PKNORM];
  ck.agam = cvs[C_AGAM]; ck.nwq = cvs[C_NWQ]; ck.nw = tf_nowiggle(geo->physics);
  const double* rowd = gi.rowd;
  const double* kd = gi.kernd;
  const int nout = lt * n_cls * (NDIR + 1);
  double acc[GL_MAXO];
#pragma unroll
  for (int r = 0; r < GL_MAXO; ++r) acc[r] = 0.0;
  for (int base = a_begin; base < a_end; base += GL_TA) {
    const int tc = min(GL_TA, a_end - base);
    for (int e = tid; e < tc * NA_IN; e += GL_THREADS) {
      const int t = e / NA_IN, x = e % NA_IN;
      const double* r = rowd + (size_t)(base + t) * NROWD;
      rv[e] = r[x];
      for (int d = 0; d < NDIR; ++d) rd[e * NDIR + d] = r[NA_IN * (1 + d) + x];
    }
    __syncthreads();
    // M_ij(a) = u K_i K_j with tangents
    for (int e = tid; e < tc * n_cls; e += GL_THREADS) {
      const int t = e / n_cls, p = e % n_cls, n = base + t;
      const double* Ki = kd + ((size_t)geo->pair_i[p] * na + n) * (NDIR + 1);
      const double* Kj = kd + ((size_t)geo->pair_j[p] * na + n) * (NDIR + 1);
      const double u = rv[t * NA_IN + A_U];
      Mv[e] = u * Ki[0] * Kj[0];
      for (int d = 0; d < NDIR; ++d)
        Md[e * NDIR + d] = rd[(t * NA_IN + A_U) * NDIR + d] * Ki[0] * Kj[0] +
                           u * (Ki[1 + d] * Kj[0] + Ki[0] * Kj[1 + d]);
    }
    // integrand with its tangents
    for (int e = tid; e < tc * lt; e += GL_THREADS) {
      const int t = e / lt, l = e % lt;
      const double* xv = rv + t * NA_IN;
      NodeX nx;
      nx.chic = xv[A_CHIC]; nx.g = xv[A_G]; nx.knl = xv[A_KNL]; nx.beta = xv[A_BETA];
      nx.alpha = xv[A_ALPHA]; nx.an = xv[A_AN]; nx.bn = xv[A_BN]; nx.lcf3 = xv[A_LCF3];
      nx.f1 = xv[A_F1]; nx.f2 = xv[A_F2]; nx.gam = xv[A_GAM]; nx.nu = xv[A_NU]; nx.mu = xv[A_MU];
      double ga[NA_IN], gcv[NC_IN];
      for (int i = 0; i < NA_IN; ++i) ga[i] = 0.0;
      for (int i = 0; i < NC_IN; ++i) gcv[i] = 0.0;
      const double P = node_fb(khs[l], lkhs[l], nx, ck, ga, gcv, lin);
      Pv[t * LT + l] = P;
      for (int d = 0; d < NDIR; ++d) {
        double s = 0.0;
        for (int i = 0; i < A_U; ++i) s += ga[i] * rd[(t * NA_IN + i) * NDIR + d];
        for (int i = 0; i < NC_IN; ++i) s += gcv[i] * cds[i * NDIR + d];
        Pd[(t * LT + l) * NDIR + d] = s;
      }
    }
    __syncthreads();
    // contraction: outputs (l, p, s), s = 0 value, 1..8 tangents
#pragma unroll
    for (int r = 0; r < GL_MAXO; ++r) {
      const int o = tid + r * GL_THREADS;
      if (o < nout) {
        const int s = o % (NDIR + 1);
        const int lp = o / (NDIR + 1);
        const int l = lp % lt, p = lp / lt;
        double part = 0.0;
        if (s == 0) {
          for (int t = 0; t < tc; ++t) part += Pv[t * LT + l] * Mv[t * n_cls + p];
        } else {
          const int d = s - 1;
          for (int t = 0; t < tc; ++t)
            part += Pd[(t * LT + l) * NDIR + d] * Mv[t * n_cls + p] +
                    Pv[t * LT + l] * Md[(t * n_cls + p) * NDIR + d];
        }
        acc[r] += part;
      }
    }
    __syncthreads();
  }
  double* part = gi.part + (size_t)split * n_cls * n_ell * (NDIR + 1);
#pragma unroll
  for (int r = 0; r < GL_MAXO; ++r) {
    const int o = tid + r * GL_THREADS;
    if (o < nout) {
      const int s = o % (NDIR + 1);
      const int lp = o / (NDIR + 1);
      const int l = lp % lt, p = lp / lt;
      const int ell = l0 + l;
      const double ef = EF[(size_t)geo->pair_i[p] * n_ell + ell] * EF[(size_t)geo->pair_j[p] * n_ell + ell];
      part[((size_t)p * n_ell + ell) * (NDIR + 1) + s] = acc[r] * ef;
    }
  }
}

// Fixed-order sum over the a splits; C_ell and the Jacobian out.  Grid (x, item).
__global__ void grad_reduce_kernel(GradBatch gb) {
  const int item = blockIdx.y;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const size_t per = (size_t)gi.geo->n_cls * gi.geo->n_ell;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < per;
       idx += (size_t)gridDim.x * blockDim.x) {
    double v[NDIR + 1];
    for (int s = 0; s <= NDIR; ++s) v[s] = 0.0;
    for (int sp = 0; sp < gb.n_split; ++sp) {
      const double* p = gi.part + ((size_t)sp * per + idx) * (NDIR + 1);
      for (int s = 0; s <= NDIR; ++s) v[s] += p[s];
    }
    if (gi.cl) gi.cl[idx] = v[0];
    for (int d = 0; d < NDIR; ++d) gi.jac[idx * NDIR + d] = v[1 + d];
  }
}

size_t grad_limber_smem(int n_cls, int LT) {
  return sizeof(double) * (NC_IN * (1 + NDIR) + 64 + GL_TA * NA_IN * (1 + NDIR) +
                           (size_t)GL_TA * n_cls * (1 + NDIR) + (size_t)GL_TA * LT * (1 + NDIR));
}

int grad_limber_tile(int n_ell, int n_cls) {
  int lt = (GL_THREADS * GL_MAXO) / (n_cls * (NDIR + 1));
  if (lt > 32) lt = 32;
  if (lt < 1) lt = 1;
  const int tiles = (n_ell + lt - 1) / lt;
  return (n_ell + tiles - 1) / tiles;
}

// The per-node physics of the fp32c table stage with the abscissae as float
// pairs (ConstTables' *_ff grids): dchi_dlna_cT, growth_qr_cT and
// eh_transferT / eh_nowiggleT of jcg_dual.cuh with FF in place of their
// double arguments, the same operations in the same order, so that no
// operand is converted from float64 at run time.
__device__ __forceinline__ FF8 dchi_dlna_f8(const BgT<FF8>& c, FF a, FF lna, FF ia) {
  const FF8 f = -3.0 * (1.0 + c.w0 + c.wa) * lna + 3.0 * c.wa * (a - ffc(1.0));
  const FF8 ef = xexp(f);
  const FF ia2 = ia * ia;
  const FF8 e2 = c.Om * (ia2 * ia) + c.Ok * ia2 + c.Ode * ef;
  return (ffc(RH) * ia) / xsqrt(e2);
}
__device__ __forceinline__ void growth_qr_f8(const BgT<FF8>& b, FF x, FF lnx, FF ix, FF8& q, FF8& r) {
  const FF8 f = -3.0 * (1.0 + b.w0 + b.wa) * lnx + 3.0 * b.wa * (x - ffc(1.0));
  const FF8 ef = xexp(f);
  const FF ix2 = ix * ix, ix3 = ix2 * ix;
  const FF8 ie2 = 1.0 / (b.Om * ix3 + b.Ok * ix2 + b.Ode * ef);
  const FF8 omm = b.Om * ix3 * ie2, omde = b.Ode * ef * ie2;
  const FF8 w = b.w0 + (ffc(1.0) - x) * b.wa;  // wT (background.py:53)
  q = (2.0 - 0.5 * (omm + (1.0 + 3.0 * w) * omde)) * ix;
  r = 1.5 * omm * ix2;
}
__device__ __noinline__ FF8 eh_nowiggle_f8(FF8 sh_d, FF8 ag, FF8 nwq, FF k) {
  const FF8 x = (ffc(0.43) * k) * sh_d, x2 = x * x;
  const FF8 q = k * nwq / (ag + (1.0 - ag) / (1.0 + x2 * x2));
  const FF8 L = xlog(2.0 * EULER_E + 1.8 * q);
  const FF8 C = 14.2 + 731.0 / (1.0 + 62.5 * q);
  return L / (L + C * q * q);
}
__device__ __forceinline__ FF8 eh_transfer_f8(const FF8* s, FF k, FF lk) {
  const FF8 k_eq = s[S_K_EQ], sh_d = s[S_SH_D];
  if (s[S_TFNW].v.hi != 0.f) return eh_nowiggle_f8(sh_d, s[S_AGAM], s[S_NWQ], k);
  const FF8 q = k / (13.41 * k_eq);
  const FF8 q108 = xexp(1.08 * (lk - s[S_LGQ]));
  const FF8 Cb = 386.0 / (1.0 + 69.9 * q108);
  const FF8 qq = q * q;
  const FF8 L1 = xlog(EULER_E + 1.8 * s[S_BETA_C] * q);
  const FF8 L2 = xlog(EULER_E + 1.8 * q);
  const FF8 Ta = L1 / (L1 + (14.2 + Cb) * qq);
  const FF8 Tb = L1 / (L1 + (14.2 / s[S_ALPHA_C] + Cb) * qq);
  const FF8 Tn = L2 / (L2 + (14.2 + Cb) * qq);
  const FF8 ksh = k * sh_d;
  const FF8 x54 = ksh / 5.4, x54s = x54 * x54;
  const FF8 f = 1.0 / (1.0 + x54s * x54s);
  const FF8 Tc = f * Ta + (1.0 - f) * Tb;
  const FF8 bn = s[S_BETA_NODE] / ksh;
  const FF8 tilde_s = sh_d / xcbrt(1.0 + bn * bn * bn);
  const FF8 x52 = ksh / 5.2;
  const FF8 bb = s[S_BETA_B] / ksh;
  const FF8 silk = xexp(-xexp(1.4 * (lk - s[S_LGKSILK])));
  const FF8 arg = k * tilde_s;
  const FF8 sinc = xsin(arg) / arg;
  const FF8 Tbar = (Tn / (1.0 + x52 * x52) + s[S_ALPHA_B] / (1.0 + bb * bb * bb) * silk) * sinc;
  return s[S_FB] * Tbar + s[S_FC] * Tc;
}

// fp32c: the table kernel's per-node evaluations (chi right-hand sides,
// growth coefficients, Romberg integrand, exp(n_s ln k) T^2 on the P(k)
// grid), one per thread, in DualFF<8> with float-pair abscissae.
// KIND 0: chi right-hand sides (nodes, midpoints); 1: growth coefficients
// (nodes, midpoints); 2: Eisenstein-Hu at the Romberg and P(k) nodes.  One
// launch per kind keeps each kernel's code small (the three inlined bodies in
// one kernel thrashed the instruction cache).
template <int KIND>
__global__ void __launch_bounds__(128) grad_nodes_kernel(GradBatch gb, const ConstTables* __restrict__ c) {
  const int item = blockIdx.y;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  const TabD* tb = gi.tab;
  // the cosmology's scalars with tangents, shared by the CTA (a per-thread
  // copy would sit in local memory)
  __shared__ FF8 sF[NSCAL];
  for (int i = threadIdx.x; i < NSCAL; i += blockDim.x) sF[i] = ff8_of(tb->sv[i], &tb->sd[0][i], NSCAL);
  __syncthreads();
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  const BgT<FF8> bgf = make_bgT(sF);
  double* dst = gb.gnode + (size_t)item * GNODE_STRIDE;
  auto putf = [&](int off, int n, int i, const FF8& x) { put_packed(dst + off, n, i, x); };
  if (KIND == 0) {
    if (w < NCHI) {
      putf(GNODE_FN, NCHI, w, dchi_dlna_f8(bgf, f2ff(c->chi_a_ff[w]), f2ff(c->lna_chi_ff[w]), f2ff(c->chi_ia_ff[w])));
    } else if (w < 2 * NCHI - 1) {
      const int i = w - NCHI + 1;
      putf(GNODE_FM, NCHI, i, dchi_dlna_f8(bgf, f2ff(c->chi_am_ff[i]), f2ff(c->chi_lnam_ff[i]), f2ff(c->chi_iam_ff[i])));
    }
  } else if (KIND == 1) {
    FF8 q, r;
    if (w < NGROW) {
      growth_qr_f8(bgf, f2ff(c->grow_a_ff[w]), f2ff(c->grow_lna_ff[w]), f2ff(c->grow_ia_ff[w]), q, r);
      putf(GNODE_QR, NGROW, w, q);
      putf(GNODE_QR + 5 * NGROW, NGROW, w, r);
    } else if (w < 2 * NGROW - 1) {
      const int i = w - NGROW + 1;
      growth_qr_f8(bgf, f2ff(c->grow_am_ff[i]), f2ff(c->grow_lnam_ff[i]), f2ff(c->grow_iam_ff[i]), q, r);
      putf(GNODE_QR + 10 * NGROW, NGROW, i, q);
      putf(GNODE_QR + 15 * NGROW, NGROW, i, r);
    }
  } else if (w < NROMB + NKH) {
    const bool romb = w < NROMB;
    const int i = romb ? w : w - NROMB;
    const FF logk = f2ff(romb ? c->romb_logk_ff[i] : c->logk_ff[i]);
    const FF8 T = eh_transfer_f8(sF, f2ff(romb ? c->romb_k_ff[i] : c->kh_ff[i]), logk);
    const FF8 TT = T * T, ex = xexp(sF[S_NS] * logk);
    if (romb) putf(GNODE_FR, NROMB, i, f2ff(c->romb_kw2_ff[i]) * (TT * ex));
    else putf(GNODE_U, NKH, i, ex * TT);
  }
}

// Scalars with tangents, one thread per (cosmology, direction): the Dual<1>
// chain of pow / log / sqrt with all lanes of a warp busy.
__global__ void __launch_bounds__(128) grad_scalars_kernel(GradBatch gb) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int item = idx / NDIR, dir = idx % NDIR;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  D1 p[8];
  for (int i = 0; i < 8; ++i) p[i] = mk1(gi.params[i], (i == dir && dir != gb.gamma_dir) ? 1.0 : 0.0);
  D1 s[NSCAL];
  cosmo_scalarsT(p, s, tf_nowiggle(gi.geo->physics));
  for (int i = 0; i < NSCAL; ++i) {
    if (dir == 0) gi.tab->sv[i] = s[i].v;
    gi.tab->sd[dir][i] = s[i].d[0];
  }
}

// fp32c: the scalars with all 8 tangents in DualFF<8> (value as a float
// pair, no float64), one thread per cosmology: the same chain as
// grad_scalars_kernel without the FP64 pipe (the float64 Dual<1> chain per
// (cosmology, direction) is bound by it).
__global__ void __launch_bounds__(64) grad_scalars32_kernel(GradBatch gb) {
  const int item = blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  FF8 p[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    p[i].v = ff_of(gi.params[i]);
#pragma unroll
    for (int d = 0; d < NDIR; ++d) p[i].d[d] = (i == d && d != gb.gamma_dir) ? 1.f : 0.f;
  }
  FF8 s[NSCAL];
  cosmo_scalarsT(p, s, tf_nowiggle(gi.geo->physics));
  for (int i = 0; i < NSCAL; ++i) {
    gi.tab->sv[i] = ffd(s[i].v);
#pragma unroll
    for (int d = 0; d < NDIR; ++d) gi.tab->sd[d][i] = s[i].d[d];
  }
}

// Small batches: one half warp per (cosmology, direction), the chain's
// independent calls on different lanes (cosmo_scalars_warpT).
__global__ void __launch_bounds__(128) grad_scalars_warp_kernel(GradBatch gb) {
  const int item = blockIdx.x, dir = threadIdx.x >> 4, lane = threadIdx.x & 15;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  D1 p[8];
  for (int i = 0; i < 8; ++i) p[i] = mk1(gi.params[i], (i == dir && dir != gb.gamma_dir) ? 1.0 : 0.0);
  D1 s[NSCAL];
  cosmo_scalars_warpT<D1>(p, s, lane, tf_nowiggle(gi.geo->physics));
  D1 v0 = mk1(0.0, 0.0), v1 = v0, v2 = v0;
#pragma unroll
  for (int k = 0; k < 16; ++k)
    if (k == lane) v0 = s[k], v1 = s[k + 16], v2 = k + 32 < NSCAL ? s[k + 32] : v0;
  if (dir == 0) {
    gi.tab->sv[lane] = v0.v;
    gi.tab->sv[lane + 16] = v1.v;
    if (lane + 32 < NSCAL) gi.tab->sv[lane + 32] = v2.v;
  }
  gi.tab->sd[dir][lane] = v0.d[0];
  gi.tab->sd[dir][lane + 16] = v1.d[0];
  if (lane + 32 < NSCAL) gi.tab->sd[dir][lane + 32] = v2.d[0];
}

// Growth for JCG_GROWTH_GAMMA (background.py:515-582) with the tangents of
// the 8 parameters (gamma held fixed): the forward growth_gamma_kernel's
// recurrence in Dual<1>, one warp per direction (warp 0 also writes the
// values).  Replaces the growth-ODE table grad_tables wrote.
__global__ void __launch_bounds__(32 * NDIR) grad_growth_gamma_kernel(GradBatch gb, const ConstTables* __restrict__ c) {
  const int item = blockIdx.x;
  if (item >= gb.n_items) return;
  const GradItem gi = grad_item(gb, item);
  if (!growth_gamma(gi.geo->physics)) return;
  __shared__ double fv[NGROW], fmv[NGROW], fd[NDIR][NGROW], fmd[NDIR][NGROW];
  const int d = threadIdx.x >> 5, lane = threadIdx.x & 31;
  TabD* tb = gi.tab;
  const D1 gam = mk1(gi.params[8], d == gb.gamma_dir ? 1.0 : 0.0);  // d/dgamma in that direction
  D1 sD[NSCAL];
  for (int i = 0; i < NSCAL; ++i) sD[i] = mk1(tb->sv[i], tb->sd[d][i]);
  const BgT<D1> bg = make_bgT(sD);
  auto f_of = [&](double lna) {
    const double a = exp(lna);
    D1 om_m, om_de;
    omT(bg, a, log(a), om_m, om_de);
    return xexp(gam * xlog(om_m));  // Omega_m^gamma
  };
  for (int i = lane; i < NGROW; i += 32) {
    const double lna = c->grow_lna[i];
    const D1 f = f_of(lna);
    if (d == 0) fv[i] = f.v;
    fd[d][i] = f.d[0];
    if (i > 0) {
      const double lp = c->grow_lna[i - 1];
      const D1 fm = f_of(lp + (lna - lp) / 2);
      if (d == 0) fmv[i] = fm.v;
      fmd[d][i] = fm.d[0];
    }
  }
  __syncthreads();
  if (lane == 0) {
    // values: the forward recurrence; tangents: the same sums of tangents
    D1 y = mk1(c->grow_lna[0], 0.0);
    D1 ys[NGROW];
    ys[0] = y;
    for (int i = 1; i < NGROW; ++i) {
      const double h = c->grow_lna[i] - c->grow_lna[i - 1];
      const D1 f0 = mk1(fv[i - 1], fd[d][i - 1]), fm = mk1(fmv[i], fmd[d][i]), f1 = mk1(fv[i], fd[d][i]);
      y = y + 1.0 / 6.0 * h * (((f0 + 2.0 * fm) + 2.0 * fm) + f1);
      ys[i] = y;
    }
    const D1 el = xexp(ys[NGROW - 1]);
    for (int i = 0; i < NGROW; ++i) {
      const D1 g = xexp(ys[i]) / el;
      if (d == 0) {
        tb->gv[i] = g.v;
        const FF gf = ff_of(g.v);
        tb->gF[i] = make_float2(gf.hi, gf.lo);  // the row stage's copy
      }
      tb->gd[d][i] = g.d[0];
      tb->gdF[i][d] = (float)g.d[0];
    }
  }
}

void launch_grad_front(const GradBatch& gb, const ConstTables* c, cudaStream_t st, unsigned stages) {
  const size_t smt = grad_tables_smem(gb.precision == JCG_FP32C);
  if (stages & GS_TABLES) {
  if (gb.n_items <= GNODE_MAX_ITEMS)
    grad_scalars_warp_kernel<<<gb.n_items, 16 * NDIR, 0, st>>>(gb);
  else if (gb.precision == JCG_FP32C)
    grad_scalars32_kernel<<<(gb.n_items + 63) / 64, 64, 0, st>>>(gb);
  else
    grad_scalars_kernel<<<(gb.n_items * NDIR + 127) / 128, 128, 0, st>>>(gb);
  if (gb.gnode) {
    grad_nodes_kernel<0><<<dim3((2 * NCHI - 1 + 127) / 128, gb.n_items), 128, 0, st>>>(gb, c);
    grad_nodes_kernel<1><<<dim3((2 * NGROW - 1 + 127) / 128, gb.n_items), 128, 0, st>>>(gb, c);
    grad_nodes_kernel<2><<<dim3((NROMB + NKH + 127) / 128, gb.n_items), 128, 0, st>>>(gb, c);
  }
  if (gb.precision == JCG_FP32C) {
    if (tf_nowiggle(gb.physics_or)) {
      cudaFuncSetAttribute(grad_tables_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smt);
      cudaFuncSetAttribute(grad_tables_kernel<true, true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);  // four CTAs per SM
      grad_tables_kernel<true, true><<<gb.n_items, 128, smt, st>>>(gb, c);
    } else {
      cudaFuncSetAttribute(grad_tables_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smt);
      cudaFuncSetAttribute(grad_tables_kernel<true, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);  // four CTAs per SM
      grad_tables_kernel<true, false><<<gb.n_items, 128, smt, st>>>(gb, c);
    }
  } else {
    cudaFuncSetAttribute(grad_tables_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smt);
    grad_tables_kernel<false, true><<<gb.n_items, 256, smt, st>>>(gb, c);
  }
  if (gb.precision == JCG_FP32C) grad_moments32_kernel<<<gb.n_items, NRT, 0, st>>>(gb, c);
  if (growth_gamma(gb.physics_or)) grad_growth_gamma_kernel<<<gb.n_items, 32 * NDIR, 0, st>>>(gb, c);
  }
  if (stages & GS_ROWS) {
    if (gb.precision == JCG_FP32C) {
      const dim3 grw = gb.listed ? dim3((gb.na + GR32_THREADS - 1) / GR32_THREADS, gb.n_items)
                                 : dim3((unsigned)(((long long)gb.na * gb.n_items + GR32_THREADS - 1) / GR32_THREADS));
      grad_rows32_kernel<<<grw, GR32_THREADS, 0, st>>>(gb, c);
    } else {
      dim3 grw((gb.na + 31) / 32, gb.n_items);
      grad_rows_kernel<<<grw, 256, 0, st>>>(gb, c);
    }
  }
  if (stages & GS_KERNELS) {
    if (gb.precision == JCG_FP32C) {
      launch_grad_kern32(gb, c, st);
    } else {
      dim3 gr((gb.na + 7) / 8, gb.n_items);
      grad_kern_kernel<<<gr, 256, 0, st>>>(gb, c);
    }
  }
}

void launch_grad(const GradBatch& gb, const ConstTables* c, cudaStream_t st) {
  launch_grad_front(gb, c, st);
  if (gb.precision == JCG_FP32C) {
    launch_grad_limber32(gb, c, st);
  } else {
    const int lt = grad_limber_tile(gb.n_ell, gb.n_cls);
    const size_t sml = grad_limber_smem(gb.n_cls, lt);
    cudaFuncSetAttribute(grad_limber_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sml);
    dim3 gl((gb.n_ell + lt - 1) / lt, gb.n_split, gb.n_items);
    grad_limber_kernel<<<gl, GL_THREADS, sml, st>>>(gb, c, lt);
  }
  const size_t per = (size_t)gb.n_cls * gb.n_ell;
  size_t bx = (per + 255) / 256;
  const size_t cap = (152 * 16 + gb.n_items - 1) / gb.n_items;
  if (bx > cap) bx = cap;
  grad_reduce_kernel<<<dim3((unsigned)(bx ? bx : 1), gb.n_items), 256, 0, st>>>(gb);
}

size_t grad_tab_bytes() { return sizeof(TabD); }

}  // namespace jcg

namespace jcg {

// ell tile and a-chunk of the Limber Jacobian kernel of each precision
int grad_tile(int precision, int n_ell, int n_cls) {
  if (precision == JCG_FP32C) return grad_limber32_tile(n_ell, n_cls);
  return grad_limber_tile(n_ell, n_cls);
}

static int grad_chunk(int precision, int n_cls) {
  return precision == JCG_FP32C ? grad_limber32_chunk(n_cls) : GL_TA;
}

// a-splits of the Limber Jacobian: enough CTAs to fill the GPU for small batches
int grad_n_split(const GeoHeader& h, int n_cosmo, int precision) {
  const int lt = grad_tile(precision, h.n_ell, h.n_cls);
  const int tiles = (h.n_ell + lt - 1) / lt;
  const int ctas = tiles * n_cosmo;
  int ns = (2 * 152 + ctas - 1) / ctas;
  const int ta = grad_chunk(precision, h.n_cls);
  const int max_ns = (h.na + ta - 1) / ta;
  if (ns > max_ns) ns = max_ns;
  if (ns < 1) ns = 1;
  return ns;
}

static size_t al256(size_t v) { return (v + 255) & ~size_t(255); }

// per-cosmology row and kernel sections of one precision
static size_t rows_bytes(const GeoHeader& h, int precision) {
  return precision == JCG_FP32C ? al256(sizeof(float) * (size_t)h.na * NROWG)
                                : al256(sizeof(double) * (size_t)h.na * NROWD);
}
static size_t kern_bytes(const GeoHeader& h, int precision) {
  const size_t el = precision == JCG_FP32C ? sizeof(float) : sizeof(double);
  return al256(el * (size_t)h.n_tr * h.na * (NDIR + 1));
}
// Taylor prefix tables of the fp32c moments, per cosmology
static size_t ptt_bytes(int precision) {
  return precision == JCG_FP32C ? PTT_STRIDE * sizeof(double) : 0;
}

// node scratch of the small-batch fp32c table path
static size_t gnode_bytes(int n, int precision) {
  // fp32c: the table stage's node evaluations always run in their own kernel
  // (one node per thread at full occupancy; the table kernel's 255-register
  // threads keep the scans)
  return precision == JCG_FP32C ? al256(sizeof(double) * GNODE_STRIDE * (size_t)n) : 0;
}

size_t grad_workspace_bytes(const GeoHeader& h, int n_cosmo, int precision) {
  const int ns = grad_n_split(h, n_cosmo, precision);
  GeoHeader hb = h;
  hb.na = h.na * n_cosmo;  // the uniform form keeps the sections batch-contiguous
  size_t o = al256(sizeof(TabD) * (size_t)n_cosmo);
  o += ptt_bytes(precision) * n_cosmo;
  o += rows_bytes(hb, precision);
  o += kern_bytes(hb, precision);
  o += al256(sizeof(double) * (size_t)ns * n_cosmo * h.n_cls * h.n_ell * (NDIR + 1));
  o += gnode_bytes(n_cosmo, precision);
  return o;
}

// ------------------------------------------------- vector-Jacobian product --
// FP64: the Jacobian, then grad[b][d] = sum_i vbar[b][i] jac[b][i][d] (one CTA
// per cosmology, fixed-order sums).
__global__ void vjp_contract_kernel(const double* __restrict__ jac, const double* __restrict__ vbar, int per,
                                    double* __restrict__ grad) {
  const int b = blockIdx.x;
  const double* J = jac + (size_t)b * per * NDIR;
  const double* v = vbar + (size_t)b * per;
  double acc[NDIR];
#pragma unroll
  for (int d = 0; d < NDIR; ++d) acc[d] = 0.0;
  for (int i = threadIdx.x; i < per; i += blockDim.x) {
    const double w = v[i];
#pragma unroll
    for (int d = 0; d < NDIR; ++d) acc[d] += w * J[(size_t)i * NDIR + d];
  }
  __shared__ double red[8][NDIR];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 0; d < NDIR; ++d) {
    double x = acc[d];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][d] = x;
  }
  __syncthreads();
  if (threadIdx.x < NDIR) {
    double x = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x += red[w][threadIdx.x];
    grad[(size_t)b * NDIR + threadIdx.x] = x;
  }
}

static size_t vjp32_item_bytes(const GeoHeader& h) {
  const size_t per = (size_t)h.n_cls * h.n_ell;
  const size_t nch = (size_t)vjp_chunks(h.na);
  return al256(sizeof(float) * nch * per) + al256(sizeof(double) * nch * NDIR) +
         al256(sizeof(float) * (size_t)h.n_tr * h.na) + al256(sizeof(double) * (size_t)kv_chunks(h.na) * NDIR);
}

size_t vjp_workspace_bytes(const GeoHeader& h, int n_cosmo, int precision) {
  const size_t per = (size_t)h.n_cls * h.n_ell;
  if (precision != JCG_FP32C)
    return grad_workspace_bytes(h, n_cosmo, precision) + al256(sizeof(double) * per * NDIR * (size_t)n_cosmo) +
           (n_cosmo > 0 ? al256(sizeof(double) * per * (size_t)n_cosmo) : 0);
  GeoHeader hb = h;
  hb.na = h.na * n_cosmo;
  size_t o = al256(sizeof(TabD) * (size_t)n_cosmo);
  o += ptt_bytes(precision) * n_cosmo;
  o += rows_bytes(hb, precision);
  o += kern_bytes(hb, precision);
  o += al256(sizeof(float) * (size_t)vjp_chunks(h.na) * per * n_cosmo);
  o += al256(sizeof(double) * (size_t)vjp_chunks(h.na) * NDIR * n_cosmo);
  o += al256(sizeof(float) * (size_t)h.n_tr * h.na * n_cosmo);
  o += al256(sizeof(double) * (size_t)kv_chunks(h.na) * NDIR * n_cosmo);
  o += al256(sizeof(int) * 9 * (size_t)kv_chunks(h.na));
  o += al256(sizeof(int) * 8 * (size_t)h.na);
  o += al256(sizeof(unsigned) * (size_t)n_cosmo);
  o += gnode_bytes(n_cosmo, precision);
  return o;
}

void vjp_run(const GeoHeader* geo, const GeoHeader& h, const double* params, int n_cosmo, int precision,
             const double* vbar, double* cl, double* grad, void* ws, const ConstTables* c, cudaStream_t st,
             int gamma_dir, unsigned stages) {
  char* base = static_cast<char*>(ws);
  const size_t per = (size_t)h.n_cls * h.n_ell;
  if (precision != JCG_FP32C) {
    const size_t gws = grad_workspace_bytes(h, n_cosmo, precision);
    double* jac = reinterpret_cast<double*>(base + gws);
    double* cl_ws = reinterpret_cast<double*>(base + gws + al256(sizeof(double) * per * NDIR * (size_t)n_cosmo));
    grad_run(geo, h, params, n_cosmo, precision, cl ? cl : cl_ws, jac, ws, c, st, gamma_dir);
    vjp_contract_kernel<<<n_cosmo, 256, 0, st>>>(jac, vbar, (int)per, grad);
    return;
  }
  GradBatch gb;
  memset(&gb, 0, sizeof(gb));
  gb.gamma_dir = gamma_dir;
  gb.n_items = n_cosmo;
  gb.precision = precision;
  gb.params = params;
  gb.geo = geo;
  GeoHeader hb = h;
  hb.na = h.na * n_cosmo;
  size_t o = 0;
  gb.tab = reinterpret_cast<TabD*>(base + o);
  o += al256(sizeof(TabD) * (size_t)n_cosmo);
  gb.ptt = reinterpret_cast<double*>(base + o);
  o += ptt_bytes(precision) * n_cosmo;
  gb.rowg = reinterpret_cast<float*>(base + o);
  o += rows_bytes(hb, precision);
  gb.kernf = reinterpret_cast<float*>(base + o);
  o += kern_bytes(hb, precision);
  gb.cpart = reinterpret_cast<float*>(base + o);
  o += al256(sizeof(float) * (size_t)vjp_chunks(h.na) * per * n_cosmo);
  gb.gpart = reinterpret_cast<double*>(base + o);
  o += al256(sizeof(double) * (size_t)vjp_chunks(h.na) * NDIR * n_cosmo);
  gb.kbar = reinterpret_cast<float*>(base + o);
  o += al256(sizeof(float) * (size_t)h.n_tr * h.na * n_cosmo);
  gb.kpart = reinterpret_cast<double*>(base + o);
  o += al256(sizeof(double) * (size_t)kv_chunks(h.na) * NDIR * n_cosmo);
  gb.krev_owner = reinterpret_cast<int*>(base + o);
  o += al256(sizeof(int) * 9 * (size_t)kv_chunks(h.na));
  gb.krev_ranges = reinterpret_cast<int*>(base + o);
  o += al256(sizeof(int) * 8 * (size_t)h.na);
  gb.cl_count = reinterpret_cast<unsigned*>(base + o);
  o += al256(sizeof(unsigned) * (size_t)n_cosmo);
  gb.gnode = gnode_bytes(n_cosmo, precision) ? reinterpret_cast<double*>(base + o) : nullptr;
  gb.vjp_rev = (vbar && grad) ? 1 : 0;
  gb.krev_u = gb.vjp_rev && krev_uniform_ok(h);
  gb.krev_wbase = krev_wbase(h);
  gb.n_wl = h.n_wl;
  gb.kern_rest = h.n_nc > 0 || h.special_bias;
  gb.vbar = vbar;
  gb.grad = grad;
  gb.cl = cl;
  gb.na = h.na;
  gb.n_tr = h.n_tr;
  gb.n_cls = h.n_cls;
  gb.n_ell = h.n_ell;
  gb.n_split = 1;
  gb.physics_or = h.physics;
  launch_grad_front(gb, c, st, stages);
  if (cl && vbar && grad) {
    // the caller's cotangent: one pass gives the partial C_ell and the product
    gb.vjp_cl = 1;
    launch_vjp32_grad(gb, st, stages);
    return;
  }
  if (cl && (stages & GS_PRODUCT)) launch_vjp32_cl(gb, st);
  if (vbar && grad) launch_vjp32_grad(gb, st, stages);
}

void grad_run(const GeoHeader* geo, const GeoHeader& h, const double* params, int n_cosmo, int precision,
              double* cl, double* jac, void* ws, const ConstTables* c, cudaStream_t st, int gamma_dir,
              const int* seg_in, int* seg_out) {
  GradBatch gb;
  memset(&gb, 0, sizeof(gb));
  gb.gamma_dir = gamma_dir;
  gb.seg_in = seg_in;
  gb.seg_out = seg_out;
  gb.n_items = n_cosmo;
  gb.precision = precision;
  gb.params = params;
  gb.geo = geo;
  GeoHeader hb = h;
  hb.na = h.na * n_cosmo;
  char* base = static_cast<char*>(ws);
  size_t o = 0;
  gb.tab = reinterpret_cast<TabD*>(base + o);
  o += al256(sizeof(TabD) * (size_t)n_cosmo);
  if (precision == JCG_FP32C) gb.ptt = reinterpret_cast<double*>(base + o);
  o += ptt_bytes(precision) * n_cosmo;
  if (precision == JCG_FP32C) gb.rowg = reinterpret_cast<float*>(base + o);
  else gb.rowd = reinterpret_cast<double*>(base + o);
  o += rows_bytes(hb, precision);
  if (precision == JCG_FP32C) gb.kernf = reinterpret_cast<float*>(base + o);
  else gb.kernd = reinterpret_cast<double*>(base + o);
  o += kern_bytes(hb, precision);
  gb.part = reinterpret_cast<double*>(base + o);
  o += al256(sizeof(double) * (size_t)grad_n_split(h, n_cosmo, precision) * n_cosmo * h.n_cls * h.n_ell * (NDIR + 1));
  gb.gnode = gnode_bytes(n_cosmo, precision) ? reinterpret_cast<double*>(base + o) : nullptr;
  gb.cl = cl;
  gb.jac = jac;
  gb.na = h.na;
  gb.n_tr = h.n_tr;
  gb.n_cls = h.n_cls;
  gb.n_ell = h.n_ell;
  gb.n_split = grad_n_split(h, n_cosmo, precision);
  gb.physics_or = h.physics;
  gb.listed = 0;
  gb.items = nullptr;
  launch_grad(gb, c, st);
}

// ----------------------------------------------------- ragged requests -----
// Listed form: every request has its own geometry; the workspace holds the
// GradItem array, then per request its tables, rows, kernels, a-split partial
// sums and (when the caller gave none) its C_ell and Jacobian.
static size_t grad_item_bytes(const GeoHeader& h, int n_split, bool own_cl, bool own_jac, int precision) {
  const size_t per = (size_t)h.n_cls * h.n_ell;
  size_t o = al256(sizeof(TabD));
  o += ptt_bytes(precision);
  o += rows_bytes(h, precision);
  o += kern_bytes(h, precision);
  o += al256(sizeof(double) * (size_t)n_split * per * (NDIR + 1));
  if (own_cl) o += al256(sizeof(double) * per);
  if (own_jac) o += al256(sizeof(double) * per * NDIR);
  return o;
}

int grad_listed_auto_split(const GradReq* r, int n, int precision) {
  int max_ell = 0, max_cls = 0, min_na = 1 << 30;
  for (int i = 0; i < n; ++i) {
    max_ell = max(max_ell, r[i].h->n_ell);
    max_cls = max(max_cls, r[i].h->n_cls);
    min_na = min(min_na, r[i].h->na);
  }
  const int lt = grad_tile(precision, max_ell, max_cls);
  long ctas = 0;
  for (int i = 0; i < n; ++i) ctas += (r[i].h->n_ell + lt - 1) / lt;
  int ns = (int)((2 * 152 + ctas - 1) / ctas);
  const int ta = grad_chunk(precision, max_cls);
  const int max_ns = (min_na + ta - 1) / ta;
  if (ns > max_ns) ns = max_ns;
  return ns < 1 ? 1 : ns;
}

// per request of the vector-Jacobian form: tables, rows and kernels with
// tangents, the product kernels' partials, C_ell (when the caller gave none)
// and the cotangent
static size_t vjp_item_bytes(const GeoHeader& h, bool own_cl) {
  const size_t per = (size_t)h.n_cls * h.n_ell;
  size_t o = al256(sizeof(TabD));
  o += ptt_bytes(JCG_FP32C);
  o += rows_bytes(h, JCG_FP32C);
  o += kern_bytes(h, JCG_FP32C);
  o += vjp32_item_bytes(h);
  if (own_cl) o += al256(sizeof(double) * per);
  o += al256(sizeof(double) * per);
  return o;
}

size_t grad_listed_bytes(const GradReq* r, int n, int n_split, int precision, bool vjp) {
  size_t o = al256(sizeof(GradItem) * (size_t)n);
  for (int i = 0; i < n; ++i)
    o += vjp ? vjp_item_bytes(*r[i].h, !r[i].cl) : grad_item_bytes(*r[i].h, n_split, !r[i].cl, !r[i].jac, precision);
  return o + gnode_bytes(n, precision) + (vjp ? al256(sizeof(unsigned) * (size_t)n) : 0);
}

cudaError_t grad_run_listed(GradReq* r, int n, int n_split, int precision, void* ws, const ConstTables* c,
                            cudaStream_t st, bool vjp, GradBatch* gb_out) {
  static thread_local std::vector<GradItem> host;
  host.resize(n);
  char* base = static_cast<char*>(ws);
  GradItem* dev_items = reinterpret_cast<GradItem*>(base);
  size_t o = al256(sizeof(GradItem) * (size_t)n);
  GradBatch gb;
  memset(&gb, 0, sizeof(gb));
  gb.gamma_dir = -1;
  for (int i = 0; i < n; ++i) {
    const GeoHeader& h = *r[i].h;
    const size_t per = (size_t)h.n_cls * h.n_ell;
    GradItem& it = host[i];
    memset(&it, 0, sizeof(it));
    it.params = r[i].params;
    it.geo = r[i].geo;
    it.tab = reinterpret_cast<TabD*>(base + o);
    o += al256(sizeof(TabD));
    if (precision == JCG_FP32C) it.ptt = reinterpret_cast<double*>(base + o);
    o += ptt_bytes(precision);
    if (precision == JCG_FP32C) it.rowg = reinterpret_cast<float*>(base + o);
    else it.rowd = reinterpret_cast<double*>(base + o);
    o += rows_bytes(h, precision);
    if (precision == JCG_FP32C) it.kernf = reinterpret_cast<float*>(base + o);
    else it.kernd = reinterpret_cast<double*>(base + o);
    o += kern_bytes(h, precision);
    if (vjp) {
      const size_t nch = (size_t)vjp_chunks(h.na);
      it.cpart = reinterpret_cast<float*>(base + o);
      o += al256(sizeof(float) * nch * per);
      it.gpart = reinterpret_cast<double*>(base + o);
      o += al256(sizeof(double) * nch * NDIR);
      it.kbar = reinterpret_cast<float*>(base + o);
      o += al256(sizeof(float) * (size_t)h.n_tr * h.na);
      it.kpart = reinterpret_cast<double*>(base + o);
      o += al256(sizeof(double) * (size_t)kv_chunks(h.na) * NDIR);
      if (!r[i].cl) {
        r[i].cl = reinterpret_cast<double*>(base + o);
        o += al256(sizeof(double) * per);
      }
      r[i].vbar = reinterpret_cast<double*>(base + o);
      o += al256(sizeof(double) * per);
      it.vbar = r[i].vbar;
      it.grad = r[i].out + 1;
      it.cl = r[i].cl;
    } else {
      it.part = reinterpret_cast<double*>(base + o);
      o += al256(sizeof(double) * (size_t)n_split * per * (NDIR + 1));
      if (!r[i].cl) {
        r[i].cl = reinterpret_cast<double*>(base + o);
        o += al256(sizeof(double) * per);
      }
      if (!r[i].jac) {
        r[i].jac = reinterpret_cast<double*>(base + o);
        o += al256(sizeof(double) * per * NDIR);
      }
      it.cl = r[i].cl;
      it.jac = r[i].jac;
    }
    gb.na = max(gb.na, h.na);
    gb.n_tr = max(gb.n_tr, h.n_tr);
    gb.n_cls = max(gb.n_cls, h.n_cls);
    gb.n_ell = max(gb.n_ell, h.n_ell);
    gb.physics_or |= h.physics;
  }
  // through the calling thread's pinned staging ring: no wait on the stream
  const cudaError_t e = stage_h2d(dev_items, host.data(), sizeof(GradItem) * (size_t)n, st);
  if (e != cudaSuccess) return e;
  gb.n_items = n;
  gb.listed = 1;
  gb.precision = precision;
  gb.items = dev_items;
  gb.n_split = vjp ? 1 : n_split;
  gb.vjp_rev = vjp ? 1 : 0;
  gb.gnode = gnode_bytes(n, precision) ? reinterpret_cast<double*>(base + o) : nullptr;
  o += gnode_bytes(n, precision);
  if (vjp) gb.cl_count = reinterpret_cast<unsigned*>(base + o);
  if (vjp) {
    launch_grad_front(gb, c, st);
    launch_vjp32_cl(gb, st);
  } else {
    launch_grad(gb, c, st);
  }
  if (gb_out) *gb_out = gb;
  return cudaSuccess;
}

}  // namespace jcg
