// Shared definitions of the Jacobian kernels (jcg_grad.cu: FP64 and the
// common stages; jcg_grad32.cu: the FP32 compensated Limber and lensing stages).
#pragma once

#include "jcg_dual.cuh"

namespace jcg {

typedef Dual<1> D1;
typedef Dual<NDIR> D8;

__device__ __forceinline__ D1 mk1(double v, double d) {
  D1 r;
  r.v = v;
  r.d[0] = d;
  return r;
}

typedef DualF<NDIR> F8;

// interpolation (scipy/interpolate.py:55-59) with a dual table fp
__device__ __forceinline__ D1 interp_d1(double x, const double* xp, const double* fv, const double* fd,
                                        int2 sg) {
  const D1 f0 = mk1(fv[sg.x], fd[sg.x]), f1 = mk1(fv[sg.y], fd[sg.y]);
  const D1 a = (f1 - f0) / (xp[sg.y] - xp[sg.x]);
  const D1 b = f0 - a * xp[sg.x];
  return a * x + b;
}



// DualF<8> from a value and 8 double tangents at stride `stride`
__device__ __forceinline__ F8 f8_of(double v, const double* d, int stride) {
  F8 r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < NDIR; ++i) r.d[i] = (float)d[i * stride];
  return r;
}

constexpr double TWO_PI2_G = 2.0 * (PI * PI);
constexpr double C2_G = C_KMS * C_KMS;
constexpr double LN10_G = 2.302585092994046;

// ------------------------------------------------------------ dual tables ---
struct TabD {
  double sv[NSCAL];
  double sd[NDIR][NSCAL];
  double chiv[NCHI];
  double chid[NDIR][NCHI];
  double gv[NGROW];
  double gd[NDIR][NGROW];
  double sigv[NRT];
  double sigd[NDIR][NRT];
  double pk3v[NKH];
  double pk3d[NDIR][NKH];
  double pad[7];
  // fp32c Jacobian only: float copies for the FP32 stages
  float c32[NDIR + 1][NCHI];   // chi (row 0) and its tangents
  float s32[NDIR + 1][NCHI];   // segment slopes (chi[i+1] - chi[i]) / (a[i+1] - a[i]) and tangents
  float pk3df[NKH][NDIR];      // P(k) k^3 tangents, node-major
  float padf[8];
  // the Eisenstein-Hu inputs of the FP32 integrand (EHg order) and their
  // tangents [NET][NDIR], formed once per cosmology for the Limber kernels
  float ehv[16];
  float eht[88];   // NET x NDIR
  float padg[8];
  float wq3f[NKH + 15];        // simpson_kh[i] * P(k_i) k_i^3 / (2 pi^2), float; padded to 64 bytes
  // fp32c row stage: the scalars, chi, growth and sigma^2(R) tables above as
  // float-pair values and float tangents (node-major, rows of 8)
  float2 svF[NSCAL];
  float sdF[NSCAL][NDIR];
  float2 chiF[NCHI];
  float chidF[NCHI][NDIR];
  float2 gF[NGROW];
  float gdF[NGROW][NDIR];
  float2 sigF[NRT];
  float sigdF[NRT][NDIR];
};
static_assert(sizeof(TabD) % 64 == 0, "TabD alignment");

// per-node inputs of the Limber integrand (node_fb), value + 8 tangents
enum NodeA { A_CHIC = 0, A_G, A_KNL, A_BETA, A_ALPHA, A_AN, A_BN, A_LCF3, A_F1, A_F2, A_GAM, A_NU, A_MU, A_U, NA_IN };
constexpr int NROWD = NA_IN * (NDIR + 1);  // [NA_IN] values then [NDIR][NA_IN] tangents
// per-cosmology inputs of the integrand
enum NodeC { C_KEQ = 0, C_SH, C_BETAC, C_ALPHAC, C_ALPHAB, C_BETAB, C_BETANODE, C_KSILK, C_FB, C_FC, C_NS, C_PKNORM,
             C_AGAM, C_NWQ, NC_IN };
__device__ __constant__ const int kNodeCScalar[NC_IN] = {S_K_EQ,  S_SH_D,      S_BETA_C,  S_ALPHA_C,
                                                         S_ALPHA_B, S_BETA_B, S_BETA_NODE, S_K_SILK,
                                                         S_FB,    S_FC,        S_NS,      S_PKNORM,
                                                         S_AGAM,  S_NWQ};

// FP32 rows of the compensated Limber Jacobian, per node: NROWV values (the
// 16 of the forward FP32 row in Row32 order, slot 16 = the Limber weight u,
// padding), then the tangents [NGT][NDIR] of the independent inputs below
// (chi_c and k_nl raw, the others in the units of their Row32 slot).
enum GTan { T_CHIC = 0, T_D2FAC, T_KNL, T_BETAN, T_ALPHAN, T_AN, T_3F1, T_F2, T_BN, T_LG2CF3, T_3MG,
            T_NUN, T_MUN, T_U, NGT };
constexpr int F_U = NROW32;
constexpr int NROWV = NROW32 + 4;
// Taylor tables of the fp32c moments, per cosmology: values as float pairs
// [NKH + 1][NTAYLOR] (in the first NPTTV doubles), then tangents float
// [NKH + 1][NTAYLOR][NDIR]
constexpr int NPTTV = (NKH + 1) * NTAYLOR;
constexpr size_t PTT_STRIDE = ((size_t)NPTTV * 8 + (size_t)NPTTV * NDIR * 4 + 255) / 256 * 256 / 8;  // doubles
__device__ __forceinline__ float* ptt_tangents(double* p) { return reinterpret_cast<float*>(p + NPTTV); }
__device__ __forceinline__ const float* ptt_tangents(const double* p) {
  return reinterpret_cast<const float*>(p + NPTTV);
}
constexpr int NROWG = NROWV + NGT * NDIR;  // 132 floats
// per-cosmology Eisenstein-Hu inputs of the FP32 integrand with tangents
enum ETan { E_KEQ = 0, E_SH, E_C18BC, E_C142AC, E_ALPHAB, E_BETAB, E_BETANODE, E_LG2KSILK, E_FB, E_FC,
            E_NS3, NET };
static_assert(NET * NDIR <= 88, "TabD::eht holds the Eisenstein-Hu tangents");
// transfer type "eisenhu": alpha_gamma and (T_cmb / 2.7)^2 / (Omega_m h) in
// the slots of k_eq and 1.8 beta_c (which that fit does not use)
constexpr int E_AGAM = E_KEQ, E_NWQ = E_C18BC;

// One (cosmology, geometry) pair of a Jacobian batch.  FP64: rowd / kernd;
// FP32C: rowg / kernf.
struct GradItem {
  const double* params;   // 8 parameters
  const GeoHeader* geo;
  TabD* tab;
  double* rowd;    // [na][NROWD]
  double* kernd;   // [n_tr][na][NDIR + 1]
  float* rowg;     // [na][NROWG]
  float* kernf;    // [n_tr][na][NDIR + 1]
  double* ptt;     // FP32C: Taylor prefix tables (values, then float tangents)
  double* part;    // [n_split][n_cls][n_ell][NDIR + 1] partial sums over a
  double* cl;      // [n_cls][n_ell] (may be NULL)
  double* jac;     // [n_cls][n_ell][NDIR]
  // vector-Jacobian product (fp32c): the cotangent of C_ell [n_cls][n_ell],
  // per a-chunk partial C_ell [n_chunk][n_cls][n_ell] and gradients
  // [n_chunk][NDIR], the gradient out [NDIR]
  const double* vbar;
  float* cpart;
  double* gpart;
  double* grad;
  // reverse form of the lensing integral (vector-Jacobian product): the
  // cotangents of the WeakLensing kernels [n_tr][na] and per node-chunk
  // gradient partials [n_kchunk][NDIR]
  float* kbar;
  double* kpart;
};

// node chunks of the reverse lensing kernels
constexpr int KV_NODES = 16;
__host__ __device__ inline int kv_chunks(int na) { return (na + KV_NODES - 1) / KV_NODES; }

// a-chunks of the vector-Jacobian product kernels: at most VJ_TA Limber
// nodes per CTA, the chunks balanced
constexpr int VJ_TA = 32;
__host__ __device__ inline int vjp_chunks(int na) { return (na + VJ_TA - 1) / VJ_TA; }
__host__ __device__ inline int vjp_tav(int na) {
  const int nc = vjp_chunks(na);
  return (na + nc - 1) / nc;
}

// Uniform form: one geometry, per-item pointers from strides.  Listed form:
// items[] (ragged requests), sizes below are the maxima over the items.
struct GradBatch {
  int n_items;
  int listed;
  int precision;
  const GradItem* items;
  const double* params;
  const GeoHeader* geo;
  TabD* tab;
  double* rowd;
  double* kernd;
  float* rowg;
  float* kernf;
  double* ptt;
  double* part;
  double* cl;
  double* jac;
  double* gnode;  // fp32c, small batches: the table kernel's node values, per item GNODE_STRIDE doubles
  int na, n_tr, n_cls, n_ell, n_split;
  int physics_or;  // OR of the items' physics switches (selects kernel variants)
  int gamma_dir;   // tangent direction carrying d/dgamma instead of its parameter's (-1: none)
  // FP64 uniform form: the halofit root find's interpolation segment per
  // (item, Limber node), packed as ind | (side > 0) << 16: recorded into
  // seg_out, or imposed from seg_in (the branch of another parameter point)
  const int* seg_in;
  int* seg_out;
  // uniform form of the vector-Jacobian product buffers (see GradItem)
  const double* vbar;
  float* cpart;
  double* gpart;
  double* grad;
  float* kbar;
  double* kpart;
  // 1: vector-Jacobian form with the lensing integral in reverse: the kernel
  // stage writes no tangents of the WeakLensing shear integral, the product
  // kernel writes their cotangents, the reverse lensing kernel adds theirs
  int vjp_rev;
  // uniform form of the reverse lensing integral (one geometry, one lensing
  // group, no single-plane n(z), 1..8 WeakLensing tracers): lanes over
  // cosmologies.  krev_wbase: the first chi table segment a Limber node or
  // lensing point can fall in; krev_owner: [kv_chunks][9] the segment ranges
  // of the 8 warps per node chunk; kern_rest: NumberCounts or NLA terms (the
  // per-cosmology kernel stage still runs for them)
  int krev_u, krev_wbase, n_wl, kern_rest;
  int* krev_owner;
  int* krev_ranges;  // [na][8] each warp's points of a node, jlo | jhi << 16
  // 1: the cotangent does not depend on C_ell (given by the caller), so the
  // product kernel also writes the chunks' partial C_ell (no forward pass)
  int vjp_cl;
  // per item: chunk CTAs done with their partial C_ell (the last one adds
  // them up and resets the count)
  unsigned* cl_count;
};

// fp32c batches run the table kernel's per-node evaluations in
// grad_nodes_kernel (one node per thread) and hand them over in the table
// kernel's shared-memory layout, each node array packed as [n] float-pair
// values then [NDIR][n] float tangents (5 n doubles): chi right-hand sides at
// nodes and midpoints, growth coefficients qa, ra, qm, rm (in a span that the
// table kernel reuses for the growth scan's scratch), the Romberg integrand,
// then exp(n_s ln k) T(k)^2 on the P(k) grid (read from global memory).
constexpr int GNODE_MAX_ITEMS = 128;  // up to this many cosmologies the scalars run on half warps
constexpr int GNODE_FN = 0;
constexpr int GNODE_FM = 5 * NCHI;
constexpr int GNODE_QR = 10 * NCHI;
constexpr int GNODE_QR_SPAN = 3200;  // >= 4 x 5 x NGROW and the growth scan's scratch
constexpr int GNODE_FR = GNODE_QR + GNODE_QR_SPAN;
constexpr int GNODE_U = (GNODE_FR + 5 * NROMB + 1) / 2 * 2;  // 16-byte aligned
constexpr size_t GNODE_STRIDE = (size_t)(GNODE_U + 5 * NKH + 31) / 32 * 32;
static_assert(GNODE_QR_SPAN >= 20 * NGROW, "growth coefficients fit their span");

__device__ __forceinline__ GradItem grad_item(const GradBatch& gb, int i) {
  if (gb.listed) return gb.items[i];
  GradItem r;
  const size_t per = (size_t)gb.n_cls * gb.n_ell;
  r.params = gb.params + (size_t)param_stride(gb.physics_or) * i;
  r.geo = gb.geo;
  r.tab = gb.tab + i;
  r.rowd = gb.rowd ? gb.rowd + (size_t)i * gb.na * NROWD : nullptr;
  r.kernd = gb.kernd ? gb.kernd + (size_t)i * gb.n_tr * gb.na * (NDIR + 1) : nullptr;
  r.rowg = gb.rowg ? gb.rowg + (size_t)i * gb.na * NROWG : nullptr;
  r.kernf = gb.kernf ? gb.kernf + (size_t)i * gb.n_tr * gb.na * (NDIR + 1) : nullptr;
  r.ptt = gb.ptt ? gb.ptt + (size_t)i * PTT_STRIDE : nullptr;
  r.cl = gb.cl ? gb.cl + (size_t)i * per : nullptr;
  r.jac = gb.jac ? gb.jac + (size_t)i * per * NDIR : nullptr;
  r.part = gb.part ? gb.part + (size_t)i * gb.n_split * per * (NDIR + 1) : nullptr;
  const int nch = vjp_chunks(gb.na);
  r.vbar = gb.vbar ? gb.vbar + (size_t)i * per : nullptr;
  r.cpart = gb.cpart ? gb.cpart + (size_t)i * nch * per : nullptr;
  r.gpart = gb.gpart ? gb.gpart + (size_t)i * nch * NDIR : nullptr;
  r.grad = gb.grad ? gb.grad + (size_t)i * NDIR : nullptr;
  r.kbar = gb.kbar ? gb.kbar + (size_t)i * gb.n_tr * gb.na : nullptr;
  r.kpart = gb.kpart ? gb.kpart + (size_t)i * kv_chunks(gb.na) * NDIR : nullptr;
  return r;
}

// n(z) b(z) H(a) of a NumberCounts tracer (probes.py:94), or the NLA
// intrinsic-alignment term n(z) b(z) H(a) (-C_1 rho_crit Omega_m / D(a)) of a
// WeakLensing tracer (probes.py:102-129), with its tangent in direction dir;
// a = z2a(z), D = growth_factor(a) from the tangent tables.
static __device__ __noinline__ void bias_term_d1(const TabD* tb, const ConstTables* c, const GeoHeader* geo, int t,
                                          int dir, double awl, double z, double nzl, bool nla, double* kv,
                                          double* kd) {
  BgT<D1> bg;
  bg.Om = mk1(tb->sv[S_OMEGA_M], tb->sd[dir][S_OMEGA_M]);
  bg.Ok = mk1(tb->sv[S_OMEGA_K], tb->sd[dir][S_OMEGA_K]);
  bg.Ode = mk1(tb->sv[S_OMEGA_DE], tb->sd[dir][S_OMEGA_DE]);
  bg.w0 = mk1(tb->sv[S_W0], tb->sd[dir][S_W0]);
  bg.wa = mk1(tb->sv[S_WA], tb->sd[dir][S_WA]);
  const D1 H = H0 * xsqrt(esqrT(bg, awl, log(awl), (D1*)nullptr));
  D1 D = mk1(1.0, 0.0);
  const int kind = geo->bias_kind[t];
  if (nla || kind == JCG_BIAS_INV_GROWTH) {
    const int2 sg = interp_segment_inc(awl, c->atab_grow, NGROW, logspace_guess(awl, NGROW));
    const D1 f0 = mk1(tb->gv[sg.x], tb->gd[dir][sg.x]), f1 = mk1(tb->gv[sg.y], tb->gd[dir][sg.y]);
    const D1 sl = (f1 - f0) / (c->atab_grow[sg.y] - c->atab_grow[sg.x]);
    D = xfmin(xfmax(sl * awl + (f0 - sl * c->atab_grow[sg.x]), 0.0), 1.0);
  }
  D1 b;
  if (kind == JCG_BIAS_INV_GROWTH) b = geo->bias[t] / D;
  else b = mk1(bias_at(geo, t, z, 1.0), 0.0);
  D1 k = nzl * b * H;
  if (nla) k = k * (-IA_C1_RHOCRIT * bg.Om / D);
  *kv = k.v;
  *kd = k.d[0];
}

// stages of the fp32c gradient pipeline (a mask selects some, for timing):
// tables (scalars, node evaluations, tables, moments), rows, radial kernels,
// the product kernel, the reverse lensing kernel with the gradient sum
enum GradStage : unsigned { GS_TABLES = 1, GS_ROWS = 2, GS_KERNELS = 4, GS_PRODUCT = 8, GS_REVERSE = 16, GS_ALL = 31 };

// FP32 compensated stages (jcg_grad32.cu)
void launch_grad_kern32(const GradBatch& gb, const ConstTables* c, cudaStream_t st);
void launch_grad_limber32(const GradBatch& gb, const ConstTables* c, cudaStream_t st);
// vector-Jacobian product (jcg_vjp32.cu): C_ell of the items into their cl,
// and the product with their cotangents vbar into their grad
void launch_vjp32_cl(const GradBatch& gb, cudaStream_t st);
void launch_vjp32_grad(const GradBatch& gb, cudaStream_t st, unsigned stages = GS_ALL);
// uniform reverse lensing: the shear kernels' values (lanes over cosmologies)
void launch_kernval32u(const GradBatch& gb, cudaStream_t st);
int krev_wbase(const GeoHeader& h);
bool krev_uniform_ok(const GeoHeader& h);
// tables, rows and radial kernels with tangents (the stages before Limber)
void launch_grad_front(const GradBatch& gb, const ConstTables* c, cudaStream_t st, unsigned stages = GS_ALL);
int grad_limber32_tile(int n_ell, int n_cls);
int grad_limber32_chunk(int n_cls);

}  // namespace jcg
