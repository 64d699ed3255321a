/* libjcg — GB300-native angular power spectra with jax_cosmo's semantics.
 *
 * C ABI of the CUDA library behind jax_cosmo_gb300.  Every entry point:
 *   - takes caller-owned DEVICE pointers (the library never frees them) and a
 *     cudaStream_t, and is asynchronous on that stream (no host synchronisation
 *     unless stated);
 *   - returns 0 (JCG_OK) or a negative JCG_ERR_* code, never aborts; the text of
 *     the last error of the calling thread is in jcg_last_error_string();
 *   - validates shapes, parameter values and workspace sizes on the host before
 *     launching anything.
 *
 * Reference citations are paths in the jax_cosmo project (DifferentiableUniverse
 * Initiative/jax_cosmo), file:line.
 *
 * Layout conventions
 *   params  [n_cosmo][8] float64: Omega_c, Omega_b, h, n_s, sigma8, Omega_k, w0, wa
 *           (the pytree leaves of Cosmology, core.py:98-108)
 *   cl      [n_cosmo][n_cls][n_ell] float64, pairs (i <= j) in the order of
 *           angular_cl._get_cl_ordering (angular_cl.py:15-25)
 *   sparse covariance [n_cls][n_cls][n_ell] float64 (sparse.py:1-11 format)
 *   dense covariance  [n_cls*n_ell][n_cls*n_ell] float64, index p*n_ell + l
 *           (angular_cl.py:158-162)
 */
#ifndef JCG_H
#define JCG_H

#include <stddef.h>
#include <stdint.h>

#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JCG_ABI_VERSION 3
#define JCG_MAX_TRACERS 16
#define JCG_MAX_PAIRS (JCG_MAX_TRACERS * (JCG_MAX_TRACERS + 1) / 2)
#define JCG_MAX_ELL 4096
#define JCG_MAX_LIMBER 4096

/* status codes */
#define JCG_OK 0
#define JCG_ERR_ARG -1         /* null pointer, bad enum, bad count */
#define JCG_ERR_SHAPE -2       /* inconsistent sizes */
#define JCG_ERR_ODD_N -3       /* Simpson rule needs an even N (scipy/integrate.py:193) */
#define JCG_ERR_VALUE -4       /* NaN / out-of-domain parameter */
#define JCG_ERR_WORKSPACE -5   /* workspace or geometry buffer too small */
#define JCG_ERR_CUDA -6        /* a CUDA call failed */
#define JCG_ERR_UNSUPPORTED -7 /* option the reference also rejects (NotImplementedError) */
#define JCG_ERR_TIMEOUT -8     /* a bounded device wait gave up */
#define JCG_ERR_ABI -9         /* descriptor abi_version mismatch */

/* tracer kinds: probes.WeakLensing (probes.py:132) / probes.NumberCounts (probes.py:226) */
#define JCG_TRACER_WL 0
#define JCG_TRACER_NC 1

/* Bias models (bias.py:10-57): the NumberCounts galaxy bias, or the
 * WeakLensing intrinsic-alignment amplitude of the NLA model (probes.py:102-129;
 * JCG_BIAS_NONE on a WeakLensing tracer: no intrinsic alignment).
 *   CONSTANT    b                                 constant_linear_bias
 *   INV_GROWTH  b / D(a)                          inverse_growth_linear_bias
 *   DES_Y1      A ((1 + z) / (1 + z0))^eta        des_y1_ia_bias
 * with b or A in `bias`, eta and z0 in `bias_eta`, `bias_z0`.  On a
 * NumberCounts tracer JCG_BIAS_NONE means CONSTANT. */
/* n(z) of a tracer: JCG_NZ_SMAIL (nz_a, nz_b, nz_z0, evaluated by the library,
 * redshift.py:61-77) or JCG_NZ_TABLE (any redshift_distribution: the caller
 * evaluates its un-normalised pz_fn at the points jcg_geometry_nz_points lists
 * and passes them to jcg_geometry_build_nz; the library normalises them with
 * simps(pz_fn, 0, zmax, 256) as redshift.py:27-31 does). */
#define JCG_NZ_SMAIL 0
#define JCG_NZ_TABLE 1
#define JCG_NZ_DELTA 2   /* single plane at nz_z0, WeakLensing only (redshift.py:108-122, probes.py:53-64) */

#define JCG_BIAS_NONE 0
#define JCG_BIAS_CONSTANT 1
#define JCG_BIAS_INV_GROWTH 2
#define JCG_BIAS_DES_Y1 3

/* Physics switches: jcg_geometry.physics, and bits 8 and up of the `what` word
 * of jcg_eval_points.  The matter power model (the nonlinear_fn of
 * angular_cl, angular_cl.py:49-98) in the low four bits:
 *   TAKAHASHI2012  power.halofit, prescription "takahashi2012" (the default)
 *   SMITH2003      power.halofit, prescription "smith2003" (power.py:182-198, 226-242)
 *   LINEAR         power.linear_matter_power (power.py:21-53), no halofit
 * and the transfer function (transfer_fn):
 *   NOWIGGLE       transfer.Eisenstein_Hu with type "eisenhu" (transfer.py:99-105),
 *                  the zero-baryon fit without oscillations; unset: "eisenhu_osc";
 * and the growth model (GROWTH_GAMMA below). */
#define JCG_PK_TAKAHASHI2012 0
#define JCG_PK_SMITH2003 1
#define JCG_PK_LINEAR 2
#define JCG_PK_MASK 0x0f
#define JCG_TF_NOWIGGLE 0x10
/* Growth from the growth-rate index gamma, f = Omega_m(a)^gamma
 * (Cosmology(gamma=...), background.py:515-582) instead of the growth ODE.
 * With this bit the parameter arrays hold 9 values per cosmology, the 9th
 * gamma.  The Jacobian columns are the first 8 parameters; dC/dgamma comes
 * from jcg_angular_cl_jacobian_dir with gamma_dir in 0..7.  Ragged requests
 * (jcg_requests_run, 8 parameters per request) reject this bit. */
#define JCG_GROWTH_GAMMA 0x20
#define JCG_PHYSICS_ALL (JCG_PK_MASK | JCG_TF_NOWIGGLE | JCG_GROWTH_GAMMA)

/* arithmetic of the Limber stage */
#define JCG_FP64 0  /* plain: float64 everywhere */
#define JCG_FP32C 1 /* float32 Limber integrand + compensated Simpson sums, float64 tables */

/* One request's tracers and grids (cosmology independent).
 * Replaces the probe/redshift containers consumed by angular_cl
 * (probes.py:132-281, redshift.py:15-77, bias.py:10-22). */
typedef struct jcg_geometry {
  int abi_version;     /* = JCG_ABI_VERSION */
  int n_tracers;       /* total redshift bins over all probes, <= JCG_MAX_TRACERS */
  int n_ell;           /* <= JCG_MAX_ELL */
  int n_limber;        /* Simpson intervals in a (angular_cl.py:96 uses 512); even */
  int n_nodes;         /* 0: Limber grid; > 0: that many caller redshift nodes
                          (jcg_geometry_build_nodes), n_limber ignored */
  double zmax;         /* max over probes of probe zmax (angular_cl.py:63) */
  int kind[JCG_MAX_TRACERS];          /* JCG_TRACER_* */
  double nz_a[JCG_MAX_TRACERS];       /* smail_nz a, b, z0 (redshift.py:75-77) */
  double nz_b[JCG_MAX_TRACERS];
  double nz_z0[JCG_MAX_TRACERS];
  double nz_zmax[JCG_MAX_TRACERS];    /* n(z) normalisation range (redshift.py:30) */
  double probe_zmax[JCG_MAX_TRACERS]; /* lensing integral upper limit (probes.py:25) */
  double bias[JCG_MAX_TRACERS];       /* bias amplitude b or A (bias.py:21, 38, 56) */
  double mult[JCG_MAX_TRACERS];       /* WeakLensing multiplicative bias m (probes.py:207) */
  double noise[JCG_MAX_TRACERS];      /* per-bin noise power (probes.py:210-223, 274-281) */
  int bias_kind[JCG_MAX_TRACERS];     /* JCG_BIAS_*: galaxy bias (NC) or NLA bias (WL) */
  double bias_eta[JCG_MAX_TRACERS];   /* des_y1_ia_bias eta, z0 (bias.py:55-57) */
  double bias_z0[JCG_MAX_TRACERS];
  int nz_kind[JCG_MAX_TRACERS];       /* JCG_NZ_* */
  int physics;                        /* JCG_PK_* | JCG_TF_* | JCG_GROWTH_GAMMA (0: the reference defaults) */
} jcg_geometry;

/* ------------------------------------------------------------- misc ---- */
int jcg_abi_version(void);
const char* jcg_last_error_string(void);

/* -------------------------------------------------------- geometry ---- */
/* Size in bytes of the cosmology-independent geometry buffer for g. */
int jcg_geometry_size(const jcg_geometry* g, size_t* bytes);

/* Build the geometry buffer: Limber nodes in a (angular_cl.py:96), n(z)
 * normalisation (redshift.py:27-31), n(z) on the Limber and lensing grids
 * (probes.py:44-51, 87), interpolation segments of every table lookup
 * (scipy/interpolate.py:34-59), WeakLensing ell factors (probes.py:73).
 * ell_dev: [n_ell] float64 device array. */
int jcg_geometry_build(const jcg_geometry* g, const double* ell_dev, void* geo_dev,
                       size_t geo_bytes, cudaStream_t stream);

/* Same tables on caller-given redshift nodes z_dev [g->n_nodes] instead of the
 * Limber grid: the radial kernels of probes.WeakLensing.kernel /
 * NumberCounts.kernel at arbitrary z (probes.py:188-208, 260-272).  Only the
 * cosmology-table and tracer-kernel stages are meaningful on such a geometry;
 * jcg_geometry_size covers it. */
/* Tabulated n(z) (JCG_NZ_TABLE tracers).  The points where the reference
 * evaluates each tracer's pz_fn, tracer after tracer: 257 normalisation points
 * linspace(0, zmax, 257) (redshift.py:30), the n_a Limber nodes (or the
 * caller's z nodes, z_nodes_dev, when n_nodes > 0), and for a WeakLensing
 * tracer n_a x 257 lensing points linspace(z_n, probe zmax, 257)
 * (probes.py:51).  *count receives the number of points; z_out_dev (may be
 * NULL for a size query) receives them.  jcg_geometry_build_nz then takes the
 * un-normalised pz_fn values at those points (entries of JCG_NZ_SMAIL tracers
 * are ignored) and builds the geometry like jcg_geometry_build(_nodes). */
int jcg_geometry_nz_points(const jcg_geometry* g, const double* z_nodes_dev, double* z_out_dev,
                           size_t* count, cudaStream_t stream);
int jcg_geometry_build_nz(const jcg_geometry* g, const double* ell_dev, const double* z_nodes_dev,
                          const double* pz_dev, size_t pz_count, void* geo_dev, size_t geo_bytes,
                          cudaStream_t stream);
int jcg_geometry_build_nodes(const jcg_geometry* g, const double* ell_dev, const double* z_dev,
                             void* geo_dev, size_t geo_bytes, cudaStream_t stream);

/* ------------------------------------------------------ angular_cl ---- */
/* Workspace bytes for n_cosmo cosmologies on geometry g. */
int jcg_workspace_size(const jcg_geometry* g, int n_cosmo, int precision, size_t* bytes);

/* C_ell of n_cosmo cosmologies sharing one geometry, one fused pipeline:
 * background tables -> halofit rows -> tracer kernels -> Limber integral.
 * Replaces angular_cl.angular_cl (angular_cl.py:49-98) with the default
 * transfer_fn = Eisenstein_Hu (transfer.py:10) and nonlinear_fn = halofit
 * takahashi2012 (power.py:144).  cl_dev: [n_cosmo][n_cls][n_ell]. */
int jcg_angular_cl(const jcg_geometry* g, const void* geo_dev, const double* params_dev,
                   int n_cosmo, int precision, double* cl_dev, void* workspace,
                   size_t workspace_bytes, cudaStream_t stream);

/* jcg_angular_cl for callers that cannot allocate device memory.
 * No counterpart in the reference (jax_cosmo lets XLA manage all buffers).
 * Some callers cannot call cudaMalloc: code running inside another
 * framework's device callback (an XLA custom call or a JAX host callback)
 * where the framework has already reserved most of the GPU memory and offers
 * no way to request scratch, so a cudaMalloc there fails or stalls every
 * stream of the device.  This entry point takes the same inputs and output as
 * jcg_angular_cl but no workspace: its scratch is one fixed array of
 * JCG_NOALLOC_SCRATCH_BYTES in the library's static device memory, which
 * every GPU that loads libjcg holds until the process exits.  Requests whose
 * scratch (jcg_workspace_size) exceeds that size are rejected with
 * JCG_ERR_WORKSPACE before anything runs.  The call allocates nothing.
 * The first call on a device looks up the array's device address and, if no
 * earlier call did, builds the constant tables, synchronising `stream` once;
 * make that first call before any stream capture.  All calls share the one
 * array: calls whose kernels can overlap on the GPU (different streams without
 * an ordering between them, or several host threads) race on it, so order
 * them on one stream.  Every scratch value is written before it is read within
 * a call, so the contents left by the previous call do not matter. */
#define JCG_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int jcg_angular_cl_noalloc(const jcg_geometry* g, const void* geo_dev, const double* params_dev,
                           int n_cosmo, int precision, double* cl_dev, cudaStream_t stream);

/* jcg_angular_cl with host buffers: params_host [n_cosmo][8] (9 with the
 * gamma growth) and cl_host [n_cosmo][n_cls][n_ell] in host memory, the
 * boundary of a caller that holds no device arrays (a JAX host callback
 * binding angular_cl.py:49-98, a CPU sampler).  The parameters are copied in
 * on `stream`; the Limber stage runs over at most JCG_HOST_SLICES ranges of
 * cosmologies (from 2048 cosmologies on: the first three quarters, then the
 * last quarter) and each range's C_ell are copied out on a copy stream of the
 * calling thread while the next range computes; `stream` then waits for the
 * last copy, so cl_host is complete once `stream` is synchronised.  With
 * pinned host memory (cudaHostAlloc / cudaHostRegister) the call returns
 * without waiting; with pageable memory the copies wait for the GPU.  The
 * workspace (jcg_host_workspace_size) is jcg_angular_cl's plus device copies
 * of the parameters and the C_ell. */
#define JCG_HOST_SLICES 4
int jcg_host_workspace_size(const jcg_geometry* g, int n_cosmo, int precision, size_t* bytes);
int jcg_angular_cl_host(const jcg_geometry* g, const void* geo_dev, const double* params_host, int n_cosmo,
                        int precision, double* cl_host, void* workspace, size_t workspace_bytes,
                        cudaStream_t stream);

/* Stage entry points of the same pipeline (for tests and for callers that keep
 * tables resident).  The workspace is the one of jcg_angular_cl. */
int jcg_stage_cosmo_tables(const jcg_geometry* g, const double* params_dev, int n_cosmo,
                           int precision, void* workspace, size_t workspace_bytes,
                           cudaStream_t stream);
int jcg_stage_halofit_rows(const jcg_geometry* g, const void* geo_dev, const double* params_dev,
                           int n_cosmo, int precision, void* workspace, size_t workspace_bytes,
                           cudaStream_t stream);
int jcg_stage_tracer_kernels(const jcg_geometry* g, const void* geo_dev, const double* params_dev,
                             int n_cosmo, int precision, void* workspace, size_t workspace_bytes,
                             cudaStream_t stream);
int jcg_stage_limber(const jcg_geometry* g, const void* geo_dev, const double* params_dev,
                     int n_cosmo, int precision, double* cl_dev, void* workspace,
                     size_t workspace_bytes, cudaStream_t stream);

/* Derivatives of angular_cl with respect to the 8 Cosmology leaves:
 * jac_dev [n_cosmo][n_cls][n_ell][8] = dC_ij(l)/d(Omega_c, Omega_b, h, n_s,
 * sigma8, Omega_k, w0, wa), and cl_dev (may be NULL) the C_ell themselves.
 * Replaces jax.grad / jax.jacfwd through angular_cl (angular_cl.py:49-98;
 * README.md:14-27): the vector-Jacobian product of a likelihood is
 * sum_ij,l v_ij(l) jac_ij(l).  Tables are differentiated forward (tangents),
 * the Limber integrand by a reverse sweep; all recomputed from params_dev.
 * precision: JCG_FP64 everywhere, or JCG_FP32C (float64 tables, root find and
 * moments; float32 lensing kernels and Limber integrand + reverse sweep with
 * compensated a-sums). */
int jcg_jacobian_workspace_size(const jcg_geometry* g, int n_cosmo, int precision, size_t* bytes);
int jcg_angular_cl_jacobian(const jcg_geometry* g, const void* geo_dev, const double* params_dev,
                            int n_cosmo, int precision, double* cl_dev, double* jac_dev, void* workspace,
                            size_t workspace_bytes, cudaStream_t stream);
/* The same with tangent direction gamma_dir (0..7) carrying the derivative
 * with respect to gamma (JCG_GROWTH_GAMMA, background.py:515-582) instead of
 * that parameter's: jac_dev[...][gamma_dir] = dC_ij(l)/dgamma, the other 7
 * columns as above.  gamma_dir = -1 is jcg_angular_cl_jacobian. */
int jcg_angular_cl_jacobian_dir(const jcg_geometry* g, const void* geo_dev, const double* params_dev,
                                int n_cosmo, int precision, int gamma_dir, double* cl_dev, double* jac_dev,
                                void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* Vector-Jacobian product of angular_cl, the form jax.grad takes for a scalar
 * function of C_ell (README.md:14-27; angular_cl.py:49-98):
 *   grad_dev [n_cosmo][8] = sum_{p,l} cl_bar_dev[b][p][l] dC_p(l)/dtheta
 * over the 8 Cosmology leaves (gamma_dir as in jcg_angular_cl_jacobian_dir),
 * and cl_dev (may be NULL) the C_ell themselves.  The matching adjoint entry
 * point of angular_cl: a likelihood's backward pass passes d logL / dC_ell
 * as cl_bar.  JCG_FP32C: tables with tangents, then the Limber integrand's
 * reverse sweep weighted by sum_p cl_bar_p(l) M_p(a) and summed over ell,
 * projected on the 8 directions once per Limber node in a; the Jacobian is
 * never formed.  JCG_FP64: the FP64 Jacobian contracted with cl_bar. */
int jcg_vjp_workspace_size(const jcg_geometry* g, int n_cosmo, int precision, size_t* bytes);
int jcg_angular_cl_vjp(const jcg_geometry* g, const void* geo_dev, const double* params_dev, int n_cosmo,
                       int precision, int gamma_dir, const double* cl_bar_dev, double* cl_dev, double* grad_dev,
                       void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* jcg_angular_cl_jacobian in FP64 with the branch of the halofit root find
 * exposed.  The reference finds the non-linear scale with an interpolation
 * whose segment is an argmin over the sigma^2(R) table (power.py:112-115,
 * scipy/interpolate.py:34-59), so C_ell is piecewise smooth in the parameters
 * and jax.grad / jax.hessian differentiate the piece of the evaluation point
 * (the argmin is locally constant).  seg_out [n_cosmo][na] (may be NULL)
 * receives each Limber node's segment (na = n_limber + 1); seg_in (may be
 * NULL) imposes segments instead of finding them, so that parameter points
 * near a base point are evaluated on the base point's piece -- the
 * second-derivative form of jax.hessian (README.md:27) takes central
 * differences of the exact gradient on that piece.  The gamma growth is not
 * supported here (JCG_ERR_UNSUPPORTED). */
int jcg_angular_cl_jacobian_branch(const jcg_geometry* g, const void* geo_dev, const double* params_dev,
                                   int n_cosmo, const int* seg_in_dev, int* seg_out_dev, double* cl_dev,
                                   double* jac_dev, void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* ------------------------------------------------ ragged requests ------ */
/* A list of requests, each with its own geometry (tracers, n(z), ell grid)
 * and cosmology, computed in one launch sequence: the continuous-batching form
 * of a serving loop.  Replaces a Python loop of angular_cl calls
 * (angular_cl.py:49-98) over sampler chains with different probes and ell,
 * each followed by jax.grad of the chain's likelihood (likelihood.py:9-61 with
 * the covariance held fixed, docs/notebooks/jax-cosmo-intro.ipynb).
 * Every request's result depends only on its own inputs: the same alone and
 * in any mix.  mode (with precision JCG_FP64 or JCG_FP32C):
 *   JCG_REQ_CL: cl -> C_ell [n_cls][n_ell];
 *   JCG_REQ_JACOBIAN: jac -> dC_ell/dtheta [n_cls][n_ell][8], cl (may be NULL);
 *   JCG_REQ_LOGLIKE_GRAD: out -> [9] = logL = -r^T P r / 2 with r = C_ell - data
 *     and its gradient -(dC/dtheta)^T P r over the 8 Cosmology leaves; data
 *     [n_cls*n_ell] in (cls, ell) order, prec [n_ell][n_cls][n_cls] the inverse
 *     covariance blocks; cl optional output (NULL: workspace).  FP64: from
 *     the Jacobian (jac an optional output); JCG_FP32C: C_ell, then the
 *     product of the cotangent -P r with dC/dtheta (jcg_angular_cl_vjp's
 *     kernels), jac not written.
 * The request tables reach the device through a pinned staging ring of the
 * calling host thread, so the call does not wait for the stream (it waits
 * only if 16 earlier calls of the thread are still queued). */
#define JCG_REQ_CL 0
#define JCG_REQ_JACOBIAN 1
#define JCG_REQ_LOGLIKE_GRAD 2
#define JCG_MAX_REQUESTS 65536

typedef struct {
  const jcg_geometry* g;   /* host description of the request's geometry */
  const void* geo_dev;     /* its device buffer (jcg_geometry_build) */
  const double* params_dev;/* 8 parameters */
  double* cl_dev;
  double* jac_dev;
  const double* data_dev;
  const double* prec_dev;
  double* out_dev;
} jcg_request;

/* Workspace for n requests: *bytes_min with no a-splits of the Jacobian,
 * *bytes_full with the splits that fill the GPU for small batches;
 * jcg_requests_run uses as many splits as ws_bytes allows. */
int jcg_requests_workspace_size(const jcg_request* reqs, int n, int mode, int precision,
                                size_t* bytes_min, size_t* bytes_full);
int jcg_requests_run(const jcg_request* reqs, int n, int mode, int precision, void* workspace,
                     size_t workspace_bytes, cudaStream_t stream);

/* Copy stage outputs for cosmology `index` out of a workspace (device to device).
 * what: 0 chi table [256], 1 growth table [128], 2 scalars [32],
 *       3 halofit rows [na][24] (FP64; with JCG_FP32C only chi, growth, k_nl,
 *       n_eff, C, dchi/da and the Limber weight are written), 4 radial
 *       kernels [n_tracers][na] (FP64 workspaces; with JCG_FP32C the kernels
 *       are kept as float and this copy is refused),
 *       5 P(k, a = 1) k^3 on the halofit k grid [257], 6 sigma^2(R) without
 *       the growth factor [256] (power.py:93-111). */
int jcg_workspace_read(const jcg_geometry* g, int n_cosmo, int precision, const void* workspace,
                       int index, int what, double* out_dev, size_t out_count,
                       cudaStream_t stream);

/* Pointwise table functions at n (k, a) points for n_cosmo cosmologies
 * (out [n_cosmo][n]).  what:
 *   0 radial_comoving_distance(a)   background.py:199-242
 *   1 growth_factor(a)              background.py:371-398
 *   2 H(a)                          background.py:129-142
 *   3 dchioverda(a)                 background.py:270-294
 *   4 Eisenstein_Hu(k)              transfer.py:10-156
 *   5 linear_matter_power(k, a)     power.py:21-53
 *   6 nonlinear_matter_power(k, a)  power.py:265-272 (halofit)
 *   7 k_nl(a)  8 n_eff(a)  9 C(a)   power.py:86-141
 *  10 transverse_comoving_distance(a)  background.py:297-344
 *  11 angular_diameter_distance(a)     background.py:347-368
 *  12 a_of_chi(chi), chi in a_dev      background.py:245-267
 *  13 growth_rate(a)                   background.py:401-440 (ODE growth)
 * in the low byte of `what`; bits 8 and up hold the physics switches
 * (JCG_PK_* | JCG_TF_* | JCG_GROWTH_GAMMA) << 8; with JCG_GROWTH_GAMMA params
 * holds 9 values per cosmology and 1 / 13 are the gamma growth factor / rate.
 * Needs a workspace of jcg_workspace_size(g=NULL -> tables only). */
int jcg_eval_points(const double* params_dev, int n_cosmo, const double* a_dev,
                    const double* k_dev, int n, int what, double* out_dev, void* workspace,
                    size_t workspace_bytes, cudaStream_t stream);
int jcg_eval_workspace_size(int n_cosmo, size_t* bytes);

/* -------------------------------------------------- covariance ---------- */
/* Gaussian covariance of n_cosmo C_ell sets: angular_cl.py:120-163.
 * ell_dev [n_ell] (n_ell >= 2, np.gradient), cl_signal_dev [n_cosmo][n_cls][n_ell]
 * with n_cls = n_tracers (n_tracers + 1) / 2.  The noise added to the signal is
 * cl_noise_dev [n_cls][n_ell] when given (shared by all cosmologies), else the
 * auto-spectrum noise of noise_cl (angular_cl.py:101-117) built from
 * tracer_noise_dev [n_tracers] when given, else zero.
 * sparse != 0: out [n_cosmo][n_cls][n_cls][n_ell]; else dense
 * [n_cosmo][N][N], N = n_cls*n_ell. */
int jcg_gaussian_covariance(const double* ell_dev, int n_ell, int n_tracers,
                            const double* cl_signal_dev, const double* cl_noise_dev,
                            const double* tracer_noise_dev, int n_cosmo, double f_sky, int sparse,
                            double* out_dev, cudaStream_t stream);

/* Gaussian log-likelihood with a covariance in the sparse block format
 * (likelihood.py:9-61; sparse.py:295-366): per-ell blocks factored by
 * Cholesky in float64.  data/mu [n_cosmo][n_cls*n_ell] (p*n_ell + l),
 * cov [n_cosmo][n_cls][n_cls][n_ell]; out [n_cosmo].  Returns
 * -0.5 * (r^T C^-1 r - logdet) when include_logdet, as likelihood.py:61.
 * status_dev [n_cosmo] (may be NULL): 0 ok, 2 a block is not positive
 * definite (out = NaN).  alpha_dev [n_cosmo][n_cls*n_ell] (may be NULL)
 * receives C^-1 (mu - data), from which the derivatives follow:
 * d logL / d mu = -alpha, d logL / d C = (alpha alpha^T + C^-1) / 2. */
int jcg_gaussian_loglike_sparse(const double* data_dev, const double* mu_dev, const double* cov_dev,
                                int n_cosmo, int n_cls, int n_ell, int include_logdet,
                                double* out_dev, int* status_dev, double* alpha_dev, void* workspace,
                                size_t workspace_bytes, cudaStream_t stream);
int jcg_loglike_workspace_size(int n_cosmo, int n_cls, int n_ell, size_t* bytes);

/* Dense covariance [n_cosmo][N][N], N = n_cls*n_ell, in the layout of
 * angular_cl.py:158-162.  A device pass checks that every n_ell x n_ell block
 * is diagonal; such matrices are factored per ell like the sparse form (the
 * same value as likelihood.py:242-248 for either inverse_method, up to
 * rounding).  status_dev [n_cosmo]: 0 ok, 1 not block-diagonal in ell
 * (out = NaN: factor it densely instead), 2 not positive definite. */
int jcg_gaussian_loglike_dense(const double* data_dev, const double* mu_dev, const double* cov_dev,
                               int n_cosmo, int n_cls, int n_ell, int include_logdet,
                               double* out_dev, int* status_dev, double* alpha_dev, void* workspace,
                               size_t workspace_bytes, cudaStream_t stream);

/* sparse.inv / sparse.slogdet of (n, n, ndiag) block-diagonal matrices
 * (sparse.py:295-366), float64, one matrix; n <= JCG_SPARSE_MAX_N.  Each
 * diagonal's n x n matrix is inverted in place by Gauss-Jordan elimination
 * with partial pivoting. */
#define JCG_SPARSE_MAX_N 160
int jcg_sparse_inv(const double* sparse_dev, int n, int ndiag, double* out_dev, cudaStream_t stream);
/* sparse.inv of n_batch matrices [n_batch][n][n][ndiag] in one launch (the
 * batched form the likelihood's derivative and the serving loop use). */
int jcg_sparse_inv_batched(const double* sparse_dev, int n_batch, int n, int ndiag, double* out_dev,
                           cudaStream_t stream);
/* work_dev: 2*ndiag float64 of caller-owned scratch (per-diagonal partials). */
int jcg_sparse_slogdet(const double* sparse_dev, int n, int ndiag, double* sign_dev,
                       double* logdet_dev, double* work_dev, cudaStream_t stream);
/* sparse.to_dense (sparse.py:52-68): (n, m, d) -> (n*d, m*d). */
int jcg_sparse_to_dense(const double* sparse_dev, int n, int m, int ndiag, double* out_dev,
                        cudaStream_t stream);
/* Products with a block-diagonal operand, float64 (sparse.py:140-292):
 *   sparse_dot_sparse  A (n, m, d) @ B (m, p, d) -> (n, p, d)          sparse.py:236-260
 *   sparse_dot_dense   A (n, m, d) @ D (m d, k) -> (n d, k)             sparse.py:164-182
 *   dense_dot_sparse   D (r, n d) @ A (n, m, d) -> (r, m d)             sparse.py:210-233
 *   dense_dot_sparse_dot_dense  X (r, n d) @ Y (n, m, d) @ Z (m d, k) -> (r, k)
 *                      sparse.py:263-292; work_dev holds n d k float64 (Y @ Z). */
int jcg_sparse_dot_sparse(const double* a_dev, int n, int m, int p, int ndiag, const double* b_dev,
                          double* out_dev, cudaStream_t stream);
int jcg_sparse_dot_dense(const double* a_dev, int n, int m, int ndiag, const double* dense_dev, int k,
                         double* out_dev, cudaStream_t stream);
int jcg_dense_dot_sparse(const double* dense_dev, int r, const double* a_dev, int n, int m, int ndiag,
                         double* out_dev, cudaStream_t stream);
int jcg_dense_dot_sparse_dot_dense(const double* x_dev, int r, const double* y_dev, int n, int m, int ndiag,
                                   const double* z_dev, int k, double* work_dev, double* out_dev,
                                   cudaStream_t stream);
/* sparse.dot(A, v) / sparse.dot(v, A) for sparse A (n, m, d) (sparse.py:71-137). */
int jcg_sparse_dot_vec(const double* sparse_dev, int n, int m, int ndiag, const double* v_dev,
                       int transpose, double* out_dev, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* JCG_H */
