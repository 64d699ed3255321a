// extern "C" entry points of libjcg: validation, buffer layouts, launches.
//
// Every function validates on the host, launches asynchronously on the given
// stream and returns a JCG_* status; nothing here aborts.  The error text of the
// last failure of the calling thread is kept in a thread-local buffer.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "jcg_internal.cuh"
#include "jcg_grad.cuh"

namespace jcg {
void launch_covariance(const double* ell, int n_ell, int n_tr, const double* cl,
                       const double* cl_noise, const double* tr_noise, int n_cosmo, double f_sky,
                       int sparse, double* out, cudaStream_t st);
void launch_loglike(const double* data, const double* mu, const double* cov, int n_cosmo, int n_cls,
                    int n_ell, int include_logdet, int dense, double* out, int* status,
                    double* partial, int* structure, double* alpha, cudaStream_t st);
void launch_sparse_inv(const double* sp, int n_batch, int n, int nd, double* out, cudaStream_t st);
void launch_sparse_dot_sparse(const double* a, const double* b, int n, int m, int p, int nd, double* c,
                              cudaStream_t st);
void launch_sparse_dot_dense(const double* a, int n, int m, int nd, const double* d, int K, double* out,
                             cudaStream_t st);
void launch_dense_dot_sparse(const double* d, int R, const double* a, int n, int m, int nd, double* out,
                             cudaStream_t st);
void launch_gemm_f64(const double* x, const double* t, int M, int Kd, int N, double* c, cudaStream_t st);
void launch_sparse_slogdet(const double* sp, int n, int nd, double* sign_part, double* ld_part,
                           double* sign_out, double* ld_out, cudaStream_t st);
void launch_sparse_to_dense(const double* sp, int n, int m, int nd, double* out, cudaStream_t st);
void launch_sparse_dot_vec(const double* sp, int n, int m, int nd, const double* v, int transpose,
                           double* out, cudaStream_t st);
}  // namespace jcg

using namespace jcg;

// ------------------------------------------------------------- errors -------
static thread_local char g_err[512] = "";

static int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

static int cuda_check(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(JCG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return JCG_OK;
}

// --------------------------------------------------- device constants -------
// One set of constant grids per device, in static device memory (no allocation).
static __device__ ConstTables g_const;
static std::mutex g_init_mu;
static bool g_init_done[64];
static ConstTables* g_const_ptr[64];

static int const_tables(ConstTables** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(JCG_ERR_CUDA, "cudaGetDevice failed");
  if (dev < 0 || dev >= 64) return fail(JCG_ERR_CUDA, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_init_mu);
  if (!g_init_done[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_const);
    if (e != cudaSuccess) return fail(JCG_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    ConstTables* c = static_cast<ConstTables*>(p);
    cudaStream_t s;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(JCG_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    launch_const_init(c, s);
    e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) return fail(JCG_ERR_CUDA, "constant tables: %s", cudaGetErrorString(e));
    g_const_ptr[dev] = c;
    g_init_done[dev] = true;
  }
  *out = g_const_ptr[dev];
  return JCG_OK;
}

// ------------------------------------------------ pinned staging ring -------
// Small host tables (the item arrays of ragged requests) reach the device
// through pinned host memory: a copy from pageable memory may wait for the
// stream before it returns, a copy from pinned memory does not.  Each host
// thread owns a ring of slots; a slot is reused once the event recorded after
// its copy has completed, which only waits when a whole ring of copies is
// still queued on the GPU.  The buffers are kept until the process exits.
namespace jcg {
namespace {
constexpr int STAGE_SLOTS = 16;
struct StageSlot {
  void* buf = nullptr;
  size_t cap = 0;
  cudaEvent_t ev = nullptr;
  bool used = false;
};
struct StageRing {
  StageSlot slot[STAGE_SLOTS];
  int next = 0;
};
}  // namespace

cudaError_t stage_h2d(void* dst_dev, const void* src_host, size_t bytes, cudaStream_t st) {
  static thread_local StageRing ring;
  StageSlot& s = ring.slot[ring.next];
  ring.next = (ring.next + 1) % STAGE_SLOTS;
  cudaError_t e;
  if (s.used && (e = cudaEventSynchronize(s.ev)) != cudaSuccess) return e;
  if (!s.ev && (e = cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming)) != cudaSuccess) return e;
  if (s.cap < bytes) {
    if (s.buf) cudaFreeHost(s.buf);
    s.buf = nullptr;
    s.cap = 0;
    const size_t cap = bytes < 65536 ? 65536 : bytes * 2;
    if ((e = cudaHostAlloc(&s.buf, cap, cudaHostAllocDefault)) != cudaSuccess) return e;
    s.cap = cap;
  }
  memcpy(s.buf, src_host, bytes);
  if ((e = cudaMemcpyAsync(dst_dev, s.buf, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
  if ((e = cudaEventRecord(s.ev, st)) != cudaSuccess) return e;
  s.used = true;
  return cudaSuccess;
}
}  // namespace jcg

// ----------------------------------------------------------- geometry -------
static int64_t align8(int64_t v) { return (v + 7) & ~int64_t(7); }  // 64-byte units

static int make_header(const jcg_geometry* g, GeoHeader* h) {
  const int n_nodes = g ? g->n_nodes : 0;
  if (!g) return fail(JCG_ERR_ARG, "geometry is NULL");
  if (g->abi_version != JCG_ABI_VERSION)
    return fail(JCG_ERR_ABI, "geometry abi_version %d, library %d", g->abi_version, JCG_ABI_VERSION);
  if (g->n_tracers < 1 || g->n_tracers > JCG_MAX_TRACERS)
    return fail(JCG_ERR_SHAPE, "n_tracers = %d (1..%d)", g->n_tracers, JCG_MAX_TRACERS);
  if (g->n_ell < 1 || g->n_ell > JCG_MAX_ELL)
    return fail(JCG_ERR_SHAPE, "n_ell = %d (1..%d)", g->n_ell, JCG_MAX_ELL);
  if (n_nodes == 0) {
    if (g->n_limber < 2 || g->n_limber > JCG_MAX_LIMBER)
      return fail(JCG_ERR_SHAPE, "n_limber = %d (2..%d)", g->n_limber, JCG_MAX_LIMBER);
    if (g->n_limber % 2 == 1)
      return fail(JCG_ERR_ODD_N, "N must be an even integer (n_limber = %d)", g->n_limber);
  } else if (n_nodes < 0 || n_nodes > 1 << 20) {
    return fail(JCG_ERR_SHAPE, "n_z = %d", n_nodes);
  }
  if (!(g->zmax > 0.0) || !isfinite(g->zmax)) return fail(JCG_ERR_VALUE, "zmax = %g", g->zmax);
  if ((g->physics & ~JCG_PHYSICS_ALL) != 0 || pk_model(g->physics) > JCG_PK_LINEAR)
    return fail(JCG_ERR_UNSUPPORTED, "physics = 0x%x", g->physics);
  memset(h, 0, sizeof(*h));
  h->physics = g->physics;
  h->magic = GEO_MAGIC;
  h->n_tr = g->n_tracers;
  h->n_ell = g->n_ell;
  h->n_limber = n_nodes ? 0 : g->n_limber;
  h->na = n_nodes ? n_nodes : g->n_limber + 1;
  h->custom_nodes = n_nodes ? 1 : 0;
  h->zmax = g->zmax;
  h->dx_limber = n_nodes ? 0.0 : (1.0 - 1.0 / (1.0 + g->zmax)) / g->n_limber;
  double zmx = 0.0;
  for (int t = 0; t < g->n_tracers; ++t) {
    const int k = g->kind[t];
    if (k != JCG_TRACER_WL && k != JCG_TRACER_NC) return fail(JCG_ERR_ARG, "tracer %d: kind %d", t, k);
    const double vals[] = {g->nz_a[t], g->nz_b[t], g->nz_z0[t], g->nz_zmax[t], g->bias[t], g->mult[t], g->noise[t]};
    for (double v : vals)
      if (!isfinite(v)) return fail(JCG_ERR_VALUE, "tracer %d has a non-finite parameter", t);
    if (!(g->nz_z0[t] > 0.0)) return fail(JCG_ERR_VALUE, "tracer %d: z0 = %g", t, g->nz_z0[t]);
    if (!(g->nz_zmax[t] > 0.0)) return fail(JCG_ERR_VALUE, "tracer %d: zmax = %g", t, g->nz_zmax[t]);
    h->kind[t] = k;
    h->nz_a[t] = g->nz_a[t];
    h->nz_b[t] = g->nz_b[t];
    h->nz_z0[t] = g->nz_z0[t];
    h->nz_zmax[t] = g->nz_zmax[t];
    h->bias[t] = g->bias[t];
    int bk = g->bias_kind[t];
    if (bk < JCG_BIAS_NONE || bk > JCG_BIAS_DES_Y1) return fail(JCG_ERR_ARG, "tracer %d: bias_kind %d", t, bk);
    if (k == JCG_TRACER_NC && bk == JCG_BIAS_NONE) bk = JCG_BIAS_CONSTANT;
    if (bk == JCG_BIAS_DES_Y1) {
      if (!isfinite(g->bias_eta[t]) || !isfinite(g->bias_z0[t]) || !(1.0 + g->bias_z0[t] > 0.0))
        return fail(JCG_ERR_VALUE, "tracer %d: des_y1_ia_bias eta = %g, z0 = %g", t, g->bias_eta[t], g->bias_z0[t]);
    }
    if (g->nz_kind[t] != JCG_NZ_SMAIL && g->nz_kind[t] != JCG_NZ_TABLE && g->nz_kind[t] != JCG_NZ_DELTA)
      return fail(JCG_ERR_ARG, "tracer %d: nz_kind %d", t, g->nz_kind[t]);
    if (g->nz_kind[t] == JCG_NZ_DELTA) {
      if (k != JCG_TRACER_WL) return fail(JCG_ERR_ARG, "tracer %d: single-plane n(z) on a NumberCounts tracer", t);
      h->has_delta = 1;
    }
    h->nz_kind[t] = g->nz_kind[t];
    h->bias_kind[t] = bk;
    h->bias_eta[t] = bk == JCG_BIAS_DES_Y1 ? g->bias_eta[t] : 0.0;
    h->bias_z0[t] = bk == JCG_BIAS_DES_Y1 ? g->bias_z0[t] : 0.0;
    if ((k == JCG_TRACER_WL && bk != JCG_BIAS_NONE) || bk >= JCG_BIAS_INV_GROWTH) h->special_bias = 1;
    h->mult[t] = g->mult[t];
    h->noise[t] = g->noise[t];
    h->probe_zmax[t] = g->probe_zmax[t];
    if (k == JCG_TRACER_WL) {
      h->n_wl++;
      const double pz = g->probe_zmax[t];
      if (!(pz > 0.0) || !isfinite(pz)) return fail(JCG_ERR_VALUE, "tracer %d: probe_zmax = %g", t, pz);
      int grp = -1;
      for (int q = 0; q < h->n_groups; ++q)
        if (h->group_zmax[q] == pz) grp = q;
      if (grp < 0) {
        grp = h->n_groups++;
        h->group_zmax[grp] = pz;
      }
      h->group[t] = grp;
      if (pz > zmx) zmx = pz;
    } else {
      h->n_nc++;
      h->group[t] = -1;
    }
  }
  int p = 0;
  for (int i = 0; i < h->n_tr; ++i)
    for (int j = i; j < h->n_tr; ++j) {
      h->pair_i[p] = i;
      h->pair_j[p] = j;
      ++p;
    }
  h->n_cls = p;
  // offsets (8-byte units), sections aligned to 64 bytes
  const int na = h->na;
  int64_t o = align8((int64_t)((sizeof(GeoHeader) + 7) / 8));
  auto take = [&](int64_t n) {
    const int64_t r = o;
    o = align8(o + n);
    return r;
  };
  h->off_a = take(na);
  h->off_z = take(na);
  h->off_wsimp = take(na);
  h->off_awl = take(na);
  h->off_seg_chi = take(na);
  h->off_seg_grow = take(na);
  h->off_seg_chiwl = take(na);
  h->off_nzl = take((int64_t)h->n_tr * na);
  h->off_ell = take(h->n_ell);
  h->off_ellfac = take((int64_t)h->n_tr * h->n_ell);
  h->off_lg2ellh = take(h->n_ell);
  h->off_kh4 = take(2 * (int64_t)h->n_ell);
  h->off_ef32 = take(((int64_t)h->n_tr * h->n_ell + 1) / 2);
  const int64_t half = ((int64_t)na * NZP + 1) / 2;  // 4-byte arrays in 8-byte units
  for (int q = 0; q < h->n_groups; ++q) {
    h->off_ap[q] = take((int64_t)na * NZP);
    h->off_segp[q] = take((int64_t)na * NZP);
    h->off_q32[q] = take(half);
    h->off_dx32[q] = take(half);
  }
  for (int t = 0; t < h->n_tr; ++t)
    if (h->kind[t] == JCG_TRACER_WL) {
      h->off_W[t] = take((int64_t)na * NZP);
      h->off_W32[t] = take(half);
    }
  h->off_qwl32 = take((na + 1) / 2);
  h->off_dxwl32 = take((na + 1) / 2);
  h->total = o;
  // n(z) points of tabulated tracers: normalisation grid, nodes, lensing grid (WL)
  int64_t np_ = 0;
  for (int t = 0; t < h->n_tr; ++t) {
    h->nzp_off[t] = np_;
    np_ += NZP + na + (h->kind[t] == JCG_TRACER_WL ? (int64_t)na * NZP : 0);
  }
  h->nzp_total = np_;
  (void)zmx;
  return JCG_OK;
}

// ---------------------------------------------------------- workspace -------
struct WsLayout {
  size_t ctab, rows64, rows32, kern, u32, kern32, total;
};

static size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

static WsLayout ws_layout(const GeoHeader* h, int n_cosmo, int precision) {
  WsLayout L;
  size_t o = 0;
  L.ctab = o;
  o = align256(o + sizeof(CosmoTab) * (size_t)n_cosmo);
  const size_t na = h ? (size_t)h->na : 0;
  const size_t ntr = h ? (size_t)h->n_tr : 0;
  L.rows64 = o;
  o = align256(o + sizeof(double) * NROW64 * na * n_cosmo);
  L.rows32 = o;
  if (precision == JCG_FP32C) o = align256(o + sizeof(float) * NROW32 * na * n_cosmo);
  L.kern = o;
  o = align256(o + sizeof(double) * ntr * na * n_cosmo);
  // fp32c: float copies of the Limber weight and the radial kernels (what
  // the Limber kernel reads, contiguous)
  L.u32 = o;
  if (precision == JCG_FP32C) o = align256(o + sizeof(float) * na * n_cosmo);
  L.kern32 = o;
  if (precision == JCG_FP32C) o = align256(o + sizeof(float) * ntr * na * n_cosmo);
  L.total = o;
  return L;
}

static int check_common(const double* params, int n_cosmo, int precision, const void* ws,
                        size_t ws_bytes, size_t need) {
  if (!params) return fail(JCG_ERR_ARG, "params is NULL");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  if (precision != JCG_FP64 && precision != JCG_FP32C) return fail(JCG_ERR_ARG, "precision = %d", precision);
  if (!ws) return fail(JCG_ERR_ARG, "workspace is NULL");
  if (ws_bytes < need) return fail(JCG_ERR_WORKSPACE, "workspace %zu bytes, need %zu", ws_bytes, need);
  if (((uintptr_t)ws) % 256 != 0) return fail(JCG_ERR_ARG, "workspace must be 256-byte aligned");
  return JCG_OK;
}

static Batch make_batch(const GeoHeader* h, const void* geo, const double* params, int n_cosmo,
                        int precision, void* ws, double* cl) {
  const WsLayout L = ws_layout(h, n_cosmo, precision);
  char* base = static_cast<char*>(ws);
  Batch b;
  memset(&b, 0, sizeof(b));
  b.n_items = n_cosmo;
  b.listed = 0;
  b.items = nullptr;
  b.params = params;
  b.geo = static_cast<const GeoHeader*>(geo);
  b.ctab = reinterpret_cast<CosmoTab*>(base + L.ctab);
  b.rows64 = reinterpret_cast<double*>(base + L.rows64);
  b.rows32 = precision == JCG_FP32C ? reinterpret_cast<float*>(base + L.rows32) : nullptr;
  b.kern = reinterpret_cast<double*>(base + L.kern);
  b.u32 = precision == JCG_FP32C && h ? reinterpret_cast<float*>(base + L.u32) : nullptr;
  b.kern32 = precision == JCG_FP32C && h ? reinterpret_cast<float*>(base + L.kern32) : nullptr;
  b.cl = cl;
  b.precision = precision;
  b.max_na = h ? h->na : 0;
  b.max_ell = h ? h->n_ell : 0;
  b.max_cls = h ? h->n_cls : 0;
  b.max_tr = h ? h->n_tr : 0;
  b.n_wl = h ? h->n_wl : 0;
  b.n_wl_groups = h ? h->n_groups : 0;
  b.chi_wbase = h ? krev_wbase(*h) : 0;
  b.special_bias = h ? h->special_bias : 0;
  b.has_delta = h ? h->has_delta : 0;
  b.physics = h ? h->physics : 0;
  b.physics_or = b.physics;
  return b;
}

static int limber_tile(int n_ell) {
  const int tiles = (n_ell + 31) / 32;
  return (n_ell + tiles - 1) / tiles;
}

// --------------------------------------------------------------- C ABI ------
extern "C" {

int jcg_abi_version(void) { return JCG_ABI_VERSION; }

const char* jcg_last_error_string(void) { return g_err; }

int jcg_geometry_size(const jcg_geometry* g, size_t* bytes) {
  if (!bytes) return fail(JCG_ERR_ARG, "bytes is NULL");
  GeoHeader h;
  const int rc = make_header(g, &h);
  if (rc) return rc;
  *bytes = (size_t)h.total * 8;
  return JCG_OK;
}

// Shared by the geometry builds: z_dev are the caller's redshift nodes (n_nodes > 0),
// pz_dev the tabulated n(z) values (JCG_NZ_TABLE tracers).
static int geometry_build(const jcg_geometry* g, const double* ell_dev, const double* z_dev,
                          const double* pz_dev, size_t pz_count, void* geo_dev, size_t geo_bytes,
                          cudaStream_t stream) {
  GeoHeader h;
  int rc = make_header(g, &h);
  if (rc) return rc;
  if (h.custom_nodes && !z_dev) return fail(JCG_ERR_ARG, "n_nodes > 0: the z nodes are NULL");
  if (!h.custom_nodes && z_dev) return fail(JCG_ERR_ARG, "z nodes given for a Limber-grid geometry");
  if (!ell_dev || !geo_dev) return fail(JCG_ERR_ARG, "ell or geometry buffer is NULL");
  bool table = false;
  for (int t = 0; t < h.n_tr; ++t) table |= h.nz_kind[t] == JCG_NZ_TABLE;
  if (table && (!pz_dev || pz_count < (size_t)h.nzp_total))
    return fail(JCG_ERR_ARG, "tabulated n(z): %zu values given, %lld needed", pz_count,
                (long long)h.nzp_total);
  if (geo_bytes < (size_t)h.total * 8)
    return fail(JCG_ERR_WORKSPACE, "geometry buffer %zu bytes, need %zu", geo_bytes, (size_t)h.total * 8);
  if (((uintptr_t)geo_dev) % 64 != 0) return fail(JCG_ERR_ARG, "geometry buffer must be 64-byte aligned");
  ConstTables* c = nullptr;
  if ((rc = const_tables(&c))) return rc;
  double* geo = static_cast<double*>(geo_dev);
  if (cudaMemcpyAsync(geo + h.off_ell, ell_dev, sizeof(double) * h.n_ell, cudaMemcpyDeviceToDevice,
                      stream) != cudaSuccess)
    return cuda_check("copy ell");
  if (h.custom_nodes && cudaMemcpyAsync(geo + h.off_z, z_dev, sizeof(double) * h.na,
                                        cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
    return cuda_check("copy z");
  launch_geometry_build(h, geo, table ? pz_dev : nullptr, c, stream);
  return cuda_check("geometry build");
}

static int no_table(const jcg_geometry* g) {
  for (int t = 0; g && t < g->n_tracers && t < JCG_MAX_TRACERS; ++t)
    if (g->nz_kind[t] == JCG_NZ_TABLE) return fail(JCG_ERR_ARG, "tabulated n(z): use jcg_geometry_build_nz");
  return JCG_OK;
}

int jcg_geometry_build(const jcg_geometry* g, const double* ell_dev, void* geo_dev, size_t geo_bytes,
                       cudaStream_t stream) {
  if (g && g->n_nodes > 0) return fail(JCG_ERR_ARG, "n_nodes > 0: use jcg_geometry_build_nodes");
  if (int rc = no_table(g)) return rc;
  return geometry_build(g, ell_dev, nullptr, nullptr, 0, geo_dev, geo_bytes, stream);
}

int jcg_geometry_build_nodes(const jcg_geometry* g, const double* ell_dev, const double* z_dev,
                             void* geo_dev, size_t geo_bytes, cudaStream_t stream) {
  if (!g || g->n_nodes < 1) return fail(JCG_ERR_SHAPE, "geometry n_nodes must be > 0");
  if (!z_dev) return fail(JCG_ERR_ARG, "ell, z or geometry buffer is NULL");
  if (int rc = no_table(g)) return rc;
  return geometry_build(g, ell_dev, z_dev, nullptr, 0, geo_dev, geo_bytes, stream);
}

int jcg_geometry_build_nz(const jcg_geometry* g, const double* ell_dev, const double* z_nodes_dev,
                          const double* pz_dev, size_t pz_count, void* geo_dev, size_t geo_bytes,
                          cudaStream_t stream) {
  return geometry_build(g, ell_dev, z_nodes_dev, pz_dev, pz_count, geo_dev, geo_bytes, stream);
}

int jcg_geometry_nz_points(const jcg_geometry* g, const double* z_nodes_dev, double* z_out_dev, size_t* count,
                           cudaStream_t stream) {
  if (!count) return fail(JCG_ERR_ARG, "count is NULL");
  GeoHeader h;
  int rc = make_header(g, &h);
  if (rc) return rc;
  if (!z_out_dev) {
    *count = (size_t)h.nzp_total;
    return JCG_OK;
  }
  if (*count < (size_t)h.nzp_total) return fail(JCG_ERR_WORKSPACE, "%zu points room, %lld needed", *count,
                                                (long long)h.nzp_total);
  if (h.custom_nodes && !z_nodes_dev) return fail(JCG_ERR_ARG, "n_nodes > 0: the z nodes are NULL");
  launch_nz_points(h, h.custom_nodes ? z_nodes_dev : nullptr, z_out_dev, stream);
  *count = (size_t)h.nzp_total;
  return cuda_check("n(z) points");
}

int jcg_workspace_size(const jcg_geometry* g, int n_cosmo, int precision, size_t* bytes) {
  if (!bytes) return fail(JCG_ERR_ARG, "bytes is NULL");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  if (precision != JCG_FP64 && precision != JCG_FP32C) return fail(JCG_ERR_ARG, "precision = %d", precision);
  GeoHeader h;
  const int rc = make_header(g, &h);
  if (rc) return rc;
  *bytes = ws_layout(&h, n_cosmo, precision).total;
  return JCG_OK;
}

static int stage_prepare(const jcg_geometry* g, const void* geo_dev, const double* params,
                         int n_cosmo, int precision, void* ws, size_t ws_bytes, GeoHeader* h,
                         ConstTables** c, bool need_geo, bool need_limber = false) {
  int rc = make_header(g, h);
  if (rc) return rc;
  if (need_limber && h->custom_nodes)
    return fail(JCG_ERR_ARG, "a geometry with caller redshift nodes has no Limber grid");
  if (need_geo && !geo_dev) return fail(JCG_ERR_ARG, "geometry buffer is NULL");
  const WsLayout L = ws_layout(h, n_cosmo, precision);
  if ((rc = check_common(params, n_cosmo, precision, ws, ws_bytes, L.total))) return rc;
  return const_tables(c);
}

int jcg_stage_cosmo_tables(const jcg_geometry* g, const double* params, int n_cosmo, int precision,
                           void* ws, size_t ws_bytes, cudaStream_t stream) {
  GeoHeader h;
  ConstTables* c;
  int rc = stage_prepare(g, nullptr, params, n_cosmo, precision, ws, ws_bytes, &h, &c, false);
  if (rc) return rc;
  const Batch b = make_batch(&h, nullptr, params, n_cosmo, precision, ws, nullptr);
  launch_cosmo_tables(b, c, stream);
  return cuda_check("cosmology tables");
}

int jcg_stage_halofit_rows(const jcg_geometry* g, const void* geo, const double* params, int n_cosmo,
                           int precision, void* ws, size_t ws_bytes, cudaStream_t stream) {
  GeoHeader h;
  ConstTables* c;
  int rc = stage_prepare(g, geo, params, n_cosmo, precision, ws, ws_bytes, &h, &c, true);
  if (rc) return rc;
  const Batch b = make_batch(&h, geo, params, n_cosmo, precision, ws, nullptr);
  launch_halofit_rows(b, c, stream);
  return cuda_check("halofit rows");
}

int jcg_stage_tracer_kernels(const jcg_geometry* g, const void* geo, const double* params,
                             int n_cosmo, int precision, void* ws, size_t ws_bytes,
                             cudaStream_t stream) {
  GeoHeader h;
  ConstTables* c;
  int rc = stage_prepare(g, geo, params, n_cosmo, precision, ws, ws_bytes, &h, &c, true);
  if (rc) return rc;
  const Batch b = make_batch(&h, geo, params, n_cosmo, precision, ws, nullptr);
  launch_tracer_kernels(b, c, stream);
  return cuda_check("tracer kernels");
}

int jcg_stage_limber(const jcg_geometry* g, const void* geo, const double* params, int n_cosmo,
                     int precision, double* cl, void* ws, size_t ws_bytes, cudaStream_t stream) {
  GeoHeader h;
  ConstTables* c;
  int rc = stage_prepare(g, geo, params, n_cosmo, precision, ws, ws_bytes, &h, &c, true, true);
  if (rc) return rc;
  if (!cl) return fail(JCG_ERR_ARG, "cl output is NULL");
  const Batch b = make_batch(&h, geo, params, n_cosmo, precision, ws, cl);
  launch_limber(b, c, limber_tile(h.n_ell), stream);
  return cuda_check("limber");
}

int jcg_angular_cl(const jcg_geometry* g, const void* geo, const double* params, int n_cosmo,
                   int precision, double* cl, void* ws, size_t ws_bytes, cudaStream_t stream) {
  GeoHeader h;
  ConstTables* c;
  int rc = stage_prepare(g, geo, params, n_cosmo, precision, ws, ws_bytes, &h, &c, true, true);
  if (rc) return rc;
  if (!cl) return fail(JCG_ERR_ARG, "cl output is NULL");
  const Batch b = make_batch(&h, geo, params, n_cosmo, precision, ws, cl);
  launch_cosmo_tables(b, c, stream);
  launch_halofit_rows(b, c, stream);
  launch_tracer_kernels(b, c, stream);
  launch_limber(b, c, limber_tile(h.n_ell), stream);
  return cuda_check("angular_cl");
}

int jcg_workspace_read(const jcg_geometry* g, int n_cosmo, int precision, const void* ws, int index,
                       int what, double* out, size_t out_count, cudaStream_t stream) {
  GeoHeader h;
  int rc = make_header(g, &h);
  if (rc) return rc;
  if (!ws || !out) return fail(JCG_ERR_ARG, "NULL pointer");
  if (index < 0 || index >= n_cosmo) return fail(JCG_ERR_SHAPE, "index %d of %d", index, n_cosmo);
  const WsLayout L = ws_layout(&h, n_cosmo, precision);
  const char* base = static_cast<const char*>(ws);
  const CosmoTab* ct = reinterpret_cast<const CosmoTab*>(base + L.ctab) + index;
  const void* src = nullptr;
  size_t count = 0;
  switch (what) {
    case 0: src = ct->chi; count = NCHI; break;
    case 1: src = ct->g; count = NGROW; break;
    case 2: src = ct->s; count = NSCAL; break;
    case 3:
      src = reinterpret_cast<const double*>(base + L.rows64) + (size_t)index * h.na * NROW64;
      count = (size_t)h.na * NROW64;
      break;
    case 4:
      if (precision == JCG_FP32C) return fail(JCG_ERR_UNSUPPORTED, "fp32c workspaces keep the radial kernels as float");
      src = reinterpret_cast<const double*>(base + L.kern) + (size_t)index * h.n_tr * h.na;
      count = (size_t)h.n_tr * h.na;
      break;
    case 5: src = ct->pk3; count = NKH; break;
    case 6: src = ct->sig; count = NRT; break;
    default: return fail(JCG_ERR_ARG, "what = %d", what);
  }
  if (out_count < count) return fail(JCG_ERR_SHAPE, "output holds %zu values, need %zu", out_count, count);
  if (cudaMemcpyAsync(out, src, count * sizeof(double), cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
    return cuda_check("workspace read");
  return JCG_OK;
}

int jcg_eval_workspace_size(int n_cosmo, size_t* bytes) {
  if (!bytes) return fail(JCG_ERR_ARG, "bytes is NULL");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  *bytes = ws_layout(nullptr, n_cosmo, JCG_FP64).total;
  return JCG_OK;
}

int jcg_eval_points(const double* params, int n_cosmo, const double* a, const double* k, int n,
                    int what, double* out, void* ws, size_t ws_bytes, cudaStream_t stream) {
  int rc = check_common(params, n_cosmo, JCG_FP64, ws, ws_bytes, ws_layout(nullptr, n_cosmo, JCG_FP64).total);
  if (rc) return rc;
  if (n < 1) return fail(JCG_ERR_SHAPE, "n = %d", n);
  const int phys = what >> 8;
  if (what < 0 || (what & 0xff) > 13) return fail(JCG_ERR_ARG, "what = %d", what);
  if ((phys & ~JCG_PHYSICS_ALL) != 0 || pk_model(phys) > JCG_PK_LINEAR)
    return fail(JCG_ERR_UNSUPPORTED, "physics = 0x%x", phys);
  const int q = what & 0xff;
  const bool need_a = (q <= 3) || q >= 5;  // a_of_chi (12) takes chi in a_dev
  const bool need_k = (q >= 4 && q <= 6);
  if ((need_a && !a) || (need_k && !k) || !out) return fail(JCG_ERR_ARG, "NULL input or output");
  ConstTables* c;
  if ((rc = const_tables(&c))) return rc;
  Batch b = make_batch(nullptr, nullptr, params, n_cosmo, JCG_FP64, ws, nullptr);
  b.physics = b.physics_or = phys;
  launch_cosmo_tables(b, c, stream);
  launch_eval_points(params, n_cosmo, b.ctab, c, a, k, n, what, out, stream);
  return cuda_check("eval points");
}

int jcg_gaussian_covariance(const double* ell, int n_ell, int n_tr, const double* cl,
                            const double* cl_noise, const double* tr_noise, int n_cosmo, double f_sky,
                            int sparse, double* out, cudaStream_t stream) {
  if (!ell || !cl || !out) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  if (n_tr < 1 || n_tr > JCG_MAX_TRACERS) return fail(JCG_ERR_SHAPE, "n_tracers = %d", n_tr);
  if (n_ell < 2) return fail(JCG_ERR_SHAPE, "np.gradient needs at least 2 ell values (n_ell = %d)", n_ell);
  if (!isfinite(f_sky)) return fail(JCG_ERR_VALUE, "f_sky = %g", f_sky);
  launch_covariance(ell, n_ell, n_tr, cl, cl_noise, tr_noise, n_cosmo, f_sky, sparse ? 1 : 0, out,
                    stream);
  return cuda_check("covariance");
}

int jcg_loglike_workspace_size(int n_cosmo, int n_cls, int n_ell, size_t* bytes) {
  if (!bytes) return fail(JCG_ERR_ARG, "bytes is NULL");
  if (n_cosmo < 1 || n_cls < 1 || n_ell < 1) return fail(JCG_ERR_SHAPE, "bad sizes");
  *bytes = align256(sizeof(double) * 2 * (size_t)n_cosmo * n_ell) + align256(sizeof(int) * 2 * (size_t)n_cosmo);
  return JCG_OK;
}

static int loglike_common(const double* data, const double* mu, const double* cov, int n_cosmo,
                          int n_cls, int n_ell, int include_logdet, int dense, double* out,
                          int* status, double* alpha, void* ws, size_t ws_bytes,
                          cudaStream_t stream) {
  if (!data || !mu || !cov || !out || !ws) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n_cosmo < 1 || n_cls < 1 || n_ell < 1) return fail(JCG_ERR_SHAPE, "bad sizes");
  if (n_cls > 160) return fail(JCG_ERR_SHAPE, "n_cls = %d above the per-ell block limit 160", n_cls);
  size_t need = 0;
  jcg_loglike_workspace_size(n_cosmo, n_cls, n_ell, &need);
  if (ws_bytes < need) return fail(JCG_ERR_WORKSPACE, "workspace %zu bytes, need %zu", ws_bytes, need);
  char* base = static_cast<char*>(ws);
  double* partial = reinterpret_cast<double*>(base);
  int* ints = reinterpret_cast<int*>(base + align256(sizeof(double) * 2 * (size_t)n_cosmo * n_ell));
  int* structure = ints;
  int* st = status ? status : ints + n_cosmo;
  launch_loglike(data, mu, cov, n_cosmo, n_cls, n_ell, include_logdet ? 1 : 0, dense, out, st,
                 partial, structure, alpha, stream);
  return cuda_check("loglike");
}

int jcg_gaussian_loglike_sparse(const double* data, const double* mu, const double* cov, int n_cosmo,
                                int n_cls, int n_ell, int include_logdet, double* out, int* status,
                                double* alpha, void* ws, size_t ws_bytes, cudaStream_t stream) {
  return loglike_common(data, mu, cov, n_cosmo, n_cls, n_ell, include_logdet, 0, out, status,
                        alpha, ws, ws_bytes, stream);
}

int jcg_gaussian_loglike_dense(const double* data, const double* mu, const double* cov, int n_cosmo,
                               int n_cls, int n_ell, int include_logdet, double* out, int* status,
                               double* alpha, void* ws, size_t ws_bytes, cudaStream_t stream) {
  return loglike_common(data, mu, cov, n_cosmo, n_cls, n_ell, include_logdet, 1, out, status,
                        alpha, ws, ws_bytes, stream);
}

int jcg_sparse_inv(const double* sp, int n, int nd, double* out, cudaStream_t stream) {
  return jcg_sparse_inv_batched(sp, 1, n, nd, out, stream);
}

int jcg_sparse_inv_batched(const double* sp, int n_batch, int n, int nd, double* out, cudaStream_t stream) {
  if (!sp || !out) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n < 1 || nd < 1 || n_batch < 1 || n_batch > 65535) return fail(JCG_ERR_SHAPE, "bad sizes");
  if (n > JCG_SPARSE_MAX_N) return fail(JCG_ERR_SHAPE, "n = %d above the block limit %d", n, JCG_SPARSE_MAX_N);
  if (sp == out) return fail(JCG_ERR_ARG, "sparse inv: input and output must differ");
  launch_sparse_inv(sp, n_batch, n, nd, out, stream);
  return cuda_check("sparse inv");
}

int jcg_sparse_slogdet(const double* sp, int n, int nd, double* sign, double* logdet, double* work,
                       cudaStream_t stream) {
  if (!sp || !sign || !logdet || !work) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n < 1 || nd < 1) return fail(JCG_ERR_SHAPE, "bad sizes");
  if (n > JCG_SPARSE_MAX_N) return fail(JCG_ERR_SHAPE, "n = %d above the block limit %d", n, JCG_SPARSE_MAX_N);
  launch_sparse_slogdet(sp, n, nd, work, work + nd, sign, logdet, stream);
  return cuda_check("sparse slogdet");
}

int jcg_sparse_to_dense(const double* sp, int n, int m, int nd, double* out, cudaStream_t stream) {
  if (!sp || !out) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n < 1 || m < 1 || nd < 1) return fail(JCG_ERR_SHAPE, "bad sizes");
  launch_sparse_to_dense(sp, n, m, nd, out, stream);
  return cuda_check("sparse to_dense");
}

int jcg_sparse_dot_sparse(const double* a, int n, int m, int p, int nd, const double* b, double* out,
                          cudaStream_t stream) {
  if (!a || !b || !out) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n < 1 || m < 1 || p < 1 || nd < 1) return fail(JCG_ERR_SHAPE, "bad sizes");
  launch_sparse_dot_sparse(a, b, n, m, p, nd, out, stream);
  return cuda_check("sparse_dot_sparse");
}

int jcg_sparse_dot_dense(const double* a, int n, int m, int nd, const double* dense, int k, double* out,
                         cudaStream_t stream) {
  if (!a || !dense || !out) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n < 1 || m < 1 || nd < 1 || k < 1) return fail(JCG_ERR_SHAPE, "bad sizes");
  launch_sparse_dot_dense(a, n, m, nd, dense, k, out, stream);
  return cuda_check("sparse_dot_dense");
}

int jcg_dense_dot_sparse(const double* dense, int r, const double* a, int n, int m, int nd, double* out,
                         cudaStream_t stream) {
  if (!a || !dense || !out) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n < 1 || m < 1 || nd < 1 || r < 1) return fail(JCG_ERR_SHAPE, "bad sizes");
  launch_dense_dot_sparse(dense, r, a, n, m, nd, out, stream);
  return cuda_check("dense_dot_sparse");
}

int jcg_dense_dot_sparse_dot_dense(const double* x, int r, const double* y, int n, int m, int nd, const double* z,
                                   int k, double* work, double* out, cudaStream_t stream) {
  if (!x || !y || !z || !work || !out) return fail(JCG_ERR_ARG, "NULL pointer");
  if (r < 1 || n < 1 || m < 1 || nd < 1 || k < 1) return fail(JCG_ERR_SHAPE, "bad sizes");
  if ((long long)n * nd > (1LL << 31) - 1 || (long long)r > 65535LL * 16) return fail(JCG_ERR_SHAPE, "too large");
  launch_sparse_dot_dense(y, n, m, nd, z, k, work, stream);  // T = Y Z, (n nd, k)
  launch_gemm_f64(x, work, r, n * nd, k, out, stream);      // X T
  return cuda_check("dense_dot_sparse_dot_dense");
}

int jcg_sparse_dot_vec(const double* sp, int n, int m, int nd, const double* v, int transpose,
                       double* out, cudaStream_t stream) {
  if (!sp || !v || !out) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n < 1 || m < 1 || nd < 1) return fail(JCG_ERR_SHAPE, "bad sizes");
  launch_sparse_dot_vec(sp, n, m, nd, v, transpose ? 1 : 0, out, stream);
  return cuda_check("sparse dot");
}

}  // extern "C"

// ------------------------------------------------- no-allocation variant -----
// Scratch of jcg_angular_cl_noalloc: one fixed array in static device memory,
// shared by every call on a device (see include/jcg.h for the contract).  It
// holds the same workspace layout as jcg_angular_cl (per-cosmology tables,
// halofit rows, radial kernels); every element a call reads is written earlier
// in the same call, so nothing has to be cleared between calls.
static __device__ __align__(256) unsigned char g_noalloc_scratch[JCG_NOALLOC_SCRATCH_BYTES];
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[64];

// Device address of the scratch array for the current device, looked up once
// per device with that device current.  A host-side reference to the array's
// name is not a device address, so only this pointer is passed to kernels.
static int noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(JCG_ERR_CUDA, "cudaGetDevice failed");
  if (dev < 0 || dev >= 64) return fail(JCG_ERR_CUDA, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(JCG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return JCG_OK;
}

// Constant tables for the no-allocation path: built on the caller's stream
// (no stream of our own is created) and waited for once per device.
static int const_tables_on(cudaStream_t stream, ConstTables** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(JCG_ERR_CUDA, "cudaGetDevice failed");
  if (dev < 0 || dev >= 64) return fail(JCG_ERR_CUDA, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_init_mu);
  if (!g_init_done[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_const);
    if (e != cudaSuccess) return fail(JCG_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    ConstTables* c = static_cast<ConstTables*>(p);
    launch_const_init(c, stream);
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(JCG_ERR_CUDA, "constant tables: %s", cudaGetErrorString(e));
    g_const_ptr[dev] = c;
    g_init_done[dev] = true;
  }
  *out = g_const_ptr[dev];
  return JCG_OK;
}

extern "C" int jcg_angular_cl_noalloc(const jcg_geometry* g, const void* geo, const double* params,
                                      int n_cosmo, int precision, double* cl, cudaStream_t stream) {
  GeoHeader h;
  int rc = make_header(g, &h);
  if (rc) return rc;
  if (!geo || !params || !cl) return fail(JCG_ERR_ARG, "geometry, params or cl is NULL");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  if (precision != JCG_FP64 && precision != JCG_FP32C) return fail(JCG_ERR_ARG, "precision = %d", precision);
  if (h.custom_nodes) return fail(JCG_ERR_ARG, "a geometry with caller redshift nodes has no Limber grid");
  const size_t need = ws_layout(&h, n_cosmo, precision).total;
  if (need > (size_t)JCG_NOALLOC_SCRATCH_BYTES)
    return fail(JCG_ERR_WORKSPACE,
                "jcg_angular_cl_noalloc: %d cosmologies on this geometry need %zu bytes of scratch, "
                "above the fixed limit of %u bytes; split the batch or use jcg_angular_cl with a "
                "workspace",
                n_cosmo, need, (unsigned)JCG_NOALLOC_SCRATCH_BYTES);
  void* scratch = nullptr;
  if ((rc = noalloc_scratch(&scratch))) return rc;
  ConstTables* c = nullptr;
  if ((rc = const_tables_on(stream, &c))) return rc;
  const Batch b = make_batch(&h, geo, params, n_cosmo, precision, scratch, cl);
  launch_cosmo_tables(b, c, stream);
  launch_halofit_rows(b, c, stream);
  launch_tracer_kernels(b, c, stream);
  launch_limber(b, c, limber_tile(h.n_ell), stream);
  return cuda_check("angular_cl_noalloc");
}

// ------------------------------------------------------- host buffers -----
// jcg_angular_cl with the parameters and the C_ell in host memory.  The
// workspace is jcg_angular_cl's followed by device copies of the parameters
// and of the C_ell.  The Limber stage runs as one or two launches over ranges
// of cosmologies; each range's C_ell leave on a copy stream of the calling
// thread as soon as its launch ends, so the first copy runs under the second
// launch; the stream then waits for the last copy.
namespace {
struct HostLayout {
  size_t params, cl, total;
};
struct HostCopy {
  cudaStream_t copy = nullptr;
  cudaEvent_t ev[JCG_HOST_SLICES + 1] = {};
};
}  // namespace

static HostLayout host_layout(const GeoHeader& h, int n_cosmo, int precision) {
  HostLayout L;
  const size_t a = 256;
  size_t o = (ws_layout(&h, n_cosmo, precision).total + a - 1) / a * a;
  L.params = o;
  o += ((size_t)n_cosmo * param_stride(h.physics) * sizeof(double) + a - 1) / a * a;
  L.cl = o;
  o += ((size_t)n_cosmo * h.n_cls * h.n_ell * sizeof(double) + a - 1) / a * a;
  L.total = o;
  return L;
}

// cosmologies [i0, i0 + n) of a uniform batch (the indexing of batch_item)
static Batch batch_slice(const Batch& b, int i0, int n) {
  Batch s = b;
  const size_t na = (size_t)b.max_na;
  s.n_items = n;
  s.params = b.params + (size_t)param_stride(b.physics) * i0;
  s.ctab = b.ctab + i0;
  if (b.rows64) s.rows64 = b.rows64 + (size_t)i0 * na * NROW64;
  if (b.rows32) s.rows32 = b.rows32 + (size_t)i0 * na * NROW32;
  s.kern = b.kern + (size_t)i0 * b.max_tr * na;
  if (b.u32) s.u32 = b.u32 + (size_t)i0 * na;
  if (b.kern32) s.kern32 = b.kern32 + (size_t)i0 * b.max_tr * na;
  s.cl = b.cl + (size_t)i0 * b.max_cls * b.max_ell;
  return s;
}

// the copy stream and events of the calling host thread on device dev
static int host_copy(int dev, HostCopy** out) {
  static thread_local HostCopy hc[64];
  HostCopy& r = hc[dev];
  if (!r.copy) {
    if (cudaStreamCreateWithFlags(&r.copy, cudaStreamNonBlocking) != cudaSuccess) {
      r.copy = nullptr;
      return cuda_check("copy stream");
    }
    for (int i = 0; i <= JCG_HOST_SLICES; ++i)
      if (cudaEventCreateWithFlags(&r.ev[i], cudaEventDisableTiming) != cudaSuccess) return cuda_check("copy events");
  }
  *out = &r;
  return JCG_OK;
}

// The Limber launches' ranges [b[k], b[k + 1]): one below 2048 cosmologies,
// else the first three quarters and the last quarter.  Only the last range's
// copy is not under a Limber launch, so it is the short one; the first
// range's copy (three times longer) runs under the last launch, and each
// extra launch costs a partly idle last wave of CTAs.
static int host_ranges(int n_cosmo, int* b) {
  b[0] = 0;
  if (n_cosmo < 2048) {
    b[1] = n_cosmo;
    return 1;
  }
  b[1] = n_cosmo - n_cosmo / 4;
  b[2] = n_cosmo;
  return 2;
}

extern "C" int jcg_host_workspace_size(const jcg_geometry* g, int n_cosmo, int precision, size_t* bytes) {
  if (!bytes) return fail(JCG_ERR_ARG, "bytes is NULL");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  if (precision != JCG_FP64 && precision != JCG_FP32C) return fail(JCG_ERR_ARG, "precision = %d", precision);
  GeoHeader h;
  const int rc = make_header(g, &h);
  if (rc) return rc;
  *bytes = host_layout(h, n_cosmo, precision).total;
  return JCG_OK;
}

extern "C" int jcg_angular_cl_host(const jcg_geometry* g, const void* geo, const double* params_host,
                                   int n_cosmo, int precision, double* cl_host, void* ws, size_t ws_bytes,
                                   cudaStream_t stream) {
  GeoHeader h;
  int rc = make_header(g, &h);
  if (rc) return rc;
  if (!geo || !cl_host) return fail(JCG_ERR_ARG, "geometry or cl is NULL");
  if (h.custom_nodes) return fail(JCG_ERR_ARG, "a geometry with caller redshift nodes has no Limber grid");
  if ((rc = check_common(params_host, n_cosmo, precision, ws, ws_bytes, 0))) return rc;
  const HostLayout HL = host_layout(h, n_cosmo, precision);
  if (ws_bytes < HL.total) return fail(JCG_ERR_WORKSPACE, "workspace %zu bytes, need %zu", ws_bytes, HL.total);
  ConstTables* c = nullptr;
  if ((rc = const_tables(&c))) return rc;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(JCG_ERR_CUDA, "cudaGetDevice failed");
  HostCopy* hc = nullptr;
  if ((rc = host_copy(dev, &hc))) return rc;
  char* base = static_cast<char*>(ws);
  double* dparams = reinterpret_cast<double*>(base + HL.params);
  double* dcl = reinterpret_cast<double*>(base + HL.cl);
  const size_t pbytes = (size_t)n_cosmo * param_stride(h.physics) * sizeof(double);
  if (cudaMemcpyAsync(dparams, params_host, pbytes, cudaMemcpyHostToDevice, stream) != cudaSuccess)
    return cuda_check("angular_cl_host parameters");
  const Batch b = make_batch(&h, geo, dparams, n_cosmo, precision, ws, dcl);
  launch_cosmo_tables(b, c, stream);
  launch_halofit_rows(b, c, stream);
  launch_tracer_kernels(b, c, stream);
  int rb[JCG_HOST_SLICES + 1];
  const int ns = host_ranges(n_cosmo, rb), lt = limber_tile(h.n_ell);
  const size_t per = (size_t)h.n_cls * h.n_ell;
  for (int k = 0; k < ns; ++k) {
    const int i0 = rb[k], i1 = rb[k + 1];
    launch_limber(batch_slice(b, i0, i1 - i0), c, lt, stream);
    if (cudaEventRecord(hc->ev[k], stream) != cudaSuccess || cudaStreamWaitEvent(hc->copy, hc->ev[k], 0) != cudaSuccess ||
        cudaMemcpyAsync(cl_host + (size_t)i0 * per, dcl + (size_t)i0 * per, (size_t)(i1 - i0) * per * sizeof(double),
                        cudaMemcpyDeviceToHost, hc->copy) != cudaSuccess)
      return cuda_check("angular_cl_host copies");
  }
  if (cudaEventRecord(hc->ev[ns], hc->copy) != cudaSuccess || cudaStreamWaitEvent(stream, hc->ev[ns], 0) != cudaSuccess)
    return cuda_check("angular_cl_host join");
  return cuda_check("angular_cl_host");
}

// --------------------------------------------------------- derivatives -----
extern "C" int jcg_jacobian_workspace_size(const jcg_geometry* g, int n_cosmo, int precision, size_t* bytes) {
  if (!bytes) return fail(JCG_ERR_ARG, "bytes is NULL");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  if (precision != JCG_FP64 && precision != JCG_FP32C) return fail(JCG_ERR_ARG, "precision = %d", precision);
  GeoHeader h;
  const int rc = make_header(g, &h);
  if (rc) return rc;
  *bytes = grad_workspace_bytes(h, n_cosmo, precision);
  return JCG_OK;
}

extern "C" int jcg_angular_cl_jacobian(const jcg_geometry* g, const void* geo, const double* params,
                                       int n_cosmo, int precision, double* cl, double* jac, void* ws,
                                       size_t ws_bytes, cudaStream_t stream) {
  return jcg_angular_cl_jacobian_dir(g, geo, params, n_cosmo, precision, -1, cl, jac, ws, ws_bytes, stream);
}

extern "C" int jcg_angular_cl_jacobian_dir(const jcg_geometry* g, const void* geo, const double* params,
                                           int n_cosmo, int precision, int gamma_dir, double* cl, double* jac,
                                           void* ws, size_t ws_bytes, cudaStream_t stream) {
  GeoHeader h;
  int rc = make_header(g, &h);
  if (rc) return rc;
  if (gamma_dir < -1 || gamma_dir >= 8) return fail(JCG_ERR_ARG, "gamma_dir = %d", gamma_dir);
  if (gamma_dir >= 0 && !growth_gamma(h.physics))
    return fail(JCG_ERR_ARG, "gamma_dir = %d without JCG_GROWTH_GAMMA", gamma_dir);
  if (!geo || !params || !jac || !ws) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  if (precision != JCG_FP64 && precision != JCG_FP32C) return fail(JCG_ERR_ARG, "precision = %d", precision);
  if (h.custom_nodes) return fail(JCG_ERR_ARG, "a geometry with caller redshift nodes has no Limber grid");
  const size_t need = grad_workspace_bytes(h, n_cosmo, precision);
  if (ws_bytes < need) return fail(JCG_ERR_WORKSPACE, "workspace %zu bytes, need %zu", ws_bytes, need);
  if (((uintptr_t)ws) % 256 != 0) return fail(JCG_ERR_ARG, "workspace must be 256-byte aligned");
  ConstTables* c = nullptr;
  if ((rc = const_tables(&c))) return rc;
  grad_run(static_cast<const GeoHeader*>(geo), h, params, n_cosmo, precision, cl, jac, ws, c, stream, gamma_dir);
  return cuda_check("angular_cl_jacobian");
}

extern "C" int jcg_angular_cl_jacobian_branch(const jcg_geometry* g, const void* geo, const double* params,
                                              int n_cosmo, const int* seg_in, int* seg_out, double* cl,
                                              double* jac, void* ws, size_t ws_bytes, cudaStream_t stream) {
  GeoHeader h;
  int rc = make_header(g, &h);
  if (rc) return rc;
  if (growth_gamma(h.physics))
    return fail(JCG_ERR_UNSUPPORTED, "jcg_angular_cl_jacobian_branch: JCG_GROWTH_GAMMA is not supported");
  if (!geo || !params || !jac || !ws) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  if (h.custom_nodes) return fail(JCG_ERR_ARG, "a geometry with caller redshift nodes has no Limber grid");
  if (seg_in && seg_in == seg_out) return fail(JCG_ERR_ARG, "seg_in and seg_out must differ");
  const size_t need = grad_workspace_bytes(h, n_cosmo, JCG_FP64);
  if (ws_bytes < need) return fail(JCG_ERR_WORKSPACE, "workspace %zu bytes, need %zu", ws_bytes, need);
  if (((uintptr_t)ws) % 256 != 0) return fail(JCG_ERR_ARG, "workspace must be 256-byte aligned");
  ConstTables* c = nullptr;
  if ((rc = const_tables(&c))) return rc;
  grad_run(static_cast<const GeoHeader*>(geo), h, params, n_cosmo, JCG_FP64, cl, jac, ws, c, stream, -1, seg_in,
           seg_out);
  return cuda_check("angular_cl_jacobian_branch");
}

extern "C" int jcg_vjp_workspace_size(const jcg_geometry* g, int n_cosmo, int precision, size_t* bytes) {
  if (!bytes) return fail(JCG_ERR_ARG, "bytes is NULL");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  if (precision != JCG_FP64 && precision != JCG_FP32C) return fail(JCG_ERR_ARG, "precision = %d", precision);
  GeoHeader h;
  const int rc = make_header(g, &h);
  if (rc) return rc;
  *bytes = vjp_workspace_bytes(h, n_cosmo, precision);
  return JCG_OK;
}

static int vjp_checked(const jcg_geometry* g, const void* geo, const double* params, int n_cosmo, int precision,
                       int gamma_dir, const double* cl_bar, double* cl, double* grad, void* ws, size_t ws_bytes,
                       cudaStream_t stream, unsigned stages);

extern "C" int jcg_angular_cl_vjp(const jcg_geometry* g, const void* geo, const double* params, int n_cosmo,
                                  int precision, int gamma_dir, const double* cl_bar, double* cl, double* grad,
                                  void* ws, size_t ws_bytes, cudaStream_t stream) {
  return vjp_checked(g, geo, params, n_cosmo, precision, gamma_dir, cl_bar, cl, grad, ws, ws_bytes, stream, GS_ALL);
}

// measurement tooling (jcg_calib.h): the fp32c pipeline's stages selected by
// a mask, on a workspace that a full call filled
extern "C" int jcg_calib_vjp_stages(const jcg_geometry* g, const void* geo, const double* params, int n_cosmo,
                                    const double* cl_bar, double* cl, double* grad, void* ws, size_t ws_bytes,
                                    unsigned stage_mask, cudaStream_t stream) {
  if ((stage_mask & ~(unsigned)GS_ALL) != 0 || stage_mask == 0) return fail(JCG_ERR_ARG, "stage_mask = 0x%x", stage_mask);
  return vjp_checked(g, geo, params, n_cosmo, JCG_FP32C, -1, cl_bar, cl, grad, ws, ws_bytes, stream, stage_mask);
}

static int vjp_checked(const jcg_geometry* g, const void* geo, const double* params, int n_cosmo, int precision,
                       int gamma_dir, const double* cl_bar, double* cl, double* grad, void* ws, size_t ws_bytes,
                       cudaStream_t stream, unsigned stages) {
  GeoHeader h;
  int rc = make_header(g, &h);
  if (rc) return rc;
  if (gamma_dir < -1 || gamma_dir >= 8) return fail(JCG_ERR_ARG, "gamma_dir = %d", gamma_dir);
  if (gamma_dir >= 0 && !growth_gamma(h.physics))
    return fail(JCG_ERR_ARG, "gamma_dir = %d without JCG_GROWTH_GAMMA", gamma_dir);
  if (!geo || !params || !cl_bar || !grad || !ws) return fail(JCG_ERR_ARG, "NULL pointer");
  if (n_cosmo < 1) return fail(JCG_ERR_SHAPE, "n_cosmo = %d", n_cosmo);
  if (precision != JCG_FP64 && precision != JCG_FP32C) return fail(JCG_ERR_ARG, "precision = %d", precision);
  if (h.custom_nodes) return fail(JCG_ERR_ARG, "a geometry with caller redshift nodes has no Limber grid");
  const size_t need = vjp_workspace_bytes(h, n_cosmo, precision);
  if (ws_bytes < need) return fail(JCG_ERR_WORKSPACE, "workspace %zu bytes, need %zu", ws_bytes, need);
  if (((uintptr_t)ws) % 256 != 0) return fail(JCG_ERR_ARG, "workspace must be 256-byte aligned");
  ConstTables* c = nullptr;
  if ((rc = const_tables(&c))) return rc;
  vjp_run(static_cast<const GeoHeader*>(geo), h, params, n_cosmo, precision, cl_bar, cl, grad, ws, c, stream,
          gamma_dir, stages);
  return cuda_check("angular_cl_vjp");
}

// ------------------------------------------------------ ragged requests -----
namespace {

struct ReqPlan {
  std::vector<GeoHeader> hdr;
  std::vector<GradReq> greq;
};

size_t cl_item_bytes(const GeoHeader& h, int precision) {
  size_t o = align256(sizeof(CosmoTab));
  o += align256(sizeof(double) * NROW64 * (size_t)h.na);
  if (precision == JCG_FP32C) o += align256(sizeof(float) * NROW32 * (size_t)h.na);
  o += align256(sizeof(double) * (size_t)h.n_tr * h.na);
  return o;
}

// host validation of every request; headers into plan
int plan_requests(const jcg_request* reqs, int n, int mode, int precision, ReqPlan* plan) {
  if (!reqs) return fail(JCG_ERR_ARG, "requests is NULL");
  if (n < 1 || n > JCG_MAX_REQUESTS) return fail(JCG_ERR_SHAPE, "n = %d (1..%d)", n, JCG_MAX_REQUESTS);
  if (mode < JCG_REQ_CL || mode > JCG_REQ_LOGLIKE_GRAD) return fail(JCG_ERR_ARG, "mode = %d", mode);
  if (precision != JCG_FP64 && precision != JCG_FP32C) return fail(JCG_ERR_ARG, "precision = %d", precision);
  plan->hdr.resize(n);
  plan->greq.resize(n);
  for (int i = 0; i < n; ++i) {
    const jcg_request& r = reqs[i];
    int rc = make_header(r.g, &plan->hdr[i]);
    if (rc) {
      char why[sizeof(g_err)];
      memcpy(why, g_err, sizeof(why));
      return fail(rc, "request %d: %s", i, why);
    }
    if (plan->hdr[i].custom_nodes) return fail(JCG_ERR_ARG, "request %d: geometry without a Limber grid", i);
    // a request carries 8 parameters and its outputs 8 derivative columns:
    // the gamma growth (a 9th parameter) is served by jcg_angular_cl(_jacobian_dir)
    if (growth_gamma(plan->hdr[i].physics))
      return fail(JCG_ERR_UNSUPPORTED, "request %d: JCG_GROWTH_GAMMA is not supported by ragged requests "
                  "(8 parameters per request)", i);
    if (!r.geo_dev || !r.params_dev) return fail(JCG_ERR_ARG, "request %d: NULL geometry or params", i);
    if (mode == JCG_REQ_CL && !r.cl_dev) return fail(JCG_ERR_ARG, "request %d: cl is NULL", i);
    if (mode == JCG_REQ_JACOBIAN && !r.jac_dev) return fail(JCG_ERR_ARG, "request %d: jac is NULL", i);
    if (mode == JCG_REQ_LOGLIKE_GRAD && (!r.data_dev || !r.prec_dev || !r.out_dev))
      return fail(JCG_ERR_ARG, "request %d: data, prec or out is NULL", i);
    GradReq& q = plan->greq[i];
    q.h = &plan->hdr[i];
    q.geo = static_cast<const GeoHeader*>(r.geo_dev);
    q.params = r.params_dev;
    q.cl = r.cl_dev;
    q.jac = mode == JCG_REQ_LOGLIKE_GRAD && precision == JCG_FP32C ? nullptr : r.jac_dev;
    q.out = r.out_dev;
    q.vbar = nullptr;
  }
  return JCG_OK;
}

// fp32c log-likelihood requests take the vector-Jacobian form
bool vjp_mode(int mode, int precision) { return mode == JCG_REQ_LOGLIKE_GRAD && precision == JCG_FP32C; }

size_t cl_listed_bytes(const ReqPlan& p, int precision) {
  size_t o = align256(sizeof(Item) * p.hdr.size());
  for (const GeoHeader& h : p.hdr) o += cl_item_bytes(h, precision);
  return o;
}

// the request table and the ell-tile partials of the request log-likelihood
size_t ll_extra_bytes(const ReqPlan& p, int n) {
  size_t tiles = 0;
  for (int i = 0; i < n; ++i) tiles += rl_tiles(p.hdr[i].n_ell);
  return align256(sizeof(ReqLL) * (size_t)n) + align256(sizeof(double) * 9 * tiles);
}

}  // namespace

extern "C" int jcg_requests_workspace_size(const jcg_request* reqs, int n, int mode, int precision,
                                           size_t* bytes_min, size_t* bytes_full) {
  if (!bytes_min || !bytes_full) return fail(JCG_ERR_ARG, "bytes is NULL");
  static thread_local ReqPlan plan;
  int rc = plan_requests(reqs, n, mode, precision, &plan);
  if (rc) return rc;
  if (mode == JCG_REQ_CL) {
    *bytes_min = *bytes_full = cl_listed_bytes(plan, precision);
    return JCG_OK;
  }
  const size_t extra = mode == JCG_REQ_LOGLIKE_GRAD ? ll_extra_bytes(plan, n) : 0;
  if (vjp_mode(mode, precision)) {
    *bytes_min = *bytes_full = extra + grad_listed_bytes(plan.greq.data(), n, 1, precision, true);
    return JCG_OK;
  }
  const int ns = grad_listed_auto_split(plan.greq.data(), n, precision);
  *bytes_min = extra + grad_listed_bytes(plan.greq.data(), n, 1, precision);
  *bytes_full = extra + grad_listed_bytes(plan.greq.data(), n, ns, precision);
  return JCG_OK;
}

extern "C" int jcg_requests_run(const jcg_request* reqs, int n, int mode, int precision, void* ws,
                                size_t ws_bytes, cudaStream_t stream) {
  static thread_local ReqPlan plan;
  int rc = plan_requests(reqs, n, mode, precision, &plan);
  if (rc) return rc;
  if (!ws) return fail(JCG_ERR_ARG, "workspace is NULL");
  if (((uintptr_t)ws) % 256 != 0) return fail(JCG_ERR_ARG, "workspace must be 256-byte aligned");
  ConstTables* c = nullptr;
  if ((rc = const_tables(&c))) return rc;
  char* base = static_cast<char*>(ws);
  if (mode == JCG_REQ_CL) {
    const size_t need = cl_listed_bytes(plan, precision);
    if (ws_bytes < need) return fail(JCG_ERR_WORKSPACE, "workspace %zu bytes, need %zu", ws_bytes, need);
    static thread_local std::vector<Item> items;
    items.resize(n);
    Item* dev_items = reinterpret_cast<Item*>(base);
    size_t o = align256(sizeof(Item) * (size_t)n);
    Batch b;
    memset(&b, 0, sizeof(b));
    for (int i = 0; i < n; ++i) {
      const GeoHeader& h = plan.hdr[i];
      Item& it = items[i];
      it.params = reqs[i].params_dev;
      it.geo = static_cast<const GeoHeader*>(reqs[i].geo_dev);
      it.ctab = reinterpret_cast<CosmoTab*>(base + o);
      o += align256(sizeof(CosmoTab));
      it.rows64 = reinterpret_cast<double*>(base + o);
      o += align256(sizeof(double) * NROW64 * (size_t)h.na);
      it.rows32 = nullptr;
      if (precision == JCG_FP32C) {
        it.rows32 = reinterpret_cast<float*>(base + o);
        o += align256(sizeof(float) * NROW32 * (size_t)h.na);
      }
      it.kern = reinterpret_cast<double*>(base + o);
      o += align256(sizeof(double) * (size_t)h.n_tr * h.na);
      it.u32 = nullptr;  // ragged requests: the Limber kernel converts the FP64 columns
      it.kern32 = nullptr;
      it.cl = reqs[i].cl_dev;
      it.precision = precision;
      it.physics = h.physics;
      b.physics_or |= h.physics;
      b.max_na = max(b.max_na, h.na);
      b.max_ell = max(b.max_ell, h.n_ell);
      b.max_cls = max(b.max_cls, h.n_cls);
      b.max_tr = max(b.max_tr, h.n_tr);
    }
    if (cudaError_t e = stage_h2d(dev_items, items.data(), sizeof(Item) * (size_t)n, stream))
      return fail(JCG_ERR_CUDA, "request table copy: %s", cudaGetErrorString(e));
    b.n_items = n;
    b.listed = 1;
    b.items = dev_items;
    b.precision = precision;
    launch_cosmo_tables(b, c, stream);
    launch_halofit_rows(b, c, stream);
    launch_tracer_kernels(b, c, stream);
    launch_limber(b, c, limber_tile(b.max_ell), stream);
    return cuda_check("requests angular_cl");
  }
  const size_t extra = mode == JCG_REQ_LOGLIKE_GRAD ? ll_extra_bytes(plan, n) : 0;
  const bool vjp = vjp_mode(mode, precision);
  const size_t need1 = extra + grad_listed_bytes(plan.greq.data(), n, 1, precision, vjp);
  if (ws_bytes < need1) return fail(JCG_ERR_WORKSPACE, "workspace %zu bytes, need %zu", ws_bytes, need1);
  int ns = vjp ? 1 : grad_listed_auto_split(plan.greq.data(), n, precision);
  while (ns > 1 && extra + grad_listed_bytes(plan.greq.data(), n, ns, precision) > ws_bytes) --ns;
  static thread_local GradBatch vgb;
  if (cudaError_t e = grad_run_listed(plan.greq.data(), n, ns, precision, base + extra, c, stream, vjp, &vgb))
    return fail(JCG_ERR_CUDA, "requests jacobian: %s", cudaGetErrorString(e));
  if (mode == JCG_REQ_LOGLIKE_GRAD) {
    static thread_local std::vector<ReqLL> ll;
    ll.resize(n);
    double* part = reinterpret_cast<double*>(base + align256(sizeof(ReqLL) * (size_t)n));
    int max_tiles = 1, max_cls = 1;
    for (int i = 0; i < n; ++i) {
      ll[i].cl = plan.greq[i].cl;
      ll[i].jac = plan.greq[i].jac;
      ll[i].vbar = plan.greq[i].vbar;
      ll[i].data = reqs[i].data_dev;
      ll[i].prec = reqs[i].prec_dev;
      ll[i].out = reqs[i].out_dev;
      ll[i].part = part;
      ll[i].n_cls = plan.hdr[i].n_cls;
      ll[i].n_ell = plan.hdr[i].n_ell;
      part += 9 * (size_t)rl_tiles(ll[i].n_ell);
      max_tiles = max(max_tiles, rl_tiles(ll[i].n_ell));
      max_cls = max(max_cls, ll[i].n_cls);
    }
    ReqLL* dev_ll = reinterpret_cast<ReqLL*>(base);
    if (cudaError_t e = stage_h2d(dev_ll, ll.data(), sizeof(ReqLL) * (size_t)n, stream))
      return fail(JCG_ERR_CUDA, "request loglike table copy: %s", cudaGetErrorString(e));
    launch_request_loglike(dev_ll, n, max_tiles, max_cls, stream);
    // fp32c: the gradient as the product of the cotangents -P r with dC/dtheta
    if (vjp) launch_vjp32_grad(vgb, stream);
  }
  return cuda_check("requests jacobian");
}
