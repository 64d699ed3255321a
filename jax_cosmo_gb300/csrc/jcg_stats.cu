// Gaussian covariance, log-likelihood and the block-diagonal ("sparse") matrix
// algebra, FP64.
//
// The covariance of angular_cl.py:120-163 is, after permuting (cls, ell) to
// (ell, cls), block diagonal with one n_cls x n_cls block per ell.  The
// log-likelihood of likelihood.py:9-61 therefore factors into per-ell Cholesky
// solves: r^T C^-1 r = sum_l r_l^T A_l^-1 r_l and logdet C = sum_l logdet A_l,
// which is what the reference's sparse path (sparse.py:295-366) computes by
// inverse and Schur complements, and its dense path by a full inverse.
#include "jcg_internal.cuh"

namespace jcg {

// index of pair (min(a,b), max(a,b)) in the ordering of angular_cl.py:15-25
__device__ __forceinline__ int pair_index(int a, int b, int n) {
  const int i = a < b ? a : b, j = a < b ? b : a;
  return i * n - (i * (i - 1)) / 2 + (j - i);
}

// np.gradient(ell) with unit spacing and first-order edges.
__device__ __forceinline__ double ell_gradient(const double* ell, int n, int l) {
  if (l == 0) return (ell[1] - ell[0]) / 1.0;
  if (l == n - 1) return (ell[n - 1] - ell[n - 2]) / 1.0;
  return (ell[l + 1] - ell[l - 1]) / 2.0;
}

// pair p -> (i, j) of the ordering of angular_cl.py:15-25
__device__ __forceinline__ int2 pair_of(int p, int n) {
  int i = 0;
  while (i < n - 1 && p >= (i + 1) * n - ((i + 1) * i) / 2) ++i;
  const int j = p - (i * n - (i * (i - 1)) / 2) + i;
  return make_int2(i, j);
}

// cl_obs = cl_signal + cl_noise (angular_cl.py:135); the noise of noise_cl
// (angular_cl.py:101-117) is noise[i] * delta_ij on auto-spectra.
__device__ __forceinline__ double cl_obs(const double* sig, const double* cl_noise,
                                         const double* tr_noise, int x, int l, int n_ell,
                                         int n_tr) {
  double nz = 0.0;
  if (cl_noise) {
    nz = cl_noise[(size_t)x * n_ell + l];
  } else if (tr_noise) {
    const int2 ij = pair_of(x, n_tr);
    const double delta = 1.0 - fmin(fmax(fabs((double)(ij.x - ij.y)), 0.0), 1.0);
    nz = __dmul_rn(__dmul_rn(tr_noise[ij.x], delta), 1.0);
  }
  return __dadd_rn(sig[(size_t)x * n_ell + l], nz);
}

// One thread per sparse element (p, q, l) of one cosmology, or per dense
// element.  angular_cl.py:138-162.
__global__ void covariance_kernel(const double* __restrict__ ell, int n_ell, int n_tr,
                                  const double* __restrict__ cl, const double* __restrict__ cl_noise,
                                  const double* __restrict__ tr_noise, int n_cosmo, double f_sky,
                                  int sparse, double* __restrict__ out) {
  const int n_cls = n_tr * (n_tr + 1) / 2;
  const size_t N = (size_t)n_cls * n_ell;
  const size_t per = sparse ? (size_t)n_cls * n_cls * n_ell : N * N;
  const size_t total = per * n_cosmo;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const size_t ci = idx / per, e = idx % per;
    int p, q, l;
    if (sparse) {
      l = (int)(e % n_ell);
      q = (int)((e / n_ell) % n_cls);
      p = (int)(e / ((size_t)n_ell * n_cls));
    } else {
      const size_t row = e / N, col = e % N;
      p = (int)(row / n_ell);
      l = (int)(row % n_ell);
      q = (int)(col / n_ell);
      const int l2 = (int)(col % n_ell);
      if (l2 != l) {
        out[idx] = 0.0;
        continue;
      }
    }
    const double* sig = cl + ci * (size_t)n_cls * n_ell;
    const int2 ij = pair_of(p, n_tr), mn = pair_of(q, n_tr);
    const int i = ij.x, j = ij.y, m = mn.x, n = mn.y;
    // (find(i,m), find(j,n), find(i,n), find(j,m))  angular_cl.py:41-45
    const int a = pair_index(i, m, n_tr), b = pair_index(j, n, n_tr);
    const int c = pair_index(i, n, n_tr), d = pair_index(j, m, n_tr);
    // unfused multiply / add: the same roundings as the reference's NumPy ops
    const double norm =
        __dmul_rn(__dmul_rn(__dadd_rn(__dmul_rn(2.0, ell[l]), 1.0), ell_gradient(ell, n_ell, l)), f_sky);
    const double oa = cl_obs(sig, cl_noise, tr_noise, a, l, n_ell, n_tr);
    const double ob = cl_obs(sig, cl_noise, tr_noise, b, l, n_ell, n_tr);
    const double oc = cl_obs(sig, cl_noise, tr_noise, c, l, n_ell, n_tr);
    const double od = cl_obs(sig, cl_noise, tr_noise, d, l, n_ell, n_tr);
    out[idx] = __ddiv_rn(__dadd_rn(__dmul_rn(oa, ob), __dmul_rn(oc, od)), norm);
  }
}

void launch_covariance(const double* ell, int n_ell, int n_tr, const double* cl,
                       const double* cl_noise, const double* tr_noise, int n_cosmo, double f_sky,
                       int sparse, double* out, cudaStream_t st) {
  const int n_cls = n_tr * (n_tr + 1) / 2;
  const size_t N = (size_t)n_cls * n_ell;
  const size_t total = (sparse ? (size_t)n_cls * n_cls * n_ell : N * N) * n_cosmo;
  const size_t blocks = (total + 255) / 256;
  const unsigned nb = (unsigned)(blocks < 152 * 64 ? (blocks ? blocks : 1) : 152 * 64);
  covariance_kernel<<<nb, 256, 0, st>>>(ell, n_ell, n_tr, cl, cl_noise, tr_noise, n_cosmo, f_sky,
                                        sparse, out);
}

// ------------------------------------------------------ block Cholesky -----
// In-place lower Cholesky of the n x n matrix A (shared memory, row-major).
// Returns false if a pivot is not positive.
__device__ bool block_cholesky(double* A, int n, volatile int* flag) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {
      const double d = A[k * n + k];
      if (!(d > 0.0)) *flag = 1;
      A[k * n + k] = sqrt(d);
    }
    __syncthreads();
    const double dk = A[k * n + k];
    for (int i = k + 1 + tid; i < n; i += nt) A[i * n + k] /= dk;
    __syncthreads();
    const int m = n - k - 1;
    for (int e = tid; e < m * m; e += nt) {
      const int i = k + 1 + e / m, j = k + 1 + e % m;
      if (j <= i) A[i * n + j] -= A[i * n + k] * A[j * n + k];
    }
    __syncthreads();
  }
  return *flag == 0;
}

// r^T A^-1 r and logdet A from the Cholesky factor (single thread: n is small).
__device__ void chol_quad_logdet(const double* L, const double* r, double* z, int n, double* quad,
                                 double* logdet) {
  double q = 0.0, ld = 0.0;
  for (int i = 0; i < n; ++i) {
    double v = r[i];
    for (int j = 0; j < i; ++j) v -= L[i * n + j] * z[j];
    z[i] = v / L[i * n + i];
    q += z[i] * z[i];
    ld += log(L[i * n + i]);
  }
  *quad = q;
  *logdet = 2.0 * ld;
}

// One CTA per (ell, cosmology): block A_l[p][q] from the sparse or dense input,
// Cholesky, then r_l^T A_l^-1 r_l and logdet A_l into the partials.
__global__ void loglike_blocks_kernel(const double* __restrict__ data, const double* __restrict__ mu,
                                      const double* __restrict__ cov, int n_cls, int n_ell,
                                      int dense, const int* __restrict__ structure,
                                      double* __restrict__ partial, int* __restrict__ status,
                                      double* __restrict__ alpha) {
  const int l = blockIdx.x, ci = blockIdx.y;
  extern __shared__ double sm[];
  double* A = sm;
  double* r = A + n_cls * n_cls;
  double* z = r + n_cls;
  __shared__ int flag;
  const size_t N = (size_t)n_cls * n_ell;
  if (threadIdx.x == 0) flag = 0;
  if (dense && structure && structure[ci] != 0) {
    if (threadIdx.x == 0) {
      partial[((size_t)ci * n_ell + l) * 2 + 0] = NAN;
      partial[((size_t)ci * n_ell + l) * 2 + 1] = NAN;
    }
    return;
  }
  for (int e = threadIdx.x; e < n_cls * n_cls; e += blockDim.x) {
    const int p = e / n_cls, q = e % n_cls;
    double v;
    if (dense) {
      v = cov[(size_t)ci * N * N + ((size_t)p * n_ell + l) * N + (size_t)q * n_ell + l];
    } else {
      v = cov[(((size_t)ci * n_cls + p) * n_cls + q) * n_ell + l];
    }
    A[e] = v;
  }
  for (int p = threadIdx.x; p < n_cls; p += blockDim.x) {
    const size_t o = (size_t)ci * N + (size_t)p * n_ell + l;
    r[p] = mu[o] - data[o];  // likelihood.py:38
  }
  __syncthreads();
  const bool ok = block_cholesky(A, n_cls, &flag);
  if (threadIdx.x == 0) {
    double q = NAN, ld = NAN;
    if (ok) chol_quad_logdet(A, r, z, n_cls, &q, &ld);
    else atomicMax(status + ci, 2);
    partial[((size_t)ci * n_ell + l) * 2 + 0] = q;
    partial[((size_t)ci * n_ell + l) * 2 + 1] = ld;
    if (alpha) {
      // C^-1 r = L^-T z (back substitution), the gradient of r^T C^-1 r / 2
      for (int i = n_cls - 1; i >= 0; --i) {
        double v = ok ? z[i] : NAN;
        for (int j = i + 1; j < n_cls; ++j) v -= A[j * n_cls + i] * z[j];
        z[i] = ok ? v / A[i * n_cls + i] : NAN;
        alpha[(size_t)ci * N + (size_t)i * n_ell + l] = z[i];
      }
    }
  }
}

// Fixed-order sum over ell of the partials: -0.5 * (quad - logdet) (likelihood.py:61).
__global__ void loglike_reduce_kernel(const double* __restrict__ partial, int n_cosmo, int n_ell,
                                      int include_logdet, double* __restrict__ out) {
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  if (ci >= n_cosmo) return;
  double q = 0.0, ld = 0.0;
  for (int l = 0; l < n_ell; ++l) {
    q += partial[((size_t)ci * n_ell + l) * 2 + 0];
    ld += partial[((size_t)ci * n_ell + l) * 2 + 1];
  }
  out[ci] = include_logdet ? -0.5 * (q - ld) : -0.5 * q;
}

// Dense input: flag cosmologies whose matrix has a non-zero outside the
// per-ell diagonals of its n_ell x n_ell blocks.
__global__ void dense_structure_kernel(const double* __restrict__ cov, int n_cosmo, int n_cls,
                                       int n_ell, int* __restrict__ structure) {
  const size_t N = (size_t)n_cls * n_ell;
  const size_t total = N * N * n_cosmo;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const size_t e = idx % (N * N);
    const size_t row = e / N, col = e % N;
    if ((row % n_ell) != (col % n_ell) && cov[idx] != 0.0) {
      structure[idx / (N * N)] = 1;
    }
  }
}

__global__ void merge_structure_kernel(const int* structure, int* status, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && structure[i]) status[i] = 1;
}

__global__ void zero_int_kernel(int* p, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0;
}

// Log-likelihood with a fixed inverse covariance P (the covariance held
// constant, as in the reference's intro notebook) and its gradient:
//   r = C_ell - data, logL = -r^T P r / 2, dlogL/dtheta = -(dC_ell/dtheta)^T P r.
// One CTA per (tile of RL_ELL ell, request): r of the tile staged in shared
// memory, per (ell, spectrum) alpha = (P r) and its 9 contributions, the
// CTA's sums to the tile's partial; a second kernel adds the tiles in order.
// Fixed-order reductions: the same result alone or in a batch.
__global__ void __launch_bounds__(128) request_loglike_part_kernel(const ReqLL* __restrict__ items, int n) {
  const int item = blockIdx.y, tile = blockIdx.x;
  if (item >= n) return;
  const ReqLL q = items[item];
  const int n_cls = q.n_cls, n_ell = q.n_ell;
  const int l0 = tile * RL_ELL;
  if (l0 >= n_ell) return;
  const int lt = min(RL_ELL, n_ell - l0);
  extern __shared__ double rs[];  // [n_cls][RL_ELL]
  for (int e = threadIdx.x; e < n_cls * lt; e += blockDim.x) {
    const int k = e / lt, j = e - k * lt;
    const size_t o = (size_t)k * n_ell + l0 + j;
    rs[k * RL_ELL + j] = q.cl[o] - q.data[o];
  }
  __syncthreads();
  double acc[9];
  for (int s = 0; s < 9; ++s) acc[s] = 0.0;
  for (int idx = threadIdx.x; idx < lt * n_cls; idx += blockDim.x) {
    const int j = idx / n_cls, p = idx - j * n_cls;
    const int l = l0 + j;
    const double* Pl = q.prec + ((size_t)l * n_cls + p) * n_cls;
    double alpha = 0.0;
    for (int k = 0; k < n_cls; ++k) alpha += Pl[k] * rs[k * RL_ELL + j];
    acc[0] += rs[p * RL_ELL + j] * alpha;
    if (q.jac) {
      const double* J = q.jac + ((size_t)p * n_ell + l) * 8;
      for (int d = 0; d < 8; ++d) acc[1 + d] += alpha * J[d];
    } else {
      q.vbar[(size_t)p * n_ell + l] = -alpha;
    }
  }
  __shared__ double red[4][9];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int s = 0; s < 9; ++s) {
    double v = acc[s];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) red[warp][s] = v;
  }
  __syncthreads();
  if (threadIdx.x < 9) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
    q.part[(size_t)tile * 9 + threadIdx.x] = v;
  }
}

__global__ void request_loglike_sum_kernel(const ReqLL* __restrict__ items, int n) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int item = idx / 9, s = idx % 9;
  if (item >= n) return;
  const ReqLL q = items[item];
  if (s > 0 && !q.jac) return;  // the gradient comes from the vector-Jacobian product
  const int tiles = rl_tiles(q.n_ell);
  double v = 0.0;
  for (int t = 0; t < tiles; ++t) v += q.part[(size_t)t * 9 + s];
  q.out[s] = s == 0 ? -0.5 * v : -v;
}

void launch_request_loglike(const ReqLL* items_dev, int n, int max_tiles, int max_cls, cudaStream_t st) {
  const size_t smem = sizeof(double) * (size_t)max_cls * RL_ELL;
  dim3 grid(max_tiles, n);
  request_loglike_part_kernel<<<grid, 128, smem, st>>>(items_dev, n);
  request_loglike_sum_kernel<<<(9 * n + 127) / 128, 128, 0, st>>>(items_dev, n);
}

void launch_loglike(const double* data, const double* mu, const double* cov, int n_cosmo, int n_cls,
                    int n_ell, int include_logdet, int dense, double* out, int* status,
                    double* partial, int* structure, double* alpha, cudaStream_t st) {
  zero_int_kernel<<<(n_cosmo + 255) / 256, 256, 0, st>>>(status, n_cosmo);
  if (dense) {
    zero_int_kernel<<<(n_cosmo + 255) / 256, 256, 0, st>>>(structure, n_cosmo);
    const size_t N = (size_t)n_cls * n_ell;
    const size_t total = N * N * n_cosmo;
    size_t blocks = (total + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    dense_structure_kernel<<<(unsigned)blocks, 256, 0, st>>>(cov, n_cosmo, n_cls, n_ell, structure);
  }
  const size_t smem = ((size_t)n_cls * n_cls + 2 * n_cls) * sizeof(double);
  cudaFuncSetAttribute(loglike_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid(n_ell, n_cosmo);
  const int threads = n_cls >= 64 ? 256 : 128;
  loglike_blocks_kernel<<<grid, threads, smem, st>>>(data, mu, cov, n_cls, n_ell, dense,
                                                      dense ? structure : nullptr, partial, status,
                                                      alpha);
  loglike_reduce_kernel<<<(n_cosmo + 127) / 128, 128, 0, st>>>(partial, n_cosmo, n_ell,
                                                               include_logdet, out);
  if (dense) {
    // status 1 where the dense matrix is not block diagonal in ell
    merge_structure_kernel<<<(n_cosmo + 255) / 256, 256, 0, st>>>(structure, status, n_cosmo);
  }
}

// -------------------------------------------------- sparse-format algebra ---
// One CTA per (diagonal index l, matrix b): in-place Gauss-Jordan inversion
// with partial (row) pivoting of the n x n matrix A_l[i][j] = sparse[b][i][j][l]
// (sparse.py:295-315), or its log|det| and sign (sparse.py:322-366 computes
// the same by Schur complements).  In place, so one n x n FP64 block of
// shared memory: n <= SPARSE_MAX_N.  The row swaps are undone on the columns
// at the end (the inverse of P A is A^-1 P^T).
constexpr int SPARSE_MAX_N = 160;

__global__ void __launch_bounds__(256) sparse_gj_kernel(const double* __restrict__ sp, int n, int nd, int mode,
                                                        double* __restrict__ out, double* __restrict__ sign_part,
                                                        double* __restrict__ logdet_part) {
  const int l = blockIdx.x;
  const size_t mat = (size_t)blockIdx.y * n * n * nd;
  extern __shared__ double A[];  // n x n, row-major
  __shared__ double fcol[SPARSE_MAX_N];
  __shared__ int perm[SPARSE_MAX_N];
  __shared__ double wv[8];
  __shared__ int wi[8];
  __shared__ int piv;
  __shared__ double sgn, ld;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  for (int e = tid; e < n * n; e += nt) A[e] = sp[mat + (size_t)e * nd + l];
  if (tid == 0) {
    sgn = 1.0;
    ld = 0.0;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    // pivot: the first row i >= k of largest |A[i][k]|
    double bv = -1.0;
    int bi = n;
    for (int i = k + tid; i < n; i += nt) {
      const double v = fabs(A[i * n + k]);
      if (v > bv) { bv = v; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if (lane == 0) wv[warp] = bv, wi[warp] = bi;
    __syncthreads();
    if (tid == 0) {
      double v = wv[0];
      int p = wi[0];
      for (int w = 1; w < nt / 32; ++w)
        if (wv[w] > v || (wv[w] == v && wi[w] < p)) v = wv[w], p = wi[w];
      if (p >= n) p = k;
      piv = p;
      perm[k] = p;
      const double d = A[p * n + k];
      if (p != k) sgn = -sgn;
      sgn *= (d > 0.0) ? 1.0 : ((d < 0.0) ? -1.0 : 0.0);
      ld += log(fabs(d));
    }
    __syncthreads();
    const int p = piv;
    if (p != k)
      for (int j = tid; j < n; j += nt) {
        const double t = A[k * n + j];
        A[k * n + j] = A[p * n + j];
        A[p * n + j] = t;
      }
    __syncthreads();
    if (mode == 0) {
      const double pinv = 1.0 / A[k * n + k];
      for (int i = tid; i < n; i += nt) fcol[i] = A[i * n + k];
      __syncthreads();
      for (int j = tid; j < n; j += nt) A[k * n + j] = (j == k) ? pinv : A[k * n + j] * pinv;
      __syncthreads();
      for (int e = tid; e < n * n; e += nt) {
        const int i = e / n, j = e - (e / n) * n;
        if (i == k) continue;
        const double f = fcol[i];
        A[e] = (j == k) ? -f * pinv : A[e] - f * A[k * n + j];
      }
    } else {
      // determinant only: plain elimination below the pivot
      const double pinv = 1.0 / A[k * n + k];
      for (int e = tid; e < (n - k - 1) * (n - k); e += nt) {
        const int i = k + 1 + e / (n - k), j = k + e % (n - k);
        if (j == k) continue;
        A[i * n + j] -= A[i * n + k] * pinv * A[k * n + j];
      }
    }
    __syncthreads();
  }
  if (mode == 0) {
    // undo the row swaps on the columns, last swap first
    for (int k = n - 1; k >= 0; --k) {
      const int p = perm[k];
      if (p != k)
        for (int i = tid; i < n; i += nt) {
          const double t = A[i * n + k];
          A[i * n + k] = A[i * n + p];
          A[i * n + p] = t;
        }
      __syncthreads();
    }
    for (int e = tid; e < n * n; e += nt) out[mat + (size_t)e * nd + l] = A[e];
  } else if (tid == 0) {
    sign_part[(size_t)blockIdx.y * nd + l] = sgn;
    logdet_part[(size_t)blockIdx.y * nd + l] = ld;
  }
}

__global__ void sparse_slogdet_reduce(const double* sign_part, const double* ld_part, int nd,
                                      double* sign_out, double* logdet_out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 1.0, ld = 0.0;
    for (int l = 0; l < nd; ++l) {
      s *= sign_part[l];
      ld += ld_part[l];
    }
    *sign_out = s;
    *logdet_out = ld;
  }
}

static size_t sparse_gj_smem(int n) { return (size_t)n * n * sizeof(double); }

void launch_sparse_inv(const double* sp, int n_batch, int n, int nd, double* out, cudaStream_t st) {
  const size_t smem = sparse_gj_smem(n);
  cudaFuncSetAttribute(sparse_gj_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  sparse_gj_kernel<<<dim3(nd, n_batch), 256, smem, st>>>(sp, n, nd, 0, out, nullptr, nullptr);
}

void launch_sparse_slogdet(const double* sp, int n, int nd, double* sign_part, double* ld_part,
                           double* sign_out, double* ld_out, cudaStream_t st) {
  const size_t smem = sparse_gj_smem(n);
  cudaFuncSetAttribute(sparse_gj_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  sparse_gj_kernel<<<dim3(nd, 1), 256, smem, st>>>(sp, n, nd, 1, nullptr, sign_part, ld_part);
  sparse_slogdet_reduce<<<1, 32, 0, st>>>(sign_part, ld_part, nd, sign_out, ld_out);
}

// Products with at least one block-diagonal operand (sparse.py:140-292), one
// thread per output element, the fastest index of the output innermost so
// that loads and stores coalesce.
// sparse_dot_sparse (sparse.py:236-260): C[i][k][l] = sum_j A[i][j][l] B[j][k][l]
__global__ void sparse_dot_sparse_kernel(const double* __restrict__ a, const double* __restrict__ b, int n, int m,
                                         int p, int nd, double* __restrict__ c) {
  const size_t total = (size_t)n * p * nd;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const int l = (int)(idx % nd);
    const size_t ik = idx / nd;
    const int i = (int)(ik / p), k = (int)(ik % p);
    double acc = 0.0;
    for (int j = 0; j < m; ++j) acc += a[((size_t)i * m + j) * nd + l] * b[((size_t)j * p + k) * nd + l];
    c[idx] = acc;
  }
}

// sparse_dot_dense (sparse.py:164-182): out[i nd + l][q] = sum_j A[i][j][l] D[j nd + l][q], D (m nd, K)
__global__ void sparse_dot_dense_kernel(const double* __restrict__ a, int n, int m, int nd,
                                        const double* __restrict__ d, int K, double* __restrict__ out) {
  const size_t total = (size_t)n * nd * K;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const int q = (int)(idx % K);
    const size_t row = idx / K;
    const int i = (int)(row / nd), l = (int)(row % nd);
    double acc = 0.0;
    for (int j = 0; j < m; ++j) acc += a[((size_t)i * m + j) * nd + l] * d[((size_t)j * nd + l) * K + q];
    out[idx] = acc;
  }
}

// dense_dot_sparse (sparse.py:210-233): out[r][j nd + l] = sum_i D[r][i nd + l] A[i][j][l], D (R, n nd)
__global__ void dense_dot_sparse_kernel(const double* __restrict__ d, int R, const double* __restrict__ a, int n,
                                        int m, int nd, double* __restrict__ out) {
  const size_t cols = (size_t)m * nd, total = (size_t)R * cols;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t r = idx / cols, col = idx % cols;
    const int j = (int)(col / nd), l = (int)(col % nd);
    const double* dr = d + r * (size_t)n * nd;
    double acc = 0.0;
    for (int i = 0; i < n; ++i) acc += dr[(size_t)i * nd + l] * a[((size_t)i * m + j) * nd + l];
    out[idx] = acc;
  }
}

// FP64 C[M][N] = X[M][Kd] T[Kd][N], 16 x 16 tiles through shared memory (the
// dense step of dense_dot_sparse_dot_dense, sparse.py:263-292)
__global__ void __launch_bounds__(256) gemm_f64_kernel(const double* __restrict__ x, const double* __restrict__ t,
                                                       int M, int Kd, int N, double* __restrict__ c) {
  __shared__ double xs[16][17], ts[16][17];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int row = blockIdx.y * 16 + ty, col = blockIdx.x * 16 + tx;
  double acc = 0.0;
  for (int k0 = 0; k0 < Kd; k0 += 16) {
    xs[ty][tx] = (row < M && k0 + tx < Kd) ? x[(size_t)row * Kd + k0 + tx] : 0.0;
    ts[ty][tx] = (k0 + ty < Kd && col < N) ? t[(size_t)(k0 + ty) * N + col] : 0.0;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) acc += xs[ty][k] * ts[k][tx];
    __syncthreads();
  }
  if (row < M && col < N) c[(size_t)row * N + col] = acc;
}

static unsigned grid_for(size_t total) {
  size_t blocks = (total + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  return blocks ? (unsigned)blocks : 1u;
}

void launch_sparse_dot_sparse(const double* a, const double* b, int n, int m, int p, int nd, double* c,
                              cudaStream_t st) {
  sparse_dot_sparse_kernel<<<grid_for((size_t)n * p * nd), 256, 0, st>>>(a, b, n, m, p, nd, c);
}

void launch_sparse_dot_dense(const double* a, int n, int m, int nd, const double* d, int K, double* out,
                             cudaStream_t st) {
  sparse_dot_dense_kernel<<<grid_for((size_t)n * nd * K), 256, 0, st>>>(a, n, m, nd, d, K, out);
}

void launch_dense_dot_sparse(const double* d, int R, const double* a, int n, int m, int nd, double* out,
                             cudaStream_t st) {
  dense_dot_sparse_kernel<<<grid_for((size_t)R * m * nd), 256, 0, st>>>(d, R, a, n, m, nd, out);
}

void launch_gemm_f64(const double* x, const double* t, int M, int Kd, int N, double* c, cudaStream_t st) {
  dim3 grid((N + 15) / 16, (M + 15) / 16);
  gemm_f64_kernel<<<grid, 256, 0, st>>>(x, t, M, Kd, N, c);
}

// sparse.to_dense (sparse.py:52-68)
__global__ void sparse_to_dense_kernel(const double* __restrict__ sp, int n, int m, int nd,
                                       double* __restrict__ out) {
  const size_t R = (size_t)n * nd, C = (size_t)m * nd;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < R * C;
       idx += (size_t)gridDim.x * blockDim.x) {
    const size_t row = idx / C, col = idx % C;
    const int i = (int)(row / nd), l = (int)(row % nd), j = (int)(col / nd), l2 = (int)(col % nd);
    out[idx] = (l == l2) ? sp[((size_t)i * m + j) * nd + l] : 0.0;
  }
}

// sparse @ v (transpose = 0) or v @ sparse (transpose = 1) (sparse.py:140-233)
__global__ void sparse_dot_vec_kernel(const double* __restrict__ sp, int n, int m, int nd,
                                      const double* __restrict__ v, int transpose,
                                      double* __restrict__ out) {
  const int rows = transpose ? m : n;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= rows * nd) return;
  const int i = idx / nd, l = idx % nd;
  double acc = 0.0;
  if (!transpose) {
    for (int j = 0; j < m; ++j) acc += sp[((size_t)i * m + j) * nd + l] * v[(size_t)j * nd + l];
  } else {
    for (int j = 0; j < n; ++j) acc += v[(size_t)j * nd + l] * sp[((size_t)j * m + i) * nd + l];
  }
  out[idx] = acc;
}

void launch_sparse_to_dense(const double* sp, int n, int m, int nd, double* out, cudaStream_t st) {
  const size_t total = (size_t)n * nd * m * nd;
  size_t blocks = (total + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (blocks == 0) blocks = 1;
  sparse_to_dense_kernel<<<(unsigned)blocks, 256, 0, st>>>(sp, n, m, nd, out);
}

void launch_sparse_dot_vec(const double* sp, int n, int m, int nd, const double* v, int transpose,
                           double* out, cudaStream_t st) {
  const int rows = (transpose ? m : n) * nd;
  sparse_dot_vec_kernel<<<(rows + 127) / 128, 128, 0, st>>>(sp, n, m, nd, v, transpose, out);
}

}  // namespace jcg
