// Multi-right-hand-side (blocked) AMG-PCG: up to 32 right-hand sides share
// every pass over the matrices.  Vectors are row-major blocks, X[i * K + k],
// and every kernel is warp-per-row with lane k handling column k: a row's
// column indices and values are read once (one coalesced load of up to 32
// entries, then broadcast by shuffles) and applied to all K columns, whose
// gathers x[c * K + k] are contiguous.  Per column the arithmetic is the
// single-vector one (products in storage order, SOR row formula, aggregate
// sums in list order), so each column follows its own CG recurrence; the CG
// scalars are per column and a converged column is frozen.
//
// The outer iteration is FP64 (the finest matrix in FP64, FP64 dots); the
// preconditioner is the hierarchy's V-cycle in the hierarchy's cycle type
// (float for cycle_f32 hierarchies), with the coarsest solve through the
// FP64 dense inverse.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "lgx_amg.cuh"
#include "lgx_internal.cuh"

namespace lgx {

constexpr int kMaxRhs = 32;
constexpr int kMThreads = 256;  // 8 warps per CTA

__device__ __forceinline__ int64_t warp_id_global() {
  return ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
}
__device__ __forceinline__ int64_t warps_global() { return ((int64_t)gridDim.x * blockDim.x) >> 5; }

inline unsigned mgrid(int64_t rows) {
  const int64_t warps_per_block = kMThreads / 32;
  const int64_t g = (rows + warps_per_block - 1) / warps_per_block;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, 65535));
}

// y = A x (or r = b - A x with b != null) for rows [rb, re) of A, K columns
template <typename VT, typename XT>
__global__ void __launch_bounds__(kMThreads)
  k_mspmv(int64_t rb, int64_t re, const int64_t *__restrict__ rowptr,
          const int32_t *__restrict__ col, const VT *__restrict__ val, int K,
          const XT *__restrict__ b, const XT *__restrict__ x, XT *__restrict__ y) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = rb + warp_id_global(); i < re; i += warps_global()) {
    const int64_t e0 = rowptr[i], e1 = rowptr[i + 1];
    XT acc = XT(0);
    for (int64_t base = e0; base < e1; base += 32) {
      const int m = e1 - base < 32 ? (int)(e1 - base) : 32;
      int32_t c_l = 0;
      VT a_l = VT(0);
      if (lane < m) {
        c_l = col[base + lane];
        a_l = val[base + lane];
      }
      for (int u = 0; u < m; ++u) {
        const int32_t c = __shfl_sync(0xffffffffu, c_l, u);
        const XT a = (XT)__shfl_sync(0xffffffffu, a_l, u);
        if (lane < K) acc = fma(a, x[(int64_t)c * K + lane], acc);
      }
    }
    if (lane < K) y[i * K + lane] = b ? b[i * K + lane] - acc : acc;
  }
}

// One colour of a multicolour SOR sweep on K columns (the row formula of
// gauss-seidel-variant/sweep.hpp:134-200, in place).  from_zero: forward
// sweep from x = 0, rows at or after visit_end read as 0.
template <typename VT, typename XT>
__global__ void __launch_bounds__(kMThreads)
  k_msor(int64_t rb, int64_t re, const int64_t *__restrict__ rowptr,
         const int32_t *__restrict__ col, const VT *__restrict__ val, int K,
         const XT *__restrict__ b, XT *x, XT relax, XT m1, int ultra, int from_zero,
         int64_t visit_end) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = rb + warp_id_global(); i < re; i += warps_global()) {
    const int64_t e0 = rowptr[i], e1 = rowptr[i + 1];
    XT accum = lane < K ? b[i * K + lane] : XT(0);
    const XT xi = (lane < K && !from_zero) ? x[i * K + lane] : XT(0);
    XT diag = XT(0);
    for (int64_t base = e0; base < e1; base += 32) {
      const int m = e1 - base < 32 ? (int)(e1 - base) : 32;
      int32_t c_l = 0;
      VT a_l = VT(0);
      if (lane < m) {
        c_l = col[base + lane];
        a_l = val[base + lane];
      }
      for (int u = 0; u < m; ++u) {
        const int32_t c = __shfl_sync(0xffffffffu, c_l, u);
        const XT a = (XT)__shfl_sync(0xffffffffu, a_l, u);
        if (c == i) {
          diag = a;
          if (ultra) accum = fma(-a, xi, accum);
        } else if (lane < K) {
          const XT xv = (from_zero && c >= visit_end) ? XT(0) : x[(int64_t)c * K + lane];
          accum = fma(-a, xv, accum);
        }
      }
    }
    if (lane < K) {
      if (ultra) {
        x[i * K + lane] = xi + relax * accum / fabs(diag);
      } else {
        const XT quot = accum / diag;
        x[i * K + lane] = fma(relax, quot, m1 * xi);
      }
    }
  }
}

// b_c[c] = sum over the aggregate's fine rows (list order) of r
template <typename XT>
__global__ void __launch_bounds__(kMThreads)
  k_mrestrict(int64_t nc, const int64_t *__restrict__ rptr, const int32_t *__restrict__ rlist,
              int K, const XT *__restrict__ r, XT *__restrict__ bc) {
  const int lane = threadIdx.x & 31;
  if (lane >= K) return;
  for (int64_t c = warp_id_global(); c < nc; c += warps_global()) {
    XT s = XT(0);
    for (int64_t k = rptr[c]; k < rptr[c + 1]; ++k) s = s + r[(int64_t)rlist[k] * K + lane];
    bc[c * K + lane] = s;
  }
}

// x_f += inv_relax * refine(x_c)
template <typename XT>
__global__ void k_mprolong(int64_t n, const uint32_t *__restrict__ agg_p, int K,
                           const XT *__restrict__ xc, XT inv_relax, XT *__restrict__ x) {
  const int64_t total = n * K;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / K;
    const int k = (int)(t - i * K);
    const uint32_t a = agg_p[i];
    const XT ref = a < kIsolated ? xc[(int64_t)a * K + k] : XT(0);
    x[t] = x[t] + ref * inv_relax;
  }
}

// X = A^-1 B with the FP64 dense inverse, warp per row, lane = column
template <typename XT>
__global__ void __launch_bounds__(kMThreads)
  k_mdense(int64_t n, const double *__restrict__ ainv, int K, const XT *__restrict__ b,
           XT *__restrict__ x) {
  const int lane = threadIdx.x & 31;
  if (lane >= K) return;
  for (int64_t i = warp_id_global(); i < n; i += warps_global()) {
    const double *row = ainv + i * n;
    double acc = 0.0;
    for (int64_t j = 0; j < n; ++j) acc = fma(row[j], (double)b[j * K + lane], acc);
    x[i * K + lane] = (XT)acc;
  }
}

template <typename T, typename U>
__global__ void k_mconvert(int64_t total, const T *__restrict__ src, U *__restrict__ dst) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    dst[t] = (U)src[t];
}

// row blocks between natural and permuted order: dst[r] = src[perm[r]]
// (gather) or dst[perm[r]] = src[r] (scatter)
__global__ void k_mpermute(int64_t n, const int32_t *__restrict__ perm, int K, int scatter,
                           const double *__restrict__ src, double *__restrict__ dst) {
  const int64_t total = n * K;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / K;
    const int k = (int)(t - r * K);
    const int64_t p = perm[r];
    if (scatter) {
      dst[p * K + k] = src[t];
    } else {
      dst[t] = src[p * K + k];
    }
  }
}

// Per-column dots: out[k] = sum_i u[i,k] v[i,k] and (w != null) out[K + k] =
// sum_i w[i,k]^2.  Each block reduces a fixed strided set of rows per column
// in a fixed tree; the host adds the block partials in index order.
__global__ void __launch_bounds__(kMThreads)
  k_mdot(int64_t n, int K, const double *__restrict__ u, const double *__restrict__ v,
         const double *__restrict__ w, double *__restrict__ partials) {
  __shared__ double sh[2][kMThreads / 32][kMaxRhs];
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  double s1 = 0.0, s2 = 0.0;
  if (lane < K) {
    for (int64_t i = warp_id_global(); i < n; i += warps_global()) {
      const int64_t t = i * K + lane;
      s1 = fma(u[t], v[t], s1);
      if (w) s2 = fma(w[t], w[t], s2);
    }
  }
  sh[0][wl][lane] = s1;
  sh[1][wl][lane] = s2;
  __syncthreads();
  if (threadIdx.x < 2 * kMaxRhs) {
    const int which = threadIdx.x / kMaxRhs, k = threadIdx.x % kMaxRhs;
    double t = 0.0;
    for (int q = 0; q < kMThreads / 32; ++q) t += sh[which][q][k];
    partials[((int64_t)blockIdx.x * 2 + which) * kMaxRhs + k] = t;
  }
}

// X += alpha P, R -= alpha Q (alpha per column)
__global__ void k_mupdate(int64_t n, int K, const double *__restrict__ alpha,
                          const double *__restrict__ p, const double *__restrict__ q,
                          double *__restrict__ x, double *__restrict__ r) {
  const int64_t total = n * K;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double a = alpha[t % K];
    x[t] = fma(p[t], a, x[t]);
    r[t] = fma(-a, q[t], r[t]);
  }
}

// P = Z + beta P for active columns (beta NaN marks a frozen column)
__global__ void k_mxpby(int64_t n, int K, const double *__restrict__ beta,
                        const double *__restrict__ z, double *__restrict__ p) {
  const int64_t total = n * K;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double bk = beta[t % K];
    if (bk == bk) p[t] = fma(p[t], bk, z[t]);
  }
}

inline unsigned egrid(int64_t total) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 16384));
}

// ---- multi-column V-cycle (permuted spaces) -------------------------------
template <typename XT>
struct MWork {
  std::vector<DBuf<XT>> b, x, r;
};

template <typename XT>
static lgx_status m_level_sor(const lgx_amg &h, const lgx_amg_level &lv, int K, int forward,
                              int from_zero, const XT *b, XT *x, cudaStream_t s) {
  const lgx_colouring &c = *lv.col;
  const Csr &p = c.pcsr;
  const XT relax = (XT)h.p.smoother_relax, m1 = XT(1) - (XT)h.p.smoother_relax;
  const int ultra = h.p.smoother_ultra;
  for (int32_t k = 0; k < c.ncolours; ++k) {
    const int32_t cid = forward ? k : c.ncolours - 1 - k;
    const int64_t rb = c.offsets[cid], re = c.offsets[cid + 1];
    if (re <= rb) continue;
    const int fz = from_zero && forward;
    if constexpr (sizeof(XT) == 8) {
      if (p.storage == LGX_F64)
        k_msor<double, double><<<mgrid(re - rb), kMThreads, 0, s>>>(
          rb, re, p.rowptr.p, p.col.p, p.v64.p, K, b, x, relax, m1, ultra, fz, rb);
      else
        k_msor<float, double><<<mgrid(re - rb), kMThreads, 0, s>>>(
          rb, re, p.rowptr.p, p.col.p, p.v32.p, K, b, x, relax, m1, ultra, fz, rb);
    } else {
      const float *v = p.storage == LGX_F32 ? p.v32.p : c.pv32.p;
      k_msor<float, float><<<mgrid(re - rb), kMThreads, 0, s>>>(rb, re, p.rowptr.p, p.col.p, v,
                                                                 K, b, x, relax, m1, ultra, fz,
                                                                 rb);
    }
    LGX_LAUNCH_CHECK();
  }
  return LGX_OK;
}

template <typename XT>
static lgx_status m_level_residual(const lgx_amg_level &lv, int K, const XT *b, const XT *x,
                                   XT *r, cudaStream_t s) {
  const Csr &p = lv.col->pcsr;
  if constexpr (sizeof(XT) == 8) {
    if (p.storage == LGX_F64)
      k_mspmv<double, double><<<mgrid(p.n), kMThreads, 0, s>>>(0, p.n, p.rowptr.p, p.col.p,
                                                               p.v64.p, K, b, x, r);
    else
      k_mspmv<float, double><<<mgrid(p.n), kMThreads, 0, s>>>(0, p.n, p.rowptr.p, p.col.p,
                                                              p.v32.p, K, b, x, r);
  } else {
    const float *v = p.storage == LGX_F32 ? p.v32.p : lv.col->pv32.p;
    k_mspmv<float, float><<<mgrid(p.n), kMThreads, 0, s>>>(0, p.n, p.rowptr.p, p.col.p, v, K, b,
                                                           x, r);
  }
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

template <typename XT>
static lgx_status m_vcycle(const lgx_amg &h, int K, MWork<XT> &w, const XT *b0, XT *x0,
                           cudaStream_t s) {
  const int64_t L = (int64_t)h.lv.size();
  auto bv = [&](int64_t l) { return l == 0 ? b0 : (const XT *)w.b[l].p; };
  auto xv = [&](int64_t l) { return l == 0 ? x0 : w.x[l].p; };
  for (int64_t l = 0; l + 1 < L; ++l) {
    const lgx_amg_level &lv = *h.lv[l];
    if (lv.a->n == 0) continue;
    LGX_CHECK(m_level_sor<XT>(h, lv, K, 1, 1, bv(l), xv(l), s));
    LGX_CHECK(m_level_residual<XT>(lv, K, bv(l), xv(l), w.r[l].p, s));
    const int64_t nc = h.lv[l + 1]->a->n;
    if (nc) {
      k_mrestrict<XT><<<mgrid(nc), kMThreads, 0, s>>>(nc, lv.rptr.p, lv.rlist.p, K, w.r[l].p,
                                                      w.b[l + 1].p);
      LGX_LAUNCH_CHECK();
    }
  }
  {
    const int64_t nc = h.lv[L - 1]->a->n;
    if (nc) {
      k_mdense<XT><<<mgrid(nc), kMThreads, 0, s>>>(nc, h.inv.p, K, bv(L - 1), xv(L - 1));
      LGX_LAUNCH_CHECK();
    }
  }
  const XT inv_relax = (XT)(1.0 / h.p.relax);
  for (int64_t l = L - 2; l >= 0; --l) {
    const lgx_amg_level &lv = *h.lv[l];
    const int64_t n = lv.a->n;
    if (n == 0) continue;
    k_mprolong<XT><<<egrid(n * K), 256, 0, s>>>(n, lv.agg_p.p, K, xv(l + 1), inv_relax, xv(l));
    LGX_LAUNCH_CHECK();
    LGX_CHECK(m_level_sor<XT>(h, lv, K, 0, 0, bv(l), xv(l), s));
  }
  return LGX_OK;
}

// Per-column CG scalars of the blocked solver.  They stay on the device, so
// that an iteration needs no host round trip and is captured once as a
// CUDA graph; the host reads the block once per iteration for the stopping
// test.
struct MState {
  double rho[kMaxRhs], r0[kMaxRhs], res2[kMaxRhs];
  int64_t it_done[kMaxRhs];  // last iteration each column took part in
  int active[kMaxRhs];
  int64_t it;                // iterations completed
  int n_active;
  int flags;                 // 1: p.Ap = 0 (breakdown), 2: non-finite
  int bad_col;               // lowest column that raised `flags`
};

// column k of the k_mdot block partials (`which` 0: u.v, 1: w.w), summed in
// block order
__device__ double m_column_sum(const double *partials, unsigned g, int which, int k) {
  double a = 0.0;
  for (unsigned q = 0; q < g; ++q) a += partials[((size_t)q * 2 + which) * kMaxRhs + k];
  return a;
}

__device__ void m_raise(MState *st, unsigned mask, int flag) {
  if (mask && threadIdx.x == 0) {
    st->flags |= flag;
    st->bad_col = __ffs(mask) - 1;
  }
}

// rho = R.Z, r0 = ||R||, active = r0 > 0 and rho != 0 (one warp)
__global__ void k_minit(unsigned g, int K, const double *__restrict__ partials, int64_t maxit,
                        MState *st) {
  const int k = threadIdx.x;
  int act = 0, bad = 0;
  if (k < K) {
    const double rho = m_column_sum(partials, g, 0, k);
    const double res2 = m_column_sum(partials, g, 1, k);
    bad = !isfinite(res2) || !isfinite(rho);
    st->rho[k] = rho;
    st->res2[k] = res2;
    st->r0[k] = sqrt(res2);
    act = !bad && st->r0[k] > 0.0 && rho != 0.0 && maxit > 0;
    st->active[k] = act;
    st->it_done[k] = 0;
  }
  const unsigned am = __ballot_sync(~0u, act), bm = __ballot_sync(~0u, bad);
  if (k == 0) {
    st->n_active = __popc(am);
    st->it = 0;
    st->flags = 0;
    st->bad_col = -1;
  }
  __syncwarp();
  m_raise(st, bm, 2);
}

// alpha = rho / P.Q for active columns, 0 for the others
__global__ void k_malpha(unsigned g, int K, const double *__restrict__ partials, MState *st,
                         double *__restrict__ alpha) {
  const int k = threadIdx.x;
  double a = 0.0;
  int zero = 0, bad = 0;
  if (k < K && st->active[k]) {
    const double den = m_column_sum(partials, g, 0, k);
    bad = !isfinite(den);
    zero = den == 0.0;
    if (!bad && !zero) a = st->rho[k] / den;
  }
  if (k < K) alpha[k] = a;
  const unsigned zm = __ballot_sync(~0u, zero), bm = __ballot_sync(~0u, bad);
  m_raise(st, zm, 1);
  __syncwarp();
  m_raise(st, bm, 2);
}

// stopping test and beta = rho_new / rho; converged and inactive columns get
// a NaN beta (k_mxpby leaves their P frozen)
__global__ void k_mbeta(unsigned g, int K, const double *__restrict__ partials, double rtol,
                        MState *st, double *__restrict__ beta) {
  const int k = threadIdx.x;
  const int64_t it = st->it + 1;
  double b = __longlong_as_double(0x7ff8000000000000ll);
  int act = 0;
  if (k < K) {
    const double rho_new = m_column_sum(partials, g, 0, k);
    const double res2 = m_column_sum(partials, g, 1, k);
    st->res2[k] = res2;
    if (st->active[k]) {
      st->it_done[k] = it;
      if (sqrt(res2) <= rtol * st->r0[k] || rho_new == 0.0) {
        st->active[k] = 0;
      } else {
        b = rho_new / st->rho[k];
        st->rho[k] = rho_new;
        act = 1;
      }
    }
    beta[k] = b;
  }
  const unsigned am = __ballot_sync(~0u, act);
  if (k == 0) {
    st->n_active = __popc(am);
    st->it = it;
  }
}

// owns the captured iterations and the stream they are recorded on
struct MGraphs {
  cudaStream_t capture = nullptr;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  ~MGraphs() {
    for (auto &e : exec)
      if (e) cudaGraphExecDestroy(e);
    if (capture) cudaStreamDestroy(capture);
  }
};

template <typename XT>
static lgx_status pcg_multi(const lgx_matrix *a, lgx_amg &h, int K, const double *d_b,
                            double *d_x, double rtol, int64_t maxit, int use_graphs,
                            cudaStream_t user_stream, int64_t *h_it, double *h_rel) {
  const int64_t n = a->n;
  const int64_t L = (int64_t)h.lv.size();
  const bool permuted = L > 1;
  const Csr &A = permuted ? h.lv[0]->col->pcsr : a->csr;
  const int32_t *perm = permuted ? h.lv[0]->col->perm.p : nullptr;
  const int64_t nk = n * K;
  // the stream every launch below goes to: the caller's, or the capture
  // stream while an iteration is recorded
  cudaStream_t s = user_stream;
  // outer vectors (permuted order): B, X, R, P, Q, Z
  DBuf<double> B, X, R, P, Q, Z, alpha_d, beta_d, partials;
  DBuf<MState> state;
  for (DBuf<double> *v : {&B, &X, &R, &P, &Q, &Z}) LGX_CHECK(v->alloc(std::max<int64_t>(nk, 1)));
  LGX_CHECK(alpha_d.alloc(kMaxRhs));
  LGX_CHECK(beta_d.alloc(kMaxRhs));
  LGX_CHECK(partials.alloc(1024 * 2 * kMaxRhs));
  LGX_CHECK(state.alloc(1));
  const unsigned gdot = std::min<unsigned>(mgrid(n), 1024);
  if (perm) {
    k_mpermute<<<egrid(nk), 256, 0, s>>>(n, perm, K, 0, d_b, B.p);
    k_mpermute<<<egrid(nk), 256, 0, s>>>(n, perm, K, 0, d_x, X.p);
    LGX_LAUNCH_CHECK();
  } else {
    LGX_CUDA(cudaMemcpyAsync(B.p, d_b, sizeof(double) * nk, cudaMemcpyDeviceToDevice, s));
    LGX_CUDA(cudaMemcpyAsync(X.p, d_x, sizeof(double) * nk, cudaMemcpyDeviceToDevice, s));
  }
  // V-cycle workspace (cycle type XT); level 0 of a float cycle has its own b/x
  MWork<XT> w;
  w.b.resize(L);
  w.x.resize(L);
  w.r.resize(L);
  for (int64_t l = 0; l < L; ++l) {
    const int64_t nl = std::max<int64_t>(h.lv[l]->a->n * K, 1);
    LGX_CHECK(w.r[l].alloc(nl));
    if (l > 0 || sizeof(XT) == 4) {
      LGX_CHECK(w.b[l].alloc(nl));
      LGX_CHECK(w.x[l].alloc(nl));
    }
  }
  auto precondition = [&](const double *r, double *z) -> lgx_status {
    if constexpr (sizeof(XT) == 8) {
      return m_vcycle<double>(h, K, w, r, z, s);
    } else {
      k_mconvert<double, float><<<egrid(nk), 256, 0, s>>>(nk, r, w.b[0].p);
      LGX_LAUNCH_CHECK();
      LGX_CHECK(m_vcycle<float>(h, K, w, w.b[0].p, w.x[0].p, s));
      k_mconvert<float, double><<<egrid(nk), 256, 0, s>>>(nk, w.x[0].p, z);
      LGX_LAUNCH_CHECK();
      return LGX_OK;
    }
  };
  auto apply = [&](const double *bb, const double *x, double *y) -> lgx_status {
    if (A.storage == LGX_F64)
      k_mspmv<double, double><<<mgrid(n), kMThreads, 0, s>>>(0, n, A.rowptr.p, A.col.p, A.v64.p,
                                                             K, bb, x, y);
    else
      k_mspmv<float, double><<<mgrid(n), kMThreads, 0, s>>>(0, n, A.rowptr.p, A.col.p, A.v32.p,
                                                            K, bb, x, y);
    LGX_LAUNCH_CHECK();
    return LGX_OK;
  };
  auto dots = [&](const double *u, const double *v, const double *ww) -> lgx_status {
    k_mdot<<<gdot, kMThreads, 0, s>>>(n, K, u, v, ww, partials.p);
    LGX_LAUNCH_CHECK();
    return LGX_OK;
  };
  // one iteration (conjugate-gradients/solver.hpp:75-117 per column); with
  // `rere` the residual is recomputed as B - A X (every 8th iteration)
  auto iteration = [&](int rere) -> lgx_status {
    // Q = A P ; alpha = rho / P.Q ; X += alpha P ; R -= alpha Q
    LGX_CHECK(apply(nullptr, P.p, Q.p));
    LGX_CHECK(dots(P.p, Q.p, nullptr));
    k_malpha<<<1, 32, 0, s>>>(gdot, K, partials.p, state.p, alpha_d.p);
    k_mupdate<<<egrid(nk), 256, 0, s>>>(n, K, alpha_d.p, P.p, Q.p, X.p, R.p);
    LGX_LAUNCH_CHECK();
    if (rere) LGX_CHECK(apply(B.p, X.p, R.p));
    // Z = M R ; beta = R.Z / rho ; P = Z + beta P
    LGX_CHECK(precondition(R.p, Z.p));
    LGX_CHECK(dots(R.p, Z.p, R.p));
    k_mbeta<<<1, 32, 0, s>>>(gdot, K, partials.p, rtol, state.p, beta_d.p);
    k_mxpby<<<egrid(nk), 256, 0, s>>>(n, K, beta_d.p, Z.p, P.p);
    LGX_LAUNCH_CHECK();
    return LGX_OK;
  };
  MGraphs graphs;
  auto capture = [&](int rere) -> lgx_status {
    if (!graphs.capture)
      LGX_CUDA(cudaStreamCreateWithFlags(&graphs.capture, cudaStreamNonBlocking));
    s = graphs.capture;
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    lgx_status st = e == cudaSuccess ? iteration(rere) : cuda_fail(e, "cudaStreamBeginCapture");
    const cudaError_t e2 = cudaStreamEndCapture(s, &gr);
    s = user_stream;
    if (st != LGX_OK) {
      if (gr) cudaGraphDestroy(gr);
      return st;
    }
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&graphs.exec[rere], gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return LGX_OK;
  };
  MState hs{};
  auto read_state = [&]() -> lgx_status {
    LGX_CUDA(cudaMemcpyAsync(&hs, state.p, sizeof(MState), cudaMemcpyDeviceToHost, s));
    LGX_CUDA(cudaStreamSynchronize(s));
    return LGX_OK;
  };
  // R = B - A X ; Z = M R ; rho = R.Z ; P = Z (conjugate-gradients/solver.hpp:50-73)
  LGX_CHECK(apply(B.p, X.p, R.p));
  LGX_CHECK(precondition(R.p, Z.p));
  LGX_CHECK(dots(R.p, Z.p, R.p));
  k_minit<<<1, 32, 0, s>>>(gdot, K, partials.p, maxit, state.p);
  LGX_LAUNCH_CHECK();
  LGX_CUDA(cudaMemcpyAsync(P.p, Z.p, sizeof(double) * nk, cudaMemcpyDeviceToDevice, s));
  LGX_CHECK(read_state());
  if (hs.flags & 2)
    return fail(LGX_ERR_NONFINITE,
                "non-finite initial residual in column " + std::to_string(hs.bad_col));
  int64_t it = 0;
  while (hs.n_active > 0 && it < maxit) {
    const int rere = (it + 1) % 8 == 0;
    if (use_graphs && it > 0) {
      // the first iteration ran eagerly; later ones replay the recording
      if (!graphs.exec[rere]) LGX_CHECK(capture(rere));
      LGX_CUDA(cudaGraphLaunch(graphs.exec[rere], s));
    } else {
      LGX_CHECK(iteration(rere));
    }
    ++it;
    LGX_CHECK(read_state());
    if (hs.flags)
      return fail(hs.flags & 2 ? LGX_ERR_NONFINITE : LGX_ERR_BREAKDOWN,
                  "column " + std::to_string(hs.bad_col) + ": p.Ap is zero or non-finite");
  }
  for (int k = 0; k < K; ++k) {
    h_it[k] = hs.it_done[k];
    h_rel[k] = hs.r0[k] > 0.0 ? std::sqrt(hs.res2[k]) / hs.r0[k] : 0.0;
  }
  if (perm) {
    k_mpermute<<<egrid(nk), 256, 0, s>>>(n, perm, K, 1, X.p, d_x);
    LGX_LAUNCH_CHECK();
  } else {
    LGX_CUDA(cudaMemcpyAsync(d_x, X.p, sizeof(double) * nk, cudaMemcpyDeviceToDevice, s));
  }
  LGX_CUDA(cudaStreamSynchronize(s));
  if (hs.n_active > 0)
    return fail(LGX_ERR_NOT_CONVERGED, "maxit reached before every column converged");
  return LGX_OK;
}

}  // namespace lgx

using namespace lgx;

extern "C" {

lgx_status lgx_pcg_multi(const lgx_matrix *a, lgx_amg *amg, int32_t nrhs, const double *d_b,
                         double *d_x, double rtol, int64_t maxit, int use_graphs,
                         lgx_stream stream, int64_t *h_iterations, double *h_rel_residual) {
  if (!a || !amg) return fail(LGX_ERR_INVALID, "null matrix or hierarchy");
  if (nrhs < 1 || nrhs > kMaxRhs) return fail(LGX_ERR_INVALID, "nrhs must be in [1, 32]");
  if (a->kind != LGX_MATRIX_CSR || amg->lv.empty() || amg->lv[0]->a != &a->csr)
    return fail(LGX_ERR_INVALID, "the hierarchy was not built from this CSR matrix");
  if (a->n > 0 && (!d_b || !d_x)) return fail(LGX_ERR_INVALID, "null vector");
  std::vector<int64_t> it(nrhs, 0);
  std::vector<double> rel(nrhs, 0.0);
  lgx_status st = amg->f32 ? pcg_multi<float>(a, *amg, nrhs, d_b, d_x, rtol, maxit, use_graphs,
                                               stream, it.data(), rel.data())
                           : pcg_multi<double>(a, *amg, nrhs, d_b, d_x, rtol, maxit, use_graphs,
                                                stream, it.data(), rel.data());
  if (h_iterations) std::copy(it.begin(), it.end(), h_iterations);
  if (h_rel_residual) std::copy(rel.begin(), rel.end(), h_rel_residual);
  return st;
}

}  // extern "C"
