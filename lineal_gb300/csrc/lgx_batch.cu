// Batching form: many independent 7-point upwind convection-diffusion systems
// (the operator of a constant velocity v and D = 1 on an n0 x n1 x n2 grid,
// unit spacing, zero Dirichlet values outside) solved by Jacobi-BiCGStab in
// ONE persistent launch.
//
// Each CTA takes systems from a work queue (largest first) and runs the whole
// BiCGStab iteration of bicgstab/solver.hpp:73-151 for that system itself:
// the operator is matrix-free (seven constants per system, products in the
// CSR row order -d0, -d1, -d2, diagonal, +d2, +d1, +d0 of the assembled
// matrix), phases are separated by __syncthreads, the dot products are
// fixed-shape block reductions (deterministic), and the termination test
// (||r|| <= rtol ||r0||, maxit, rho == 0, as run_iterative_solver) is taken
// on the device.  No host round trip and no further launch happens until
// every system is done.  A system that the alpha step solves exactly (r = 0,
// where the reference's omega = 0 / 0 would give NaN) ends as converged.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "lgx_internal.cuh"

namespace lgx {

int sm_count();

constexpr int kBatchThreads = 512;

struct BatchSys {
  int32_t n0, n1, n2;
  int64_t off;      // first row in the concatenated vectors
  double c[6];      // |a_ij| toward -d0, +d0, -d1, +d1, -d2, +d2
  double diag, rdiag;
};

namespace {

// Jacobi from zero, fma(relax, p / d, m1 * 0): the quotient as p times the
// reciprocal of the system's constant diagonal (one FP64 multiply instead of
// a division; within an ulp of the quotient), and for relax = 1 the product
// itself (fma(1, q, +0) == q for q != 0; both are zero otherwise).
__device__ __forceinline__ double jacobi0(const BatchSys &S, double p, double relax, double m1,
                                          bool relax_one) {
  const double q = S.rdiag != 0.0 ? p * S.rdiag : p / S.diag;
  return relax_one ? q + 0.0 : fma(relax, q, m1 * 0.0);
}

// (A x)_i in the assembled row's column order
__device__ __forceinline__ double apply_row(const BatchSys &S, const double *x, int64_t i,
                                            int p0, int p1, int p2) {
  const int64_t s1 = S.n2, s0 = (int64_t)S.n1 * S.n2;
  double ax = 0.0;
  if (p0 > 0) ax = fma(-S.c[0], x[i - s0], ax);
  if (p1 > 0) ax = fma(-S.c[2], x[i - s1], ax);
  if (p2 > 0) ax = fma(-S.c[4], x[i - 1], ax);
  ax = fma(S.diag, x[i], ax);
  if (p2 + 1 < S.n2) ax = fma(-S.c[5], x[i + 1], ax);
  if (p1 + 1 < S.n1) ax = fma(-S.c[3], x[i + s1], ax);
  if (p0 + 1 < S.n0) ax = fma(-S.c[1], x[i + s0], ax);
  return ax;
}

template <int T>
__device__ __forceinline__ void block_sum3(double &a, double &b, double &c, double *sh) {
  double *sa = sh, *sb = sh + T, *sc = sh + 2 * T;
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  sc[threadIdx.x] = c;
  __syncthreads();
#pragma unroll
  for (int s = T / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sa[threadIdx.x] += sa[threadIdx.x + s];
      sb[threadIdx.x] += sb[threadIdx.x + s];
      sc[threadIdx.x] += sc[threadIdx.x + s];
    }
    __syncthreads();
  }
  a = sa[0];
  b = sb[0];
  c = sc[0];
  __syncthreads();
}

template <int T>
__device__ __forceinline__ void block_sum2(double &a, double &b, double *sh) {
  double *sa = sh, *sb = sh + T;
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
#pragma unroll
  for (int s = T / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sa[threadIdx.x] += sa[threadIdx.x + s];
      sb[threadIdx.x] += sb[threadIdx.x + s];
    }
    __syncthreads();
  }
  a = sa[0];
  b = sb[0];
  __syncthreads();
}

struct Pos {
  int p0, p1, p2;
};
__device__ __forceinline__ Pos pos_of(const BatchSys &S, int64_t i) {
  const unsigned u = (unsigned)i, n2 = (unsigned)S.n2, n1 = (unsigned)S.n1;
  const unsigned q = u / n2;
  return Pos{(int)(q / n1), (int)(q % n1), (int)(u % n2)};
}

}  // namespace

// status: 0 converged, 1 breakdown, 2 non-finite, 3 maxit reached
__global__ void __launch_bounds__(kBatchThreads)
  k_batch_bicgstab(int32_t nsys, const BatchSys *__restrict__ sys, const int32_t *__restrict__ order,
                   unsigned *queue, const double *__restrict__ bvec, double *xvec, double *ws,
                   int64_t total, double rtol, int64_t maxit, int64_t rere, double relax,
                   int64_t *iters_out, double *rel_out, int *status_out) {
  constexpr int T = kBatchThreads;
  __shared__ double sh[3 * T];
  __shared__ int s_q;
  const double m1 = 1.0 - relax;
  const bool relax_one = relax == 1.0;
  for (;;) {
    if (threadIdx.x == 0) s_q = (int)atomicAdd(queue, 1u);
    __syncthreads();
    const int q = s_q;
    __syncthreads();
    if (q >= nsys) return;
    const int id = order[q];
    const BatchSys S = sys[id];
    const int64_t n = (int64_t)S.n0 * S.n1 * S.n2;
    const double *b = bvec + S.off;
    double *x = xvec + S.off;
    double *r = ws + S.off, *r0 = ws + total + S.off, *p = ws + 2 * total + S.off,
           *v = ws + 3 * total + S.off, *t = ws + 4 * total + S.off, *z = ws + 5 * total + S.off;

    // r = b - A x, r0 = p = r, rho = ||r||^2 (bicgstab/solver.hpp:51-71)
    double res2 = 0.0, dummy = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += T) {
      const Pos P = pos_of(S, i);
      const double rv = b[i] - apply_row(S, x, i, P.p0, P.p1, P.p2);
      r[i] = rv;
      r0[i] = rv;
      p[i] = rv;
      res2 = fma(rv, rv, res2);
    }
    block_sum2<T>(res2, dummy, sh);
    const double r0n = sqrt(res2);
    double rho = res2, alpha = 0.0, omega = 0.0;
    int64_t it = 0;
    int status = 0;
    if (!isfinite(res2)) status = 2;
    while (status == 0 && it < maxit && sqrt(res2) > rtol * r0n && rho != 0.0) {
      // z = J(p)
      for (int64_t i = threadIdx.x; i < n; i += T) z[i] = jacobi0(S, p[i], relax, m1, relax_one);
      __syncthreads();
      // v = A z ; den = r0.v ; alpha = rho / den
      double den = 0.0;
      for (int64_t i = threadIdx.x; i < n; i += T) {
        const Pos P = pos_of(S, i);
        const double vv = apply_row(S, z, i, P.p0, P.p1, P.p2);
        v[i] = vv;
        den = fma(r0[i], vv, den);
      }
      block_sum2<T>(den, dummy, sh);
      if (!isfinite(rho) || !isfinite(den)) status = 2;
      if (den == 0.0) status = status ? status : 1;
      if (status) break;
      alpha = rho / den;
      // x += alpha z ; r -= alpha v (ss = ||r||^2) ; z = J(r)
      double ss = 0.0;
      for (int64_t i = threadIdx.x; i < n; i += T) {
        x[i] = fma(z[i], alpha, x[i]);
        const double rv = fma(-alpha, v[i], r[i]);
        r[i] = rv;
        ss = fma(rv, rv, ss);
        z[i] = jacobi0(S, rv, relax, m1, relax_one);
      }
      __syncthreads();
      // t = A z ; omega = t.r / t.t
      double tr = 0.0, tt = 0.0;
      for (int64_t i = threadIdx.x; i < n; i += T) {
        const Pos P = pos_of(S, i);
        const double tv = apply_row(S, z, i, P.p0, P.p1, P.p2);
        t[i] = tv;
        tr = fma(tv, r[i], tr);
        tt = fma(tv, tv, tt);
      }
      block_sum3<T>(tr, tt, ss, sh);
      if (ss == 0.0) {
        // the alpha step solved the system exactly (omega would be 0 / 0)
        ++it;
        res2 = 0.0;
        break;
      }
      if (!isfinite(tr) || !isfinite(tt)) status = 2;
      if (tt == 0.0) status = status ? status : 1;
      if (status) break;
      omega = tr / tt;
      ++it;
      const bool recompute = rere > 0 && it % rere == 0;
      // x += omega z ; r -= omega t (or r = b - A x) ; rho_new = r.r0, res2 = r.r
      for (int64_t i = threadIdx.x; i < n; i += T) x[i] = fma(z[i], omega, x[i]);
      if (recompute) __syncthreads();
      double rho_new = 0.0, rr = 0.0;
      for (int64_t i = threadIdx.x; i < n; i += T) {
        double rv;
        if (recompute) {
          const Pos P = pos_of(S, i);
          rv = b[i] - apply_row(S, x, i, P.p0, P.p1, P.p2);
        } else {
          rv = fma(-omega, t[i], r[i]);
        }
        r[i] = rv;
        rho_new = fma(rv, r0[i], rho_new);
        rr = fma(rv, rv, rr);
      }
      block_sum2<T>(rho_new, rr, sh);
      res2 = rr;
      if (!isfinite(rho_new) || !isfinite(omega) || !isfinite(rr)) status = 2;
      if (omega == 0.0) status = status ? status : 1;
      if (status) break;
      const double beta = (rho_new / rho) * (alpha / omega);
      rho = rho_new;
      // p = r + beta (p - omega v)
      for (int64_t i = threadIdx.x; i < n; i += T) p[i] = fma(fma(-omega, v[i], p[i]), beta, r[i]);
      __syncthreads();
    }
    if (status == 0 && sqrt(res2) > rtol * r0n && rho != 0.0) status = 3;
    if (threadIdx.x == 0) {
      iters_out[id] = it;
      rel_out[id] = r0n > 0.0 ? sqrt(res2) / r0n : 0.0;
      status_out[id] = status;
    }
    __syncthreads();
  }
}

}  // namespace lgx

using namespace lgx;

extern "C" {

lgx_status lgx_batch_convdiff_bicgstab(int32_t nsys, const lgx_convdiff_system *h_systems,
                                       const double *d_b, double *d_x, double rtol, int64_t maxit,
                                       int64_t rere_period, double relax, lgx_stream stream,
                                       int64_t *h_iterations, double *h_rel_residual,
                                       int32_t *h_status) {
  if (nsys < 0 || (nsys > 0 && !h_systems)) return fail(LGX_ERR_INVALID, "bad system list");
  if (nsys == 0) return LGX_OK;
  std::vector<BatchSys> sys(nsys);
  std::vector<int64_t> rows(nsys);
  int64_t total = 0;
  for (int32_t s = 0; s < nsys; ++s) {
    const lgx_convdiff_system &in = h_systems[s];
    if (in.dims[0] < 1 || in.dims[1] < 1 || in.dims[2] < 1)
      return fail(LGX_ERR_INVALID, "system with an empty grid");
    const int64_t n = in.dims[0] * in.dims[1] * in.dims[2];
    if (n > INT32_MAX) return fail(LGX_ERR_INVALID, "system too large");
    BatchSys &S = sys[s];
    S.n0 = (int32_t)in.dims[0];
    S.n1 = (int32_t)in.dims[1];
    S.n2 = (int32_t)in.dims[2];
    S.off = total;
    double diag = 0.0;
    for (int d = 0; d < 3; ++d) {
      const double up_minus = in.v[d] > 0.0 ? in.v[d] : 0.0;
      const double up_plus = in.v[d] < 0.0 ? -in.v[d] : 0.0;
      S.c[2 * d] = 1.0 + up_minus;
      S.c[2 * d + 1] = 1.0 + up_plus;
    }
    for (int e = 0; e < 6; ++e) diag = diag + S.c[e];
    S.diag = diag;
    const int ex = (int)((reinterpret_cast<const uint64_t &>(diag) >> 52) & 0x7ff);
    S.rdiag = (ex > 1023 - 400 && ex < 1023 + 400) ? 1.0 / diag : 0.0;
    rows[s] = n;
    total += n;
  }
  if (!d_b || !d_x) return fail(LGX_ERR_INVALID, "null vector");
  // largest systems first
  std::vector<int32_t> order(nsys);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return rows[a] > rows[b]; });
  DBuf<BatchSys> d_sys;
  DBuf<int32_t> d_order, d_status;
  DBuf<unsigned> d_queue;
  DBuf<double> ws, d_rel;
  DBuf<int64_t> d_iters;
  LGX_CHECK(d_sys.alloc(nsys));
  LGX_CHECK(d_order.alloc(nsys));
  LGX_CHECK(d_status.alloc(nsys));
  LGX_CHECK(d_queue.alloc(1));
  LGX_CHECK(ws.alloc(6 * total));
  LGX_CHECK(d_rel.alloc(nsys));
  LGX_CHECK(d_iters.alloc(nsys));
  LGX_CUDA(cudaMemcpyAsync(d_sys.p, sys.data(), sizeof(BatchSys) * nsys, cudaMemcpyHostToDevice,
                           stream));
  LGX_CUDA(cudaMemcpyAsync(d_order.p, order.data(), sizeof(int32_t) * nsys,
                           cudaMemcpyHostToDevice, stream));
  LGX_CUDA(cudaMemsetAsync(d_queue.p, 0, sizeof(unsigned), stream));
  int per_sm = 0;
  LGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_bicgstab,
                                                         kBatchThreads, 0));
  const int64_t g = (int64_t)sm_count() * std::max(per_sm, 1);
  const unsigned grid = (unsigned)std::min<int64_t>(g, nsys);
  k_batch_bicgstab<<<grid, kBatchThreads, 0, stream>>>(nsys, d_sys.p, d_order.p, d_queue.p, d_b,
                                                      d_x, ws.p, total, rtol, maxit, rere_period,
                                                      relax, d_iters.p, d_rel.p, d_status.p);
  LGX_LAUNCH_CHECK();
  std::vector<int64_t> it(nsys);
  std::vector<double> rel(nsys);
  std::vector<int32_t> st(nsys);
  LGX_CUDA(cudaMemcpyAsync(it.data(), d_iters.p, sizeof(int64_t) * nsys, cudaMemcpyDeviceToHost,
                           stream));
  LGX_CUDA(cudaMemcpyAsync(rel.data(), d_rel.p, sizeof(double) * nsys, cudaMemcpyDeviceToHost,
                           stream));
  LGX_CUDA(cudaMemcpyAsync(st.data(), d_status.p, sizeof(int32_t) * nsys, cudaMemcpyDeviceToHost,
                           stream));
  LGX_CUDA(cudaStreamSynchronize(stream));
  if (h_iterations) std::copy(it.begin(), it.end(), h_iterations);
  if (h_rel_residual) std::copy(rel.begin(), rel.end(), h_rel_residual);
  if (h_status) std::copy(st.begin(), st.end(), h_status);
  for (int32_t s = 0; s < nsys; ++s)
    if (st[s] == 1 || st[s] == 2)
      return fail(st[s] == 1 ? LGX_ERR_BREAKDOWN : LGX_ERR_NONFINITE,
                  "system " + std::to_string(s) + (st[s] == 1 ? ": breakdown" : ": non-finite"));
  return LGX_OK;
}

}  // extern "C"
