// Adjoint kernels of the differentiation form: for x = A(theta)^-1 b and a
// loss L(x), dL/dtheta = -lambda^T (dA/dtheta) x with lambda = A^-T dL/dx.
//
// * k_sampled_outer: the outer product lambda x^T sampled on the sparsity
//   pattern of A (out[e] = alpha * u[row(e)] * v[col(e)] for every stored
//   entry e), i.e. dL/dA restricted to the pattern for alpha = -1.  A caller
//   with its own parameterisation of the values contracts it with dA/dtheta.
// * k_diffusion7_grad: the contraction fused in for the 7-point operator of
//   lgx_gen_7pt with k = exp(theta) per cell: face coefficients
//   c_ij = hm(k_i, k_j) = 2 k_i k_j / (k_i + k_j) enter A_ii, A_jj with + and
//   A_ij, A_ji with -, and each axis-0 boundary face adds 2 k_i to A_ii
//   (the Dirichlet rows of the generator).  Hence
//     dL/dtheta_i = -( sum_j dc_ij/dtheta_i (lambda_i - lambda_j)(x_i - x_j)
//                     + nb_i 2 k_i lambda_i x_i ),
//     dc_ij/dtheta_i = k_i * 2 k_j^2 / (k_i + k_j)^2 = c_ij k_j / (k_i + k_j).
//   One thread per cell sums its six faces in a fixed order: no atomics, the
//   result is deterministic.  Bytes per cell: k, lambda, x (8 B each) plus the
//   neighbours' (cached) and the gradient (8 B).
// * k_residual_dot2: b - A x with compensated row sums, the residual of the
//   iterative refinement that makes finite-difference checks meaningful on
//   ill-conditioned grids.
#include <cuda_runtime.h>

#include <algorithm>

#include "lgx_internal.cuh"

namespace lgx {

__global__ void k_sampled_outer(int64_t n, const int64_t *__restrict__ rowptr,
                                const int32_t *__restrict__ col, double alpha,
                                const double *__restrict__ u, const double *__restrict__ v,
                                double *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double ui = alpha * u[i];
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e) out[e] = ui * __ldg(v + col[e]);
  }
}

__global__ void k_diffusion7_grad(int64_t n0, int64_t n1, int64_t n2,
                                  const double *__restrict__ k, const double *__restrict__ lam,
                                  const double *__restrict__ x, double *__restrict__ grad) {
  const int64_t n = n0 * n1 * n2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p0 = i / (n1 * n2), p1 = (i / n2) % n1, p2 = i % n2;
    const double ki = k[i], li = lam[i], xi = x[i];
    double acc = 0.0;
    const int64_t stride[3] = {n1 * n2, n2, 1};
    const int64_t pos[3] = {p0, p1, p2};
    const int64_t ext[3] = {n0, n1, n2};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
      for (int sgn = -1; sgn <= 1; sgn += 2) {
        const int64_t q = pos[d] + sgn;
        if (q < 0 || q >= ext[d]) continue;
        const int64_t j = i + sgn * stride[d];
        const double kj = k[j];
        const double s = ki + kj;
        const double dc = 2.0 * ki * kj * kj / (s * s);
        acc = fma(dc * (li - lam[j]), xi - x[j], acc);
      }
    }
    const int nb = (p0 == 0) + (p0 + 1 == n0);
    if (nb) acc = fma((double)nb * 2.0 * ki, li * xi, acc);
    grad[i] = -acc;
  }
}

// r = b - A x with every row's sum evaluated by the compensated dot product
// Dot2 of T. Ogita, S. M. Rump, S. Oishi, "Accurate sum and dot product",
// SIAM J. Sci. Comput. 26(6), 2005 (Algorithm 5.3): error-free products
// (fma) and sums (TwoSum) carry the rounding errors, so the row is as
// accurate as if computed in twice the working precision and then rounded.
// Used to refine solutions to full FP64 accuracy (finite-difference checks,
// FP64 verification).  About 10 FP64 operations per entry.
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = __dadd_rn(a, b);
  const double z = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, z)), __dsub_rn(b, z));
}

__global__ void k_residual_dot2(int64_t n, const int64_t *__restrict__ rowptr,
                                const int32_t *__restrict__ col, const double *__restrict__ val,
                                const double *__restrict__ b, const double *__restrict__ x,
                                double *__restrict__ r) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double p = b[i], s = 0.0;
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e) {
      const double a = -val[e], xv = x[col[e]];
      const double h = __dmul_rn(a, xv);
      const double hr = fma(a, xv, -h);
      double q;
      two_sum(p, h, p, q);
      s = __dadd_rn(s, __dadd_rn(q, hr));
    }
    r[i] = __dadd_rn(p, s);
  }
}

}  // namespace lgx

using namespace lgx;

extern "C" {

lgx_status lgx_sampled_outer(const lgx_matrix *a, double alpha, const double *d_u,
                             const double *d_v, double *d_out, lgx_stream stream) {
  if (!a) return fail(LGX_ERR_INVALID, "null matrix");
  if (a->kind != LGX_MATRIX_CSR)
    return fail(LGX_ERR_UNSUPPORTED, "lgx_sampled_outer needs a CSR matrix");
  if (a->n > 0 && (!d_u || !d_v || (a->nnz > 0 && !d_out)))
    return fail(LGX_ERR_INVALID, "null argument");
  if (a->n == 0) return LGX_OK;
  const Csr &c = a->csr;
  k_sampled_outer<<<std::min<unsigned>(grid_for(c.n, 256), 16384), 256, 0, stream>>>(
    c.n, c.rowptr.p, c.col.p, alpha, d_u, d_v, d_out);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

lgx_status lgx_residual_compensated(const lgx_matrix *a, const double *d_b, const double *d_x,
                                   double *d_r, lgx_stream stream) {
  if (!a) return fail(LGX_ERR_INVALID, "null matrix");
  if (a->kind != LGX_MATRIX_CSR || a->csr.storage != LGX_F64)
    return fail(LGX_ERR_UNSUPPORTED, "lgx_residual_compensated needs an FP64 CSR matrix");
  if (a->n > 0 && (!d_b || !d_x || !d_r)) return fail(LGX_ERR_INVALID, "null argument");
  if (a->n == 0) return LGX_OK;
  const Csr &c = a->csr;
  k_residual_dot2<<<std::min<unsigned>(grid_for(c.n, 256), 16384), 256, 0, stream>>>(
    c.n, c.rowptr.p, c.col.p, c.v64.p, d_b, d_x, d_r);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

lgx_status lgx_diffusion7_grad(const int64_t dims[3], const double *d_k, const double *d_lambda,
                               const double *d_x, double *d_grad, lgx_stream stream) {
  if (!dims || dims[0] < 0 || dims[1] < 0 || dims[2] < 0)
    return fail(LGX_ERR_INVALID, "invalid grid dimensions");
  const int64_t n = dims[0] * dims[1] * dims[2];
  if (n == 0) return LGX_OK;
  if (!d_k || !d_lambda || !d_x || !d_grad) return fail(LGX_ERR_INVALID, "null argument");
  k_diffusion7_grad<<<std::min<unsigned>(grid_for(n, 256), 16384), 256, 0, stream>>>(
    dims[0], dims[1], dims[2], d_k, d_lambda, d_x, d_grad);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

}  // extern "C"
