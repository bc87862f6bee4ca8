// Stationary smoothers: Jacobi (jacobi/sweep.hpp:66-87) and multicolour SOR,
// the GB300 replacement of the thread-block-hybrid SOR of
// gauss-seidel-variant/sweep.hpp:134-200, plus graph colouring.
//
// A multicolour sweep works on a colour-permuted copy of the matrix: colour c
// occupies the contiguous rows [offsets[c], offsets[c+1]), so every colour
// pass is a coalesced row-block kernel.  Rows keep their original column
// order, hence each row sum is formed in exactly the order of the
// reference's scalar CSR path; the sweep equals the reference SOR run in the
// order "rows sorted by (colour, index)".
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <cmath>
#include <vector>

#include "lgx_internal.cuh"
#include "lgx_rows.cuh"

namespace lgx {

// ---- Jacobi ----------------------------------------------------------------
template <typename VT>
struct JacobiOp {
  const double *x_in;  // nullptr: zero input vector
  double *x_out;
  const double *b;
  double relax, m1;
  using X = double;
  static constexpr bool kReduce = false;
  double *partials = nullptr;
  unsigned *counter = nullptr;
  template <int W>
  __device__ __forceinline__ double row(int64_t i, const int32_t *c, const VT *v, int len) const {
    double accum = b[i], diag = 0.0;
    for (int k = 0; k < len; ++k) {
      const int32_t j = c[k];
      const double a = (double)v[k];
      if (j == i) {
        diag = a;
      } else {
        accum = fma(-a, x_in ? __ldg(x_in + j) : 0.0, accum);
      }
    }
    const double quot = accum / diag;
    x_out[i] = fma(relax, quot, m1 * (x_in ? x_in[i] : 0.0));
    return 0.0;
  }
  __device__ __forceinline__ void finish(double) const {}
};

// Jacobi from a zero start with a cached diagonal (stencil matrices):
// x = fma(relax, b / d, m1 * 0) -- the reference's arithmetic with x_in = 0.
__global__ void k_jacobi_diag_zero(int64_t n, const double *__restrict__ d, double relax,
                                   const double *__restrict__ b, double *__restrict__ x) {
  const double m1 = 1.0 - relax;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = fma(relax, b[i] / d[i], m1 * 0.0);
}

// Stencil Jacobi with a general input: accum = b - sum_{j != i} a_ij x_j via
// y = A x (off-diagonal part: A x - d x would reorder the sum), so it is
// computed from the assembled rows; used through the CSR path instead.

// ---- graph colouring -----------------------------------------------------
__device__ __forceinline__ uint64_t splitmix(uint64_t seed, uint64_t i) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + i + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// One Jones-Plassmann round (see the oracle's lo_colour_jp): a vertex that
// beats all uncoloured neighbours on (priority, index) takes the smallest
// colour unused by coloured neighbours.  Colours of this round go to `next`.
__global__ void k_jp_round(int64_t n, const int64_t *__restrict__ rowptr,
                           const int32_t *__restrict__ col, uint64_t seed,
                           const int32_t *__restrict__ colour, int32_t *__restrict__ next) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    next[i] = -1;
    if (colour[i] >= 0) continue;
    const uint64_t pi = splitmix(seed, (uint64_t)i);
    bool is_max = true;
    uint64_t used = 0;
    const int64_t b = rowptr[i], e = rowptr[i + 1];
    for (int64_t k = b; k < e; ++k) {
      const int64_t j = col[k];
      if (j == i) continue;
      const int32_t cj = colour[j];
      if (cj < 0) {
        const uint64_t pj = splitmix(seed, (uint64_t)j);
        if (pj > pi || (pj == pi && j > i)) {
          is_max = false;
          break;
        }
      } else if (cj < 64) {
        used |= 1ull << cj;
      }
    }
    if (!is_max) continue;
    int32_t c = 0;
    for (;;) {
      bool taken;
      if (c < 64) {
        taken = (used >> c) & 1ull;
      } else {
        taken = false;
        for (int64_t k = b; k < e; ++k)
          if (col[k] != i && colour[col[k]] == c) taken = true;
      }
      if (!taken) break;
      ++c;
    }
    next[i] = c;
  }
}

__global__ void k_jp_commit(int64_t n, int32_t *colour, const int32_t *next,
                            unsigned long long *remaining, int *maxc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (next[i] >= 0) {
      colour[i] = next[i];
      atomicMax(maxc, next[i]);
    }
    if (colour[i] < 0) atomicAdd(remaining, 1ull);
  }
}

lgx_status colouring_jp(const Csr &a, uint64_t seed, cudaStream_t s, DBuf<int32_t> &colour,
                        int32_t &ncolours) {
  const int64_t n = a.n;
  LGX_CHECK(colour.alloc(n));
  DBuf<int32_t> next;
  DBuf<unsigned long long> rem;
  DBuf<int> maxc;
  LGX_CHECK(next.alloc(n));
  LGX_CHECK(rem.alloc(1));
  LGX_CHECK(maxc.alloc(1));
  LGX_CUDA(cudaMemsetAsync(colour.p, 0xFF, sizeof(int32_t) * std::max<int64_t>(n, 1), s));
  LGX_CUDA(cudaMemsetAsync(maxc.p, 0xFF, sizeof(int), s));
  const unsigned g = (unsigned)std::min<int64_t>(grid_for(n, 256), 16384);
  unsigned long long h_rem = (unsigned long long)n;
  int64_t rounds = 0;
  while (h_rem > 0) {
    if (++rounds > n + 1) return fail(LGX_ERR_INVALID, "colouring did not terminate");
    k_jp_round<<<g, 256, 0, s>>>(n, a.rowptr.p, a.col.p, seed, colour.p, next.p);
    LGX_LAUNCH_CHECK();
    LGX_CUDA(cudaMemsetAsync(rem.p, 0, sizeof(unsigned long long), s));
    k_jp_commit<<<g, 256, 0, s>>>(n, colour.p, next.p, rem.p, maxc.p);
    LGX_LAUNCH_CHECK();
    LGX_CUDA(cudaMemcpyAsync(&h_rem, rem.p, sizeof(h_rem), cudaMemcpyDeviceToHost, s));
    LGX_CUDA(cudaStreamSynchronize(s));
  }
  int h_max = -1;
  LGX_CUDA(cudaMemcpyAsync(&h_max, maxc.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  ncolours = h_max + 1;
  return LGX_OK;
}

__global__ void k_colour_flag(int64_t n, const int32_t *colour, int32_t c, int64_t *flag,
                              int *bad, int32_t ncolours) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t ci = colour[i];
    if (c == 0 && (ci < 0 || ci >= ncolours)) atomicOr(bad, 1);
    flag[i] = ci == c;
  }
}

__global__ void k_colour_place(int64_t n, const int32_t *colour, int32_t c, const int64_t *pos,
                               int64_t base, int32_t *perm, int32_t *iperm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (colour[i] != c) continue;
    const int64_t p = base + pos[i];
    perm[p] = (int32_t)i;
    iperm[i] = (int32_t)p;
  }
}

// adjacent rows must not share a colour
__global__ void k_colour_validate(int64_t n, const int64_t *rowptr, const int32_t *col,
                                  const int32_t *colour, int *bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (col[k] != i && colour[col[k]] == colour[i]) atomicOr(bad, 2);
}

__global__ void k_perm_rowlen(int64_t n, const int64_t *rowptr, const int32_t *perm,
                              int64_t *len) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm[r];
    len[r] = rowptr[i + 1] - rowptr[i];
  }
}

// one warp per permuted row: the row's entries copy coalesced (a thread
// per row walked 32 scattered rows per warp instruction: 216 GB/s at 256^3)
template <typename VT>
__global__ void k_perm_fill(int64_t n, const int64_t *rowptr, const int32_t *col, const VT *val,
                            const int32_t *perm, const int32_t *iperm, const int64_t *prowptr,
                            int32_t *pcol, VT *pval) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < n; r += nw) {
    const int64_t i = perm[r];
    const int64_t b = rowptr[i], len = rowptr[i + 1] - b, o = prowptr[r];
    for (int64_t k = lane; k < len; k += 32) {
      pcol[o + k] = iperm[col[b + k]];
      pval[o + k] = val[b + k];
    }
  }
}

// Reciprocal of every permuted row's diagonal, rounded once by the IEEE
// division; 0 marks rows whose diagonal lies outside [2^-400, 2^400] in
// magnitude (or is not finite), where the sweep divides directly.
template <typename VT>
__global__ void k_colour_rdiag(int64_t n, const int64_t *rowptr, const int32_t *col,
                               const VT *val, double *rdiag, double *pdiag) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
      if (col[k] == r) d = (double)val[k];
    pdiag[r] = d;
    if (rdiag) {
      const int e = (int)((__double_as_longlong(d) >> 52) & 0x7ff);
      rdiag[r] = (e > 1023 - 400 && e < 1023 + 400) ? 1.0 / d : 0.0;
    }
  }
}

__global__ void k_to_f32(int64_t n, const double *src, float *dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

lgx_status colouring_build(const Csr &a, const int32_t *d_colour, int32_t ncolours,
                           cudaStream_t s, lgx_colouring &out) {
  const int64_t n = a.n;
  if (ncolours < 1 && n > 0) return fail(LGX_ERR_INVALID, "colouring needs at least one colour");
  out.n = n;
  out.ncolours = ncolours;
  if (out.colour.p != d_colour) {
    LGX_CHECK(out.colour.alloc(n));
    LGX_CUDA(cudaMemcpyAsync(out.colour.p, d_colour, sizeof(int32_t) * n,
                             cudaMemcpyDeviceToDevice, s));
  }
  LGX_CHECK(out.perm.alloc(n));
  LGX_CHECK(out.iperm.alloc(n));
  DBuf<int64_t> flag, pos;
  DBuf<int> bad;
  LGX_CHECK(flag.alloc(n));
  LGX_CHECK(pos.alloc(n + 1));
  LGX_CHECK(bad.alloc(1));
  LGX_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  const unsigned g = (unsigned)std::min<int64_t>(grid_for(n, 256), 16384);
  out.offsets.assign((size_t)ncolours + 1, 0);
  int64_t base = 0;
  for (int32_t c = 0; c < ncolours; ++c) {
    k_colour_flag<<<g, 256, 0, s>>>(n, out.colour.p, c, flag.p, bad.p, ncolours);
    LGX_LAUNCH_CHECK();
    LGX_CHECK(inclusive_offsets(n, flag.p, pos.p, s));
    k_colour_place<<<g, 256, 0, s>>>(n, out.colour.p, c, pos.p, base, out.perm.p, out.iperm.p);
    LGX_LAUNCH_CHECK();
    int64_t cnt = 0;
    LGX_CUDA(cudaMemcpyAsync(&cnt, pos.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    LGX_CUDA(cudaStreamSynchronize(s));
    out.offsets[c] = base;
    base += cnt;
  }
  out.offsets[ncolours] = base;
  k_colour_validate<<<g, 256, 0, s>>>(n, a.rowptr.p, a.col.p, out.colour.p, bad.p);
  LGX_LAUNCH_CHECK();
  int h_bad = 0;
  LGX_CUDA(cudaMemcpyAsync(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  if (h_bad & 1) return fail(LGX_ERR_INVALID, "colour index out of range");
  if (h_bad & 2) return fail(LGX_ERR_INVALID, "adjacent rows share a colour");
  if (base != n) return fail(LGX_ERR_INVALID, "colouring does not cover every row");
  // permuted CSR
  Csr &p = out.pcsr;
  p.n = n;
  p.nnz = a.nnz;
  p.symmetric = a.symmetric;
  p.storage = a.storage;
  p.max_row = a.max_row;
  LGX_CHECK(p.rowptr.alloc(n + 3));  // +2: staged row-offset spans
  LGX_CHECK(csr_alloc_arrays(p, a.nnz, a.storage));
  k_perm_rowlen<<<g, 256, 0, s>>>(n, a.rowptr.p, out.perm.p, flag.p);
  LGX_LAUNCH_CHECK();
  LGX_CHECK(inclusive_offsets(n, flag.p, p.rowptr.p, s));
  if (a.storage == LGX_F64) {
    k_perm_fill<double><<<g, 256, 0, s>>>(n, a.rowptr.p, a.col.p, a.v64.p, out.perm.p,
                                          out.iperm.p, p.rowptr.p, p.col.p, p.v64.p);
  } else {
    k_perm_fill<float><<<g, 256, 0, s>>>(n, a.rowptr.p, a.col.p, a.v32.p, out.perm.p, out.iperm.p,
                                         p.rowptr.p, p.col.p, p.v32.p);
  }
  LGX_LAUNCH_CHECK();
  if (n > 0) {
    LGX_CHECK(out.pdiag.alloc(n));
    if (a.storage == LGX_F64) {
      LGX_CHECK(out.rdiag.alloc(n));
      k_colour_rdiag<double><<<g, 256, 0, s>>>(n, p.rowptr.p, p.col.p, p.v64.p, out.rdiag.p,
                                               out.pdiag.p);
    } else {
      k_colour_rdiag<float><<<g, 256, 0, s>>>(n, p.rowptr.p, p.col.p, p.v32.p, nullptr,
                                              out.pdiag.p);
    }
    LGX_LAUNCH_CHECK();
  }
  return csr_compute_max_window(p, s);
}

lgx_status colouring_make_f32(lgx_colouring &c, cudaStream_t s) {
  if (c.pcsr.storage == LGX_F32 || c.pv32.p) return LGX_OK;
  LGX_CHECK(c.pv32.alloc(c.pcsr.nnz + kCsrPad));
  k_to_f32<<<std::min<int64_t>(grid_for(c.pcsr.nnz, 256), 16384), 256, 0, s>>>(
    c.pcsr.nnz, c.pcsr.v64.p, c.pv32.p);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

// bfloat16 copy of the permuted values scaled by the row's diagonal:
// pv16 = bf16(a_ij / a_ii) (the diagonal becomes exactly 1), pscale = a_ii.
// Rows without a nonzero diagonal keep scale 1 and bf16(a_ij).
template <typename VT>
__global__ void k_to_bf16_scaled(int64_t n, const int64_t *rowptr, const int32_t *col,
                                 const VT *val, bf16 *out, float *scale) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
      if (col[k] == r) d = (double)val[k];
    const bool use = d != 0.0 && isfinite(d);
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
      out[k] = __float2bfloat16_rn((float)(use ? (double)val[k] / d : (double)val[k]));
    scale[r] = use ? (float)d : 1.0f;
  }
}

lgx_status colouring_make_bf16(lgx_colouring &c, cudaStream_t s) {
  if (c.pv16.p) return LGX_OK;
  const Csr &p = c.pcsr;
  LGX_CHECK(c.pv16.alloc(p.nnz + kCsrPad));
  LGX_CHECK(c.pscale.alloc(std::max<int64_t>(p.n, 1)));
  if (p.n == 0) return LGX_OK;
  const unsigned g = (unsigned)std::min<int64_t>(grid_for(p.n, 256), 16384);
  if (p.storage == LGX_F64)
    k_to_bf16_scaled<double><<<g, 256, 0, s>>>(p.n, p.rowptr.p, p.col.p, p.v64.p, c.pv16.p,
                                               c.pscale.p);
  else
    k_to_bf16_scaled<float><<<g, 256, 0, s>>>(p.n, p.rowptr.p, p.col.p, p.v32.p, c.pv16.p,
                                              c.pscale.p);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

// ---- multicolour SOR -------------------------------------------------------
// One row of gauss-seidel-variant/sweep.hpp:134-200 in place: rows of other
// colours already visited in this sweep hold their new values in x, the rest
// their input values; rows of the same colour are never adjacent.
// With rdiag (FP64 values and vectors) the regular row divides through the
// reciprocal table (same quotient), and relax == 1 skips the (1 - relax) x_i
// term where it cannot change the result (q nonzero, x_i finite).
template <typename VT, typename XT>
struct SorOp {
  const XT *b;
  XT *x;
  XT relax, m1;
  int ultra;
  const double *rdiag = nullptr;
  int relax_one = 0;
  // forward sweep from x = 0 without clearing x first: rows of colours not
  // yet visited in this sweep (index >= visit_end) read as 0, this row too
  int from_zero = 0;
  int64_t visit_end = 0;
  const float *scale = nullptr;  // bfloat16 values: row factor (the diagonal)
  using X = XT;
  static constexpr bool kReduce = false;
  static constexpr int kTuneClass = 1;
  double *partials = nullptr;
  unsigned *counter = nullptr;
  template <int W>
  __device__ __forceinline__ double row(int64_t i, const int32_t *c, const VT *v, int len) const {
    if constexpr (kIsBf16<VT>) {
      return row_scaled<W>(i, c, v, len);
    }
    XT accum = b[i], diag = XT(0);
    const XT xi = from_zero ? XT(0) : x[i];
    for (int k = 0; k < len; k += W) {
      const int m = len - k < W ? len - k : W;
      XT xv[W];
#pragma unroll
      for (int u = 0; u < W; ++u)
        if (u < m) xv[u] = (from_zero && c[k + u] >= visit_end) ? XT(0) : x[c[k + u]];
#pragma unroll
      for (int u = 0; u < W; ++u) {
        if (u < m) {
          const XT a = cvt<XT>(v[k + u]);
          if (c[k + u] == i) {
            diag = a;
            if (ultra) accum = fma(-a, xi, accum);
          } else {
            accum = fma(-a, xv[u], accum);
          }
        }
      }
    }
    if (ultra) {
      x[i] = xi + relax * accum / fabs(diag);
      return 0.0;
    }
    XT quot;
    if constexpr (sizeof(XT) == 8) {
      const double y = rdiag ? rdiag[i] : 0.0;
      quot = (nonzero_bits(y) && exponent_within_400(accum)) ? div_by_recip(accum, diag, y)
                                                             : accum / diag;
      if (relax_one && nonzero_bits(quot) && exponent_field(xi) != 0x7ff) {
        x[i] = quot;  // fma(1, q, 0 * x_i) == q for nonzero q and finite x_i
        return 0.0;
      }
    } else {
      quot = accum / diag;
    }
    x[i] = fma(relax, quot, m1 * xi);
    return 0.0;
  }
  // bfloat16 values v with a_ij = s_i v_ij: accum = b_i - s_i sum_{j != i} v_ij x_j,
  // a_ii = s_i v_ii (float arithmetic; a precision-form smoother, not the
  // reference's bits)
  template <int W>
  __device__ __forceinline__ double row_scaled(int64_t i, const int32_t *c, const VT *v,
                                               int len) const {
    const XT si = scale[i];
    const XT xi = from_zero ? XT(0) : x[i];
    XT t = XT(0), vd = XT(0);
    for (int k = 0; k < len; k += W) {
      const int m = len - k < W ? len - k : W;
      XT xv[W];
#pragma unroll
      for (int u = 0; u < W; ++u)
        if (u < m) xv[u] = (from_zero && c[k + u] >= visit_end) ? XT(0) : x[c[k + u]];
#pragma unroll
      for (int u = 0; u < W; ++u) {
        if (u < m) {
          const XT a = cvt<XT>(v[k + u]);
          if (c[k + u] == i) {
            vd = a;
          } else {
            t = fma(a, xv[u], t);
          }
        }
      }
    }
    const XT diag = si * vd;
    XT accum = fma(-si, t, b[i]);
    if (ultra) {
      accum = fma(-diag, xi, accum);
      x[i] = xi + relax * accum / fabs(diag);
    } else {
      x[i] = fma(relax, accum / diag, m1 * xi);
    }
    return 0.0;
  }
  __device__ __forceinline__ void finish(double) const {}
};

// First colour of a forward sweep from x = 0: every neighbour still reads 0,
// so the row's products with them leave accum = b_i (an fma with a zero
// product; where only the sign of a zero could differ, the row's result is
// +0 either way) and the row needs only b_i and its diagonal: 32 bytes per
// row instead of the whole row.  Same quotient and update as SorOp.
template <typename VT, typename XT>
__global__ void k_sor_first_colour(int64_t rb, int64_t re, const double *__restrict__ pdiag,
                                   const double *__restrict__ rdiag,
                                   const float *__restrict__ scale, const XT *__restrict__ b,
                                   XT *__restrict__ x, XT relax, XT m1, int ultra,
                                   int relax_one) {
  pdl_trigger();
  pdl_wait();
  for (int64_t i = rb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < re;
       i += (int64_t)gridDim.x * blockDim.x) {
    const XT accum = b[i];
    XT diag;
    if constexpr (kIsBf16<VT>) {
      diag = scale[i];  // s_i * v_ii with v_ii = 1 (scaled by the diagonal)
    } else {
      diag = (XT)pdiag[i];
    }
    const XT xi = XT(0);
    if (ultra) {
      x[i] = xi + relax * accum / fabs(diag);
      continue;
    }
    XT quot;
    if constexpr (sizeof(XT) == 8 && !kIsBf16<VT>) {
      const double y = rdiag ? rdiag[i] : 0.0;
      quot = (nonzero_bits(y) && exponent_within_400(accum)) ? div_by_recip(accum, diag, y)
                                                             : accum / diag;
      if (relax_one && nonzero_bits(quot)) {
        x[i] = quot;
        continue;
      }
    } else {
      quot = accum / diag;
    }
    x[i] = fma(relax, quot, m1 * xi);
  }
}

template <typename VT, typename XT>
lgx_status mc_sor_sweep(const lgx_colouring &c, const VT *val, double relax, int forward,
                        int ultra, const XT *b, XT *x, cudaStream_t s, int from_zero,
                        const float *scale, XT *r_last, int64_t *res_from) {
  if (res_from) *res_from = c.n;
  const Csr &p = c.pcsr;
  SorOp<VT, XT> op{b, x, (XT)relax, XT(1) - (XT)relax, ultra};
  op.scale = scale;
  if (kIsBf16<VT> && !scale) return fail(LGX_ERR_INVALID, "bfloat16 values need row scales");
  if constexpr (sizeof(VT) == 8 && sizeof(XT) == 8) {
    op.rdiag = c.rdiag.p;
    op.relax_one = relax == 1.0;
  }
  op.from_zero = from_zero && forward;
  if (from_zero && !forward && c.n > 0)
    LGX_CUDA(cudaMemsetAsync(x, 0, sizeof(XT) * c.n, s));
  for (int32_t k = 0; k < c.ncolours; ++k) {
    const int32_t col_id = forward ? k : c.ncolours - 1 - k;
    const int64_t rb = c.offsets[col_id], re = c.offsets[col_id + 1];
    if (op.from_zero && k == 0 && c.pdiag.p) {
      if (re > rb) {
        const unsigned g = (unsigned)std::min<int64_t>(grid_for(re - rb, 256), 16384);
        LGX_CUDA(launch_pdl(sizeof(XT) == 4 || re - rb <= pdl_fp64_rows(),
                            k_sor_first_colour<VT, XT>, dim3(g), dim3(256), 0,
                            s, rb, re, (const double *)c.pdiag.p, (const double *)op.rdiag,
                            scale, b, x, op.relax, op.m1, ultra, op.relax_one));
        count_launch();
      }
      continue;
    }
    op.visit_end = rb;  // forward: exactly the rows before this colour are visited
    // the last colour of a forward sweep on grid rows can also leave its
    // rows' residuals in r_last
    const bool with_res = r_last && res_from && forward && k == c.ncolours - 1 && re > rb &&
                          !kIsBf16<VT> && sizeof(XT) == 4 && grid_sweep_residual(p);
    bool done = false;
    LGX_CHECK((grid_sor_rows<VT, XT>(p, val, rb, re, b, x, relax, ultra, op.rdiag, op.relax_one,
                                     op.from_zero, op.visit_end, scale, s, &done,
                                     with_res ? r_last : nullptr)));
    if (done) {
      if (with_res) *res_from = rb;
      continue;
    }
    LGX_CHECK(launch_rows<VT>(rb, re, p, val, op, s));
  }
  return LGX_OK;
}

template lgx_status mc_sor_sweep<double, double>(const lgx_colouring &, const double *, double,
                                                 int, int, const double *, double *,
                                                 cudaStream_t, int, const float *, double *,
                                                 int64_t *);
template lgx_status mc_sor_sweep<float, double>(const lgx_colouring &, const float *, double, int,
                                                int, const double *, double *, cudaStream_t, int,
                                                const float *, double *, int64_t *);
template lgx_status mc_sor_sweep<float, float>(const lgx_colouring &, const float *, double, int,
                                               int, const float *, float *, cudaStream_t, int,
                                               const float *, float *, int64_t *);
template lgx_status mc_sor_sweep<bf16, float>(const lgx_colouring &, const bf16 *, double, int,
                                              int, const float *, float *, cudaStream_t, int,
                                              const float *, float *, int64_t *);

lgx_status jacobi_csr(const Csr &a, double relax, const double *x_in, double *x_out,
                      const double *b, cudaStream_t s) {
  if (a.n == 0) return LGX_OK;
  if (a.storage == LGX_F64)
    return launch_rows<double>(0, a.n, a, a.v64.p,
                               JacobiOp<double>{x_in, x_out, b, relax, 1.0 - relax}, s);
  return launch_rows<float>(0, a.n, a, a.v32.p,
                            JacobiOp<float>{x_in, x_out, b, relax, 1.0 - relax}, s);
}

lgx_status jacobi_diag_zero(int64_t n, const double *d, double relax, const double *b, double *x,
                            cudaStream_t s) {
  if (n == 0) return LGX_OK;
  k_jacobi_diag_zero<<<std::min<int64_t>(grid_for(n, 256), 16384), 256, 0, s>>>(n, d, relax, b,
                                                                                 x);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

// Public sweep on natural-order vectors: gather into the permuted order,
// sweep in place, scatter back.
lgx_status colouring_sweep_natural(lgx_colouring &c, double relax, int forward, int ultra,
                                   const double *x_in, double *x_out, const double *b,
                                   cudaStream_t s) {
  const int64_t n = c.n;
  if (!c.work_b.p) {
    LGX_CHECK(c.work_b.alloc(n));
    LGX_CHECK(c.work_x.alloc(n));
  }
  LGX_CHECK(gather<double, double>(n, c.perm.p, b, c.work_b.p, s));
  if (x_in) LGX_CHECK(gather<double, double>(n, c.perm.p, x_in, c.work_x.p, s));
  const int from_zero = x_in == nullptr;
  if (c.pcsr.storage == LGX_F64) {
    LGX_CHECK(mc_sor_sweep<double, double>(c, c.pcsr.v64.p, relax, forward, ultra, c.work_b.p,
                                           c.work_x.p, s, from_zero));
  } else {
    LGX_CHECK(mc_sor_sweep<float, double>(c, c.pcsr.v32.p, relax, forward, ultra, c.work_b.p,
                                          c.work_x.p, s, from_zero));
  }
  return scatter<double, double>(n, c.perm.p, c.work_x.p, x_out, s);
}

}  // namespace lgx

using namespace lgx;

extern "C" {

lgx_status lgx_jacobi_sweep(const lgx_matrix *a, double relax, const double *d_x_in,
                            double *d_x_out, const double *d_b, lgx_stream stream) {
  if (!a || (a->n > 0 && (!d_x_out || !d_b))) return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind == LGX_MATRIX_CSR) return jacobi_csr(a->csr, relax, d_x_in, d_x_out, d_b, stream);
  if (d_x_in) return fail(LGX_ERR_UNSUPPORTED,
                          "stencil Jacobi sweeps start from zero; assemble the matrix for a "
                          "general input vector");
  const double *d = nullptr;
  LGX_CHECK(matrix_diagonal(const_cast<lgx_matrix *>(a), stream, &d));
  return jacobi_diag_zero(a->n, d, relax, d_b, d_x_out, stream);
}

lgx_status lgx_colouring_create_jp(const lgx_matrix *a, uint64_t seed, lgx_stream stream,
                                   lgx_colouring **out) {
  if (!a || !out) return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind != LGX_MATRIX_CSR) return fail(LGX_ERR_UNSUPPORTED, "colouring needs a CSR matrix");
  auto *c = new lgx_colouring();
  int32_t nc = 0;
  lgx_status st = colouring_jp(a->csr, seed, stream, c->colour, nc);
  if (st == LGX_OK) st = colouring_build(a->csr, c->colour.p, nc, stream, *c);
  if (st != LGX_OK) {
    delete c;
    return st;
  }
  *out = c;
  return LGX_OK;
}

// Smallest-last greedy colouring on the host.  Ordering: vertices sit in
// buckets by their degree among the vertices not yet removed (off-diagonal
// pattern entries), each bucket a list with the most recently inserted vertex
// at its head; the initial insertion runs in index order; each step removes
// the head of the lowest non-empty bucket and moves each remaining neighbour
// (in CSR order) to the head of the bucket below.  Colouring: in the reverse
// of the removal order, each vertex takes the smallest colour none of its
// coloured neighbours has.  O(nnz); every step is fixed, so the colouring is
// deterministic.
// The pattern's adjacency as the colouring sees it: the rows themselves when
// the off-diagonal pattern is structurally symmetric, else every row's sorted
// union with the matching column of the transpose (the pattern of A + A^T),
// so that a colouring is proper for both directions of every edge.  Returns
// false when the rows are used as given.
static bool symmetrised_pattern(int64_t n, const int64_t *rowptr, const int32_t *col,
                                std::vector<int64_t> &sptr, std::vector<int32_t> &scol) {
  std::vector<int64_t> tptr((size_t)n + 1, 0);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e)
      if (col[e] != i) ++tptr[(size_t)col[e] + 1];
  for (int64_t i = 0; i < n; ++i) tptr[(size_t)i + 1] += tptr[(size_t)i];
  std::vector<int32_t> tcol((size_t)tptr[(size_t)n]);
  std::vector<int64_t> fill(tptr.begin(), tptr.end() - 1);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e)
      if (col[e] != i) tcol[(size_t)fill[(size_t)col[e]]++] = (int32_t)i;
  bool symmetric = true;
  std::vector<int32_t> row;
  for (int64_t i = 0; i < n && symmetric; ++i) {
    row.clear();
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e)
      if (col[e] != i) row.push_back(col[e]);
    std::sort(row.begin(), row.end());
    symmetric = std::equal(row.begin(), row.end(), tcol.begin() + tptr[(size_t)i],
                           tcol.begin() + tptr[(size_t)i + 1]) &&
                (int64_t)row.size() == tptr[(size_t)i + 1] - tptr[(size_t)i];
  }
  if (symmetric) return false;
  sptr.assign((size_t)n + 1, 0);
  scol.clear();
  for (int64_t i = 0; i < n; ++i) {
    row.clear();
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e)
      if (col[e] != i) row.push_back(col[e]);
    row.insert(row.end(), tcol.begin() + tptr[(size_t)i], tcol.begin() + tptr[(size_t)i + 1]);
    std::sort(row.begin(), row.end());
    row.erase(std::unique(row.begin(), row.end()), row.end());
    scol.insert(scol.end(), row.begin(), row.end());
    sptr[(size_t)i + 1] = (int64_t)scol.size();
  }
  return true;
}

}  // extern "C"

namespace lgx {
lgx_status colour_smallest_last(int64_t n, const int64_t *rowptr, const int32_t *col,
                                int32_t *colour, int32_t *ncolours, bool known_symmetric);
}  // namespace lgx

extern "C" lgx_status lgx_colour_smallest_last(int64_t n, const int64_t *rowptr,
                                               const int32_t *col, int32_t *colour,
                                               int32_t *ncolours) {
  return lgx::colour_smallest_last(n, rowptr, col, colour, ncolours, false);
}

// known_symmetric: the caller's matrix is symmetric (the AMG levels of a
// symmetric matrix), so its pattern needs no symmetrisation check
lgx_status lgx::colour_smallest_last(int64_t n, const int64_t *rowptr, const int32_t *col,
                                     int32_t *colour, int32_t *ncolours, bool known_symmetric) {
  if (n < 0 || n > INT32_MAX || (n > 0 && (!rowptr || !col || !colour)) || !ncolours)
    return fail(LGX_ERR_INVALID, "bad argument");
  *ncolours = 0;
  if (n == 0) return LGX_OK;
  if (rowptr[0] != 0) return fail(LGX_ERR_INVALID, "row offsets must start at 0");
  for (int64_t i = 0; i < n; ++i)
    if (rowptr[i + 1] < rowptr[i]) return fail(LGX_ERR_INVALID, "decreasing row offsets");
  for (int64_t e = 0; e < rowptr[n]; ++e)
    if (col[e] < 0 || col[e] >= n) return fail(LGX_ERR_INVALID, "column index out of range");
  std::vector<int64_t> sptr;
  std::vector<int32_t> scol;
  if (!known_symmetric && symmetrised_pattern(n, rowptr, col, sptr, scol)) {
    rowptr = sptr.data();
    col = scol.data();
  }
  std::vector<int64_t> deg((size_t)n), next((size_t)n, -1), prev((size_t)n, -1);
  int64_t maxdeg = 0;
  for (int64_t i = 0; i < n; ++i) {
    int64_t d = 0;
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e) d += col[e] != i;
    deg[(size_t)i] = d;
    maxdeg = std::max(maxdeg, d);
  }
  std::vector<int64_t> head((size_t)maxdeg + 1, -1);
  auto unlink = [&](int64_t v) {
    const int64_t p = prev[(size_t)v], q = next[(size_t)v];
    if (p >= 0) next[(size_t)p] = q; else head[(size_t)deg[(size_t)v]] = q;
    if (q >= 0) prev[(size_t)q] = p;
  };
  auto push = [&](int64_t v) {
    const int64_t h = head[(size_t)deg[(size_t)v]];
    prev[(size_t)v] = -1;
    next[(size_t)v] = h;
    if (h >= 0) prev[(size_t)h] = v;
    head[(size_t)deg[(size_t)v]] = v;
  };
  for (int64_t i = 0; i < n; ++i) push(i);
  std::vector<uint8_t> removed((size_t)n, 0);
  std::vector<int32_t> order;
  order.reserve((size_t)n);
  int64_t low = 0;
  for (int64_t step = 0; step < n; ++step) {
    while (head[(size_t)low] < 0) ++low;
    const int64_t v = head[(size_t)low];
    unlink(v);
    removed[(size_t)v] = 1;
    order.push_back((int32_t)v);
    for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e) {
      const int64_t u = col[e];
      if (u == v || removed[(size_t)u]) continue;
      unlink(u);
      --deg[(size_t)u];
      push(u);
    }
    if (low > 0) --low;  // a neighbour may now sit one bucket lower
  }
  std::vector<int64_t> stamp((size_t)maxdeg + 2, -1);
  for (int64_t i = 0; i < n; ++i) colour[i] = -1;
  int32_t used = 0;
  for (int64_t k = n - 1; k >= 0; --k) {
    const int64_t v = order[(size_t)k];
    for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e) {
      const int32_t c = colour[col[e]];
      if (col[e] != v && c >= 0 && c <= maxdeg) stamp[(size_t)c] = v;
    }
    int32_t c = 0;
    while (stamp[(size_t)c] == v) ++c;
    colour[v] = c;
    used = std::max(used, c + 1);
  }
  *ncolours = used;
  return LGX_OK;
}

extern "C" {

lgx_status lgx_colouring_create(const lgx_matrix *a, const int32_t *d_colour, int32_t ncolours,
                                lgx_stream stream, lgx_colouring **out) {
  if (!a || !out || (a->n > 0 && !d_colour)) return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind != LGX_MATRIX_CSR) return fail(LGX_ERR_UNSUPPORTED, "colouring needs a CSR matrix");
  auto *c = new lgx_colouring();
  lgx_status st = colouring_build(a->csr, d_colour, ncolours, stream, *c);
  if (st != LGX_OK) {
    delete c;
    return st;
  }
  *out = c;
  return LGX_OK;
}

lgx_status lgx_colouring_grid27(lgx_colouring *c, const int64_t dims[3], int with_float,
                                lgx_stream stream, int *attached) {
  if (!c || !dims) return fail(LGX_ERR_INVALID, "null argument");
  if (c->stencil_rb) {
    if (attached) *attached = 0;
    return LGX_OK;
  }
  if (with_float && c->pcsr.storage == LGX_F64) LGX_CHECK(colouring_make_f32(*c, stream));
  bool att = false;
  LGX_CHECK(grid27_attach(*c, dims, 27, stream, &att));
  if (attached) *attached = att ? 1 : 0;
  return LGX_OK;
}

}  // extern "C"

namespace lgx {
// The failure path of the kernels' bounded waits, exercised on purpose: one
// thread initialises an mbarrier that expects one arrival, issues nothing,
// and waits on it with the same bounded wait the row engine uses (about
// one second of SM clock); the wait gives up, the kernel records it in the
// device error flag and returns.  No copy is ever in flight.
__global__ void k_wait_selftest(int *err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  fence_mbar_init();
  if (!mbar_wait_bounded(&bar, 0)) atomicOr(err, 1);
}

__global__ void k_red_black_colour(int64_t n, int64_t n1, int64_t n2, int32_t *colour) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    colour[i] = (int32_t)(((i / (n1 * n2)) + ((i / n2) % n1) + (i % n2)) & 1);
}
}  // namespace lgx

extern "C" {

lgx_status lgx_wait_selftest(lgx_stream stream) {
  int *err = device_error_flag();
  if (!err) return fail(LGX_ERR_NOMEM, "device error flag not allocated");
  k_wait_selftest<<<1, 32, 0, stream>>>(err);
  LGX_LAUNCH_CHECK();
  return check_device_error(stream);
}

lgx_status lgx_colouring_create_red_black(const lgx_matrix *a, lgx_stream stream,
                                          lgx_colouring **out) {
  if (!a || !out) return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind == LGX_MATRIX_CSR)
    return fail(LGX_ERR_UNSUPPORTED,
                "red-black colouring is for stencil matrices (CSR: lgx_colouring_create)");
  auto c = std::make_unique<lgx_colouring>();
  const int64_t n0 = a->st.dims[0], n1 = a->st.dims[1], n2 = a->st.dims[2];
  c->n = a->n;
  c->ncolours = 2;
  c->stencil_rb = true;
  LGX_CHECK(c->colour.alloc(a->n));
  if (a->n) {
    k_red_black_colour<<<std::min<int64_t>(grid_for(a->n, 256), 16384), 256, 0, stream>>>(
      a->n, n1, n2, c->colour.p);
    LGX_LAUNCH_CHECK();
  }
  // colour 0 holds the cells with even p0 + p1 + p2
  int64_t even = 0;
  for (int64_t p0 = 0; p0 < n0; ++p0)
    for (int64_t p1 = 0; p1 < n1; ++p1) even += (n2 + 1 - ((p0 + p1) & 1)) / 2;
  c->offsets = {0, even, a->n};
  LGX_CUDA(cudaStreamSynchronize(stream));
  *out = c.release();
  return LGX_OK;
}

lgx_status lgx_colouring_destroy(lgx_colouring *c) {
  delete c;
  return LGX_OK;
}

lgx_status lgx_colouring_export(const lgx_colouring *c, int32_t *d_colour, int32_t *ncolours,
                                lgx_stream stream) {
  if (!c) return fail(LGX_ERR_INVALID, "null colouring");
  if (d_colour && c->n)
    LGX_CUDA(cudaMemcpyAsync(d_colour, c->colour.p, sizeof(int32_t) * c->n,
                             cudaMemcpyDeviceToDevice, stream));
  if (ncolours) *ncolours = c->ncolours;
  LGX_CUDA(cudaStreamSynchronize(stream));
  return LGX_OK;
}

lgx_status lgx_sor_sweep(const lgx_matrix *a, const lgx_colouring *c, double relax, int forward,
                         int ultra, const double *d_x_in, double *d_x_out, const double *d_b,
                         lgx_stream stream) {
  if (!a || !c || (a->n > 0 && (!d_x_out || !d_b))) return fail(LGX_ERR_INVALID, "null argument");
  if (c->n != a->n) return fail(LGX_ERR_INVALID, "colouring does not match the matrix");
  if (c->stencil_rb != (a->kind != LGX_MATRIX_CSR))
    return fail(LGX_ERR_UNSUPPORTED, a->kind == LGX_MATRIX_CSR
                                       ? "a stencil's red-black colouring on a CSR matrix"
                                       : "a stencil matrix sweeps with its red-black colouring");
  if (c->stencil_rb)
    return stencil_sor_sweep(a, relax, forward, ultra, d_x_in, d_x_out, d_b, stream);
  return colouring_sweep_natural(*const_cast<lgx_colouring *>(c), relax, forward, ultra, d_x_in,
                                 d_x_out, d_b, stream);
}

lgx_status lgx_colouring_permute(const lgx_colouring *c, const double *d_src, double *d_dst,
                                 lgx_stream stream) {
  if (!c || (c->n > 0 && (!d_src || !d_dst))) return fail(LGX_ERR_INVALID, "null argument");
  if (c->stencil_rb)
    return fail(LGX_ERR_UNSUPPORTED, "a stencil colouring sweeps in natural order (lgx_sor_sweep)");
  return gather<double, double>(c->n, c->perm.p, d_src, d_dst, stream);
}

lgx_status lgx_colouring_unpermute(const lgx_colouring *c, const double *d_src, double *d_dst,
                                   lgx_stream stream) {
  if (!c || (c->n > 0 && (!d_src || !d_dst))) return fail(LGX_ERR_INVALID, "null argument");
  if (c->stencil_rb)
    return fail(LGX_ERR_UNSUPPORTED, "a stencil colouring sweeps in natural order (lgx_sor_sweep)");
  return scatter<double, double>(c->n, c->perm.p, d_src, d_dst, stream);
}

lgx_status lgx_sor_sweep_permuted(const lgx_colouring *c, double relax, int forward, int ultra,
                                  double *d_x, const double *d_b, lgx_stream stream) {
  if (!c || (c->n > 0 && (!d_x || !d_b))) return fail(LGX_ERR_INVALID, "null argument");
  if (c->stencil_rb)
    return fail(LGX_ERR_UNSUPPORTED, "a stencil colouring sweeps in natural order (lgx_sor_sweep)");
  if (c->pcsr.storage == LGX_F64)
    return mc_sor_sweep<double, double>(*c, c->pcsr.v64.p, relax, forward, ultra, d_b, d_x,
                                        stream);
  return mc_sor_sweep<float, double>(*c, c->pcsr.v32.p, relax, forward, ultra, d_b, d_x, stream);
}

lgx_status lgx_sor_sweep_permuted_f32(lgx_colouring *c, float relax, int forward, int ultra,
                                      float *d_x, const float *d_b, lgx_stream stream) {
  if (!c || (c->n > 0 && (!d_x || !d_b))) return fail(LGX_ERR_INVALID, "null argument");
  if (c->stencil_rb)
    return fail(LGX_ERR_UNSUPPORTED, "a stencil colouring sweeps in natural order (lgx_sor_sweep)");
  const float *v = c->pcsr.v32.p;
  if (c->pcsr.storage == LGX_F64) {
    LGX_CHECK(colouring_make_f32(*c, stream));
    v = c->pv32.p;
  }
  return mc_sor_sweep<float, float>(*c, v, relax, forward, ultra, d_b, d_x, stream);
}

}  // extern "C"
