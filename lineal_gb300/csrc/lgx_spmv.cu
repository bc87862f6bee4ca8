// Sparse matrix-vector products: CSR (row blocks staged through shared
// memory, one thread per row) and matrix-free 7-point diffusion stencils.
//
// GB300 note: FP64 runs at ~1.2 TFLOP/s on this part (58x below FP32), so
// every FP64 kernel is co-limited by the FP64 pipe.  The CSR kernels use one
// thread per row (27 FMAs for a 27-point row, no shuffle reductions whose
// FP64 adds would multiply the pipe load) and stage each block's contiguous
// CSR segment in shared memory so the global reads stay fully coalesced.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>

#include "lgx_internal.cuh"
#include "lgx_rows.cuh"

namespace lgx {

// ---------------------------------------------------------------------------
// CSR operations on the staged row engine (lgx_rows.cuh)
// ---------------------------------------------------------------------------
template <typename VT, typename XT>
struct SpmvOp {
  const XT *x;
  XT *y;
  using X = XT;
  static constexpr bool kReduce = false;
  double *partials = nullptr;
  unsigned *counter = nullptr;
  template <int W>
  __device__ __forceinline__ double row(int64_t i, const int32_t *c, const VT *v, int len) const {
    y[i] = row_dot<W, VT, XT>(c, v, len, x, XT(0));
    return 0.0;
  }
  __device__ __forceinline__ void finish(double) const {}
};

// r = b - A x, optionally ||r||^2 into *out (deterministic)
template <typename VT, typename XT, bool NORM>
struct ResidualOp {
  const XT *b, *x;
  XT *r;
  double *out;
  using X = XT;
  static constexpr bool kReduce = NORM;
  double *partials;
  unsigned *counter;
  const float *scale = nullptr;  // bfloat16 values: row factor
  template <int W>
  __device__ __forceinline__ double row(int64_t i, const int32_t *c, const VT *v, int len) const {
    XT ax = row_dot<W, VT, XT>(c, v, len, x, XT(0));
    if constexpr (kIsBf16<VT>) ax = ax * scale[i];
    const XT rv = b[i] - ax;
    r[i] = rv;
    return NORM ? (double)rv * (double)rv : 0.0;
  }
  __device__ __forceinline__ void finish(double t) const { *out = t; }
};

template <typename VT, typename XT>
lgx_status csr_spmv(const Csr &a, const VT *val, const XT *x, XT *y, cudaStream_t s) {
  if (a.n == 0) return LGX_OK;
  bool done = false;
  LGX_CHECK((grid_spmv<VT, XT>(a, val, x, y, s, &done)));
  if (done) return LGX_OK;
  return launch_rows<VT>(0, a.n, a, val, SpmvOp<VT, XT>{x, y}, s);
}

template <typename VT, typename XT>
lgx_status csr_residual(const Csr &a, const VT *val, const XT *b, const XT *x, XT *r,
                        double *norm, double *partials, unsigned *counter, cudaStream_t s,
                        const float *scale) {
  if (a.n == 0) {
    if (norm) LGX_CUDA(cudaMemsetAsync(norm, 0, sizeof(double), s));
    return LGX_OK;
  }
  if (norm)
    return launch_rows<VT>(0, a.n, a, val,
                           ResidualOp<VT, XT, true>{b, x, r, norm, partials, counter, scale}, s);
  bool done = false;
  LGX_CHECK((grid_residual<VT, XT>(a, val, b, x, r, scale, s, &done)));
  if (done) return LGX_OK;
  return launch_rows<VT>(0, a.n, a, val,
                         ResidualOp<VT, XT, false>{b, x, r, nullptr, nullptr, nullptr, scale},
                         s);
}

// partial-sum slots of a reducing row launch
// the row engine's grid never exceeds sm_count() * kRowsMaxCtasPerSm blocks
int64_t csr_partials(int64_t /*n*/) { return (int64_t)sm_count() * kRowsMaxCtasPerSm; }

template lgx_status csr_spmv<double, double>(const Csr &, const double *, const double *,
                                             double *, cudaStream_t);
template lgx_status csr_spmv<float, double>(const Csr &, const float *, const double *, double *,
                                            cudaStream_t);
template lgx_status csr_spmv<float, float>(const Csr &, const float *, const float *, float *,
                                           cudaStream_t);
template lgx_status csr_residual<double, double>(const Csr &, const double *, const double *,
                                                 const double *, double *, double *, double *,
                                                 unsigned *, cudaStream_t, const float *);
template lgx_status csr_residual<float, double>(const Csr &, const float *, const double *,
                                                const double *, double *, double *, double *,
                                                unsigned *, cudaStream_t, const float *);
template lgx_status csr_residual<float, float>(const Csr &, const float *, const float *,
                                               const float *, float *, double *, double *,
                                               unsigned *, cudaStream_t, const float *);
template lgx_status csr_residual<bf16, float>(const Csr &, const bf16 *, const float *,
                                              const float *, float *, double *, double *,
                                              unsigned *, cudaStream_t, const float *);

// ---------------------------------------------------------------------------
// Matrix-free 7-point diffusion stencil
//
// Row semantics (stencil/matrix/algorithm.hpp:93-227, scalar valued
// unordered iteration): off-diagonal to the neighbour on side s of axis d is
// -conn_d(i, j); the diagonal is the Dirichlet border terms of axis 0
// (2 q_0 c_i per boundary face) followed by the six connection values in the
// visiting order before(d = 0,1,2), after(d = 2,1,0); zero_to_one maps a zero
// diagonal to 1.  The product accumulates fma(-conn, x_j, sum) in the same
// visiting order and finishes with fma(diag, x_i, sum).
//
// The diagonal is computed once per matrix and cached (8 B/cell): on GB300
// the six FP64 additions per cell would otherwise nearly double the FP64
// pipe load of every product.  For the value valuator the harmonic means
// (one FP64 division per face) are likewise computed once into three face
// arrays; FP64 division runs at ~59 G/s on this part, so recomputing them
// would make the product ~10x slower than streaming the cached faces.
// ---------------------------------------------------------------------------
struct StencilDev {
  int n0, n1, n2;
  int lookup;
  double conn[48];  // lookup tables, staged into shared memory by each block
  const uint8_t *mat;
  const double *face0, *face1, *face2;  // value valuator: face d of cell i joins i and i+stride_d
  const double *diag;
};

// Copies the lookup tables of S into shared memory (all threads of the block
// must call it).
__device__ __forceinline__ const double *stage_conn(const StencilDev &S, double *sh) {
  const unsigned t = threadIdx.x + blockDim.x * threadIdx.y;
  if (S.lookup && t < 48) sh[t] = S.conn[t];
  __syncthreads();
  return sh;
}

__device__ __forceinline__ double st_conn_lookup(const double *conn, const uint8_t *mat, int d,
                                                 int64_t i, int64_t j) {
  return conn[d * 16 + mat[i] * 4 + mat[j]];
}

// off-diagonal connection values of cell (p0,p1,p2) = i, in visiting order
template <bool LOOKUP>
__device__ __forceinline__ void st_row(const StencilDev &S, const double *conn, int p0, int p1,
                                       int p2, int64_t i, double cv[6], int64_t cj[6],
                                       bool has[6]) {
  const int64_t s0 = (int64_t)S.n1 * S.n2, s1 = S.n2;
  // before: d = 0, 1, 2 ; after: d = 2, 1, 0
  has[0] = p0 > 0;
  has[1] = p1 > 0;
  has[2] = p2 > 0;
  has[3] = p2 + 1 < S.n2;
  has[4] = p1 + 1 < S.n1;
  has[5] = p0 + 1 < S.n0;
  cj[0] = i - s0;
  cj[1] = i - s1;
  cj[2] = i - 1;
  cj[3] = i + 1;
  cj[4] = i + s1;
  cj[5] = i + s0;
  if constexpr (LOOKUP) {
    cv[0] = has[0] ? st_conn_lookup(conn, S.mat, 0, i, cj[0]) : 0.0;
    cv[1] = has[1] ? st_conn_lookup(conn, S.mat, 1, i, cj[1]) : 0.0;
    cv[2] = has[2] ? st_conn_lookup(conn, S.mat, 2, i, cj[2]) : 0.0;
    cv[3] = has[3] ? st_conn_lookup(conn, S.mat, 2, i, cj[3]) : 0.0;
    cv[4] = has[4] ? st_conn_lookup(conn, S.mat, 1, i, cj[4]) : 0.0;
    cv[5] = has[5] ? st_conn_lookup(conn, S.mat, 0, i, cj[5]) : 0.0;
  } else {
    cv[0] = has[0] ? S.face0[cj[0]] : 0.0;
    cv[1] = has[1] ? S.face1[cj[1]] : 0.0;
    cv[2] = has[2] ? S.face2[cj[2]] : 0.0;
    cv[3] = has[3] ? S.face2[i] : 0.0;
    cv[4] = has[4] ? S.face1[i] : 0.0;
    cv[5] = has[5] ? S.face0[i] : 0.0;
  }
}

__device__ __forceinline__ double hm_dev(double a, double b) {
  const double p = __dmul_rn(a, b);
  return p != 0.0 ? __ddiv_rn(__dadd_rn(p, p), __dadd_rn(a, b)) : 0.0;
}

// value valuator faces: face_d[i] = hm(k_i, k_{i+stride_d}) * q_d
// k0/k1/k2: the conductivities of axes 0/1/2 (all k for the value valuator;
// one array per axis for the values valuator)
__global__ void k_st_faces(int n0, int n1, int n2, const double *k0, const double *k1,
                           const double *k2, double q0, double q1, double q2, double *f0,
                           double *f1, double *f2) {
  const int p2 = blockIdx.x * blockDim.x + threadIdx.x;
  const int p1 = blockIdx.y * blockDim.y + threadIdx.y;
  const int p0 = blockIdx.z;
  if (p2 >= n2 || p1 >= n1) return;
  const int64_t s0 = (int64_t)n1 * n2;
  const int64_t i = (int64_t)p0 * s0 + (int64_t)p1 * n2 + p2;
  f0[i] = p0 + 1 < n0 ? __dmul_rn(hm_dev(k0[i], k0[i + s0]), q0) : 0.0;
  f1[i] = p1 + 1 < n1 ? __dmul_rn(hm_dev(k1[i], k1[i + n2]), q1) : 0.0;
  f2[i] = p2 + 1 < n2 ? __dmul_rn(hm_dev(k2[i], k2[i + 1]), q2) : 0.0;
}

template <bool LOOKUP>
__global__ void k_st_diag(StencilDev S, const double *cell_value, double border_q0,
                          int zero_to_one, double *diag) {
  __shared__ double sh_conn[48];
  const double *conn = stage_conn(S, sh_conn);
  const int p2 = blockIdx.x * blockDim.x + threadIdx.x;
  const int p1 = blockIdx.y * blockDim.y + threadIdx.y;
  const int p0 = blockIdx.z;
  if (p2 >= S.n2 || p1 >= S.n1) return;
  const int64_t i = ((int64_t)p0 * S.n1 + p1) * S.n2 + p2;
  double cv[6];
  int64_t cj[6];
  bool has[6];
  st_row<LOOKUP>(S, conn, p0, p1, p2, i, cv, cj, has);
  const double c = cell_value[i];
  double d = 0.0;
  const double bt = __dmul_rn(border_q0, c);
  if (p0 == 0) d = __dadd_rn(d, bt);
  if (p0 + 1 == S.n0) d = __dadd_rn(d, bt);
#pragma unroll
  for (int e = 0; e < 6; ++e)
    if (has[e]) d = __dadd_rn(d, cv[e]);
  if (zero_to_one && d == 0.0) d = 1.0;
  diag[i] = d;
}

// cell values of the lookup valuator: coeffs[mat[i]]
__global__ void k_st_cellvalue(int64_t n, const uint8_t *mat, double c0, double c1, double c2,
                               double c3, double *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t m = mat[i];
    out[i] = m == 0 ? c0 : m == 1 ? c1 : m == 2 ? c2 : c3;
  }
}

template <bool LOOKUP, bool RESID, bool NORM>
__global__ void __launch_bounds__(256)
  k_st_apply(StencilDev S, const double *__restrict__ x, const double *__restrict__ b,
             double *__restrict__ y, double *norm, double *partials, unsigned *counter) {
  __shared__ double sh_conn[48];
  const double *conn = stage_conn(S, sh_conn);
  const int p2 = blockIdx.x * blockDim.x + threadIdx.x;
  const int p1 = blockIdx.y * blockDim.y + threadIdx.y;
  const int p0 = blockIdx.z;
  double contrib = 0.0;
  if (p2 < S.n2 && p1 < S.n1) {
    const int64_t i = ((int64_t)p0 * S.n1 + p1) * S.n2 + p2;
    double cv[6];
    int64_t cj[6];
    bool has[6];
    st_row<LOOKUP>(S, conn, p0, p1, p2, i, cv, cj, has);
    double sum = 0.0;
#pragma unroll
    for (int e = 0; e < 6; ++e)
      if (has[e]) sum = fma(-cv[e], __ldg(x + cj[e]), sum);
    sum = fma(S.diag[i], x[i], sum);
    if constexpr (RESID) {
      const double rv = b[i] - sum;
      y[i] = rv;
      contrib = rv * rv;
    } else {
      y[i] = sum;
    }
  }
  if constexpr (NORM) {
    const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
    __shared__ double sh[256];
    __shared__ bool last;
    // flatten (x, y) thread index for the block reduction
    const unsigned t = threadIdx.x + blockDim.x * threadIdx.y;
    sh[t] = contrib;
    __syncthreads();
    for (unsigned s = 128; s > 0; s >>= 1) {
      if (t < s) sh[t] += sh[t + s];
      __syncthreads();
    }
    if (t == 0) {
      partials[bid] = sh[0];
      __threadfence();
      last = atomicAdd(counter, 1u) == nb - 1;
    }
    __syncthreads();
    if (last) {
      __threadfence();
      double acc = 0.0;
      for (unsigned k = t; k < nb; k += 256) acc += ((volatile double *)partials)[k];
      sh[t] = acc;
      __syncthreads();
      for (unsigned s = 128; s > 0; s >>= 1) {
        if (t < s) sh[t] += sh[t + s];
        __syncthreads();
      }
      if (t == 0) {
        norm[0] = sh[0];
        *counter = 0;
      }
    }
  }
}

// ---- red-black SOR on the matrix-free stencil --------------------------------
// One colour of a red-black sweep, colour c = (p0 + p1 + p2) & 1, in natural
// order: thread (m, p1, p0) owns the cell p2 = 2 m + ((p0 + p1 + c) & 1) of
// its grid line.  Every neighbour has the other colour, so `nb` is where all
// of them are read: x_out once that colour was visited in this sweep, x_in
// before (null: zero).  The row is the SorOp row of the assembled matrix
// (gauss-seidel-variant/sweep.hpp:134-200, csr/create-from.hpp): accum = b_i,
// then in ascending column order (before axes 0, 1, 2; the diagonal; after
// axes 2, 1, 0) fma(conn, x_j, accum) for every non-zero connection -- the
// assembled entry is -conn -- and, in the ultra variant, fma(-a_ii, x_i,
// accum) at the diagonal; regular: x_i = fma(relax, accum / a_ii,
// (1 - relax) x_i); ultra: x_i + relax accum / |a_ii|.  The result equals
// the SOR of the assembled matrix in the row order sorted by (colour, index)
// bit for bit.
// 1 / diagonal, correctly rounded, for the rows whose diagonal lies within
// [2^-400, 2^400] in magnitude; 0 elsewhere (those rows divide directly)
__global__ void k_st_rdiag(int64_t n, const double *diag, double *rdiag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    rdiag[i] = exponent_within_400(diag[i]) ? 1.0 / diag[i] : 0.0;
}

template <bool LOOKUP>
__global__ void __launch_bounds__(256)
  k_st_sor_colour(StencilDev S, int colour, const double *nb, double relax, double m1, int ultra,
                  int relax_one, const double *__restrict__ rdiag, const double *x_in,
                  double *x_out, const double *__restrict__ b) {
  __shared__ double sh_conn[48];
  const double *conn = stage_conn(S, sh_conn);
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int p1 = blockIdx.y * blockDim.y + threadIdx.y;
  const int p0 = blockIdx.z;
  const int p2 = 2 * m + ((p0 + p1 + colour) & 1);
  if (p1 >= S.n1 || p2 >= S.n2) return;
  const int64_t i = ((int64_t)p0 * S.n1 + p1) * S.n2 + p2;
  double cv[6];
  int64_t cj[6];
  bool has[6];
  st_row<LOOKUP>(S, conn, p0, p1, p2, i, cv, cj, has);
  const double xi = x_in ? x_in[i] : 0.0;
  const double diag = S.diag[i];
  double accum = b[i];
#pragma unroll
  for (int e = 0; e < 6; ++e) {
    if (e == 3 && ultra) accum = fma(-diag, xi, accum);
    if (has[e] && nonzero_bits(cv[e])) accum = fma(cv[e], nb ? nb[cj[e]] : 0.0, accum);
  }
  if (ultra) {
    x_out[i] = xi + relax * accum / fabs(diag);
    return;
  }
  // the quotient through the reciprocal table (the same bits as accum /
  // diag), and relax = 1's shortcut where it cannot change the result
  const double y = rdiag[i];
  const double quot = (nonzero_bits(y) && exponent_within_400(accum))
                        ? div_by_recip(accum, diag, y) : accum / diag;
  if (relax_one && nonzero_bits(quot) && exponent_field(xi) != 0x7ff) {
    x_out[i] = quot;  // fma(1, q, 0 * x_i) == q for nonzero q and finite x_i
    return;
  }
  x_out[i] = fma(relax, quot, m1 * xi);
}

__global__ void k_st_rhs(int n0, int n1, int n2, const double *cell_value, double border_q0,
                         double us, double ue, double *b) {
  const int p2 = blockIdx.x * blockDim.x + threadIdx.x;
  const int p1 = blockIdx.y * blockDim.y + threadIdx.y;
  const int p0 = blockIdx.z;
  if (p2 >= n2 || p1 >= n1) return;
  const int64_t i = ((int64_t)p0 * n1 + p1) * n2 + p2;
  const double bt = __dmul_rn(border_q0, cell_value[i]);
  double sum = 0.0;
  if (p0 == 0) sum = __dadd_rn(sum, __dmul_rn(bt, us));
  if (p0 + 1 == n0) sum = __dadd_rn(sum, __dmul_rn(bt, ue));
  b[i] = sum;
}

// ---- plane-marching stencil kernel: x planes staged by TMA -----------------
// A CTA owns a tile of kStT1 x kStT2 cells of the (axis 1, axis 2) plane and
// marches along axis 0 through a slab of planes.  Every x plane of the tile,
// with a one-cell halo on axis 1 and a two-cell halo on axis 2 (so that the
// copy starts on a 16-byte boundary), arrives in shared memory through one
// cp.async.bulk.tensor.3d copy issued by thread 0 into a ring of four
// stages; planes p0 - 1, p0 and p0 + 1 are resident while plane p0 is
// computed and plane p0 + 2 is in flight.  Coordinates outside the grid read
// as 0 (they are never used: the has[] flags exclude them).  Each cell forms
// its sum in the order of k_st_apply, so results are bit-identical.
constexpr int kStT1 = 8, kStT2 = 64;
constexpr int kStHalo2 = 2;  // two doubles = 16 bytes
constexpr int kStBox1 = kStT1 + 2, kStBox2 = kStT2 + 2 * kStHalo2;
constexpr int kStStages = 4;
constexpr int kStPlaneBytes = kStBox1 * kStBox2 * 8;
constexpr int kStStageStride = (kStPlaneBytes + 127) & ~127;
constexpr int kStPlaneThreads = kStT1 * kStT2;
static_assert(kStBox2 * 8 % 16 == 0, "TMA rows must be whole 16-byte units");

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            int c2, uint64_t *bar) {
  asm volatile(
    "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
    " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
    "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
    : "memory");
}

template <bool LOOKUP, bool RESID, bool NORM>
__global__ void __launch_bounds__(kStPlaneThreads)
  k_st_apply_planes(const __grid_constant__ CUtensorMap xmap, StencilDev S, int slab,
                    const double *__restrict__ b, double *__restrict__ y, double *norm,
                    double *partials, unsigned *counter, int *err) {
  __shared__ __align__(128) unsigned char planes[kStStages * kStStageStride];
  __shared__ uint64_t bar[kStStages];
  __shared__ double sh_conn[48];
  __shared__ bool last;
  const double *conn = stage_conn(S, sh_conn);
  const int t = threadIdx.x;
  const int t1 = t / kStT2, t2 = t % kStT2;
  const int c1 = blockIdx.y * kStT1, c2 = blockIdx.x * kStT2;
  const int p1 = c1 + t1, p2 = c2 + t2;
  const int z0 = blockIdx.z * slab, z1 = min(z0 + slab, S.n0);
  const bool in = p1 < S.n1 && p2 < S.n2;
  // plane q lives in stage (q - z0 + 1) mod 4, in its ((q - z0 + 1) / 4)-th use
  auto stage_of = [&](int q) { return (q - z0 + 1) & (kStStages - 1); };
  auto parity_of = [&](int q) { return (unsigned)(((q - z0 + 1) >> 2) & 1); };
  auto plane = [&](int q) {
    return reinterpret_cast<const double *>(planes + stage_of(q) * kStStageStride);
  };
  auto issue = [&](int q) {
    const int st = stage_of(q);
    if (q < 0 || q >= S.n0) {
      // planes outside the grid are never read (has[] excludes them): the
      // stage's phase completes without a copy
      mbar_arrive(&bar[st]);
      return;
    }
    fence_proxy_async();
    mbar_expect_tx(&bar[st], kStPlaneBytes);
    tma_load_3d(planes + st * kStStageStride, &xmap, c2 - kStHalo2, c1 - 1, q, &bar[st]);
  };
  if (t == 0) {
    for (int st = 0; st < kStStages; ++st) mbar_init(&bar[st], 1);
    fence_mbar_init();
  }
  __syncthreads();
  // planes z0 - 1 .. z1 are read; the first four are issued up front
  int issued = min(z0 + 2, z1);
  if (t == 0)
    for (int q = z0 - 1; q <= issued; ++q) issue(q);
  int awaited = z0 - 2;
  bool ok = true;
  double contrib = 0.0;
  const int r = (t1 + 1) * kStBox2 + (t2 + kStHalo2);
  for (int p0 = z0; p0 < z1; ++p0) {
    bool mine = true;
    for (int q = awaited + 1; q <= p0 + 1; ++q)
      mine = mine && mbar_wait_bounded(&bar[stage_of(q)], parity_of(q));
    if (__syncthreads_or(!mine)) {
      ok = false;
      break;
    }
    awaited = p0 + 1;
    if (in) {
      const int64_t i = ((int64_t)p0 * S.n1 + p1) * S.n2 + p2;
      double cv[6];
      int64_t cj[6];
      bool has[6];
      st_row<LOOKUP>(S, conn, p0, p1, p2, i, cv, cj, has);
      const double *P0 = plane(p0);
      const double xv[6] = {plane(p0 - 1)[r], P0[r - kStBox2], P0[r - 1],
                            P0[r + 1],        P0[r + kStBox2], plane(p0 + 1)[r]};
      double sum = 0.0;
#pragma unroll
      for (int e = 0; e < 6; ++e)
        if (has[e]) sum = fma(-cv[e], xv[e], sum);
      sum = fma(S.diag[i], P0[r], sum);
      if constexpr (RESID) {
        const double rv = b[i] - sum;
        y[i] = rv;
        if constexpr (NORM) contrib += rv * rv;
      } else {
        y[i] = sum;
      }
    }
    __syncthreads();  // plane p0 - 1 is no longer read: its stage takes plane p0 + 3
    if (t == 0 && p0 + 3 <= z1) {
      issue(p0 + 3);
      issued = p0 + 3;
    }
  }
  if (!ok) {
    // a copy did not land in time: record it, let this CTA's copies finish
    // (bounded) and leave without a result
    if (t == 0) {
      atomicExch(err, 1);
      for (int q = awaited + 1; q <= issued; ++q)
        mbar_wait_bounded(&bar[stage_of(q)], parity_of(q));
    }
    return;
  }
  if constexpr (NORM) {
    const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
    // fixed-order block sum: lanes by shuffle-free halving in shared memory
    __shared__ double sh[kStPlaneThreads];
    sh[t] = contrib;
    __syncthreads();
    for (unsigned h = kStPlaneThreads / 2; h > 0; h >>= 1) {
      if (t < h) sh[t] += sh[t + h];
      __syncthreads();
    }
    if (t == 0) {
      partials[bid] = sh[0];
      __threadfence();
      last = atomicAdd(counter, 1u) == nb - 1;
    }
    __syncthreads();
    if (last) {
      __threadfence();
      double acc = 0.0;
      for (unsigned k = t; k < nb; k += kStPlaneThreads) acc += ((volatile double *)partials)[k];
      sh[t] = acc;
      __syncthreads();
      for (unsigned h = kStPlaneThreads / 2; h > 0; h >>= 1) {
        if (t < h) sh[t] += sh[t + h];
        __syncthreads();
      }
      if (t == 0) {
        norm[0] = sh[0];
        *counter = 0;
      }
    }
  }
}

// EffDiffCalc (component-wise/sink/effective-diffusion.hpp:226-320) over the
// middle planes of the flow axis: one CTA, each thread sums its cells of
// plane mid in order (stride 1024), then a fixed tree: out[0] = flux
// sum hm(c1, c2) (x(c2) - x(c1)), out[1] = filled-cell count (AreaPartSink)
constexpr int kEffThreads = 1024;
struct StDfac {
  double v[16];
};
__global__ void __launch_bounds__(kEffThreads)
  k_st_effdiff(int64_t other, int64_t base, const uint8_t *__restrict__ mat,
               const double *__restrict__ k, StDfac dfac, unsigned none_mask,
               const double *__restrict__ sol, const int64_t *__restrict__ cmap, double *out) {
  __shared__ double shf[kEffThreads];
  __shared__ double shn[kEffThreads];
  const int t = threadIdx.x;
  double flux = 0.0, filled = 0.0;
  for (int64_t c = t; c < other; c += kEffThreads) {
    const int64_t i1 = base + c, i2 = i1 + other;
    double hm;
    if (mat) {
      const unsigned m1 = mat[i1], m2 = mat[i2];
      filled += (double)(((none_mask >> m1) & 1u) == 0u) + (double)(((none_mask >> m2) & 1u) == 0u);
      hm = dfac.v[m1 * 4 + m2];  // the lookup valuator's diffusion_coeff
    } else {
      filled += 2.0;
      hm = hm_dev(k[i1], k[i2]);
    }
    if (cmap) {
      const int64_t k1 = cmap[i1], k2 = cmap[i2];
      if (k1 >= 0 && k2 >= 0) flux = fma(hm, sol[k2] - sol[k1], flux);
    } else {
      flux = fma(hm, sol[i2] - sol[i1], flux);
    }
  }
  shf[t] = flux;
  shn[t] = filled;
  __syncthreads();
  for (int h = kEffThreads / 2; h > 0; h >>= 1) {
    if (t < h) {
      shf[t] += shf[t + h];
      shn[t] += shn[t + h];
    }
    __syncthreads();
  }
  if (t == 0) {
    out[0] = shf[0];
    out[1] = shn[0];
  }
}

static dim3 st_grid(const StencilDesc &st) {
  return dim3((unsigned)((st.dims[2] + 31) / 32), (unsigned)((st.dims[1] + 7) / 8),
              (unsigned)st.dims[0]);
}
static const dim3 kStBlock(32, 8, 1);

int64_t stencil_partials(const StencilDesc &st) {
  const dim3 g = st_grid(st);
  return (int64_t)g.x * g.y * g.z;
}

}  // namespace lgx

// Device view of a stencil matrix.  The value valuator keeps its face arrays
// behind the conductivities in one buffer: k (n) | face0 (n) | face1 (n) |
// face2 (n).
namespace lgx {

static StencilDev dev_of(const lgx_matrix *a) {
  StencilDev S;
  S.n0 = (int)a->st.dims[0];
  S.n1 = (int)a->st.dims[1];
  S.n2 = (int)a->st.dims[2];
  S.lookup = a->st.lookup;
  S.mat = a->mat.p;
  S.face0 = S.face1 = S.face2 = nullptr;
  S.diag = a->diag.p;
  for (int t = 0; t < 48; ++t) S.conn[t] = a->st.conn[t];
  if (!a->st.lookup) {
    const double *base = a->k.p;
    S.face0 = base + a->n;
    S.face1 = base + 2 * a->n;
    S.face2 = base + 3 * a->n;
  }
  return S;
}

lgx_status stencil_ensure(lgx_matrix *a, cudaStream_t s, const double *k1, const double *k2) {
  if (a->diag.p) return LGX_OK;
  const StencilDesc &st = a->st;
  const int64_t n = a->n;
  if (!st.lookup) {
    // faces into k buffer slots 1..3
    double *base = a->k.p;
    k_st_faces<<<st_grid(st), kStBlock, 0, s>>>(
      (int)st.dims[0], (int)st.dims[1], (int)st.dims[2], base, k1 ? k1 : base, k2 ? k2 : base,
      st.q[0], st.q[1], st.q[2], base + n, base + 2 * n, base + 3 * n);
    LGX_LAUNCH_CHECK();
  }
  DBuf<double> cellv;
  const double *cell_value = a->k.p;
  if (st.lookup) {
    LGX_CHECK(cellv.alloc(n));
    k_st_cellvalue<<<std::min<int64_t>(grid_for(n, 256), 8192), 256, 0, s>>>(
      n, a->mat.p, st.coeffs[0], st.coeffs[1], st.coeffs[2], st.coeffs[3], cellv.p);
    LGX_LAUNCH_CHECK();
    cell_value = cellv.p;
  }
  LGX_CHECK(a->diag.alloc(n));
  StencilDev S = dev_of(a);
  const double bq0 = 2.0 * st.q[0];
  if (st.lookup) {
    k_st_diag<true><<<st_grid(st), kStBlock, 0, s>>>(S, cell_value, bq0, st.zero_to_one,
                                                     a->diag.p);
  } else {
    k_st_diag<false><<<st_grid(st), kStBlock, 0, s>>>(S, cell_value, bq0, st.zero_to_one,
                                                      a->diag.p);
  }
  LGX_LAUNCH_CHECK();
  LGX_CUDA(cudaStreamSynchronize(s));  // cellv is released on return
  return LGX_OK;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda)
static EncodeTiledFn encode_tiled() {
  static const EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (EncodeTiledFn) nullptr;
    }
    return (EncodeTiledFn)p;
  }();
  return fn;
}

// Stencil engine: 0 thread per cell (default), 1 plane march with TMA-staged
// x planes.  Both are FP64-pipe bound on GB300 (7 FMAs per cell against 25-48
// bytes); the thread-per-cell kernel keeps more cells in flight and is the
// faster one (256^3: 0.204-0.214 ms against 0.267-0.275 ms).
static std::atomic<int> g_stencil_engine{[] {
  const char *e = std::getenv("LGX_STENCIL_PLANES");
  return (e && e[0] == '1') ? 1 : 0;
}()};

static bool stencil_planes_enabled() { return g_stencil_engine.load(std::memory_order_relaxed); }

template <bool LOOKUP, bool RESID, bool NORM>
static lgx_status launch_planes(const StencilDesc &st, const CUtensorMap &map,
                                const StencilDev &S, const double *b, double *y, double *norm,
                                double *partials, unsigned *counter, cudaStream_t s) {
  // CTAs per SM, queried once per kernel (0 until the first query succeeds)
  static std::atomic<int> cached{0};
  int per_sm = cached.load(std::memory_order_relaxed);
  if (per_sm == 0) {
    int v = 0;
    LGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &v, k_st_apply_planes<LOOKUP, RESID, NORM>, kStPlaneThreads, 0));
    per_sm = std::max(v, 1);
    cached.store(per_sm, std::memory_order_relaxed);
  }
  const int64_t n0 = st.dims[0], n1 = st.dims[1], n2 = st.dims[2];
  const int64_t gx = (n2 + kStT2 - 1) / kStT2, gy = (n1 + kStT1 - 1) / kStT1;
  // slabs along axis 0 so that about one wave of CTAs is resident
  const int64_t slots = (int64_t)sm_count() * per_sm;
  const int64_t slabs = std::min<int64_t>(std::max<int64_t>(slots / (gx * gy), 1), n0);
  const int slab = (int)((n0 + slabs - 1) / slabs);
  const dim3 g((unsigned)gx, (unsigned)gy, (unsigned)((n0 + slab - 1) / slab));
  k_st_apply_planes<LOOKUP, RESID, NORM><<<g, kStPlaneThreads, 0, s>>>(
    map, S, slab, b, y, norm, partials, counter, device_error_flag());
  LGX_LAUNCH_CHECK();
  count_launch();
  return LGX_OK;
}

// Runs the plane-marching kernel when its TMA preconditions hold (x on a
// 16-byte boundary, even axis-2 length so every plane row is a whole number
// of 16-byte units); *done tells whether it ran.
static lgx_status stencil_apply_planes(const lgx_matrix *a, const double *x, const double *b,
                                       double *y, double *norm, double *partials,
                                       unsigned *counter, cudaStream_t s, bool *done) {
  *done = false;
  const StencilDesc &st = a->st;
  const EncodeTiledFn encode = encode_tiled();
  if (!stencil_planes_enabled() || !encode || st.dims[2] % 2 != 0 ||
      (reinterpret_cast<uintptr_t>(x) & 15) != 0 || st.dims[1] > (int64_t)kStT1 * 65535)
    return LGX_OK;
  CUtensorMap map;
  const cuuint64_t gdim[3] = {(cuuint64_t)st.dims[2], (cuuint64_t)st.dims[1],
                              (cuuint64_t)st.dims[0]};
  const cuuint64_t gstride[2] = {(cuuint64_t)st.dims[2] * 8,
                                 (cuuint64_t)st.dims[2] * st.dims[1] * 8};
  const cuuint32_t box[3] = {(cuuint32_t)kStBox2, (cuuint32_t)kStBox1, 1};
  const cuuint32_t estride[3] = {1, 1, 1};
  if (encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double *>(x), gdim, gstride, box,
             estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return LGX_OK;
  const StencilDev S = dev_of(a);
  const bool lk = st.lookup;
  if (!b) {
    LGX_CHECK((lk ? launch_planes<true, false, false> : launch_planes<false, false, false>)(
      st, map, S, b, y, norm, partials, counter, s));
  } else if (!norm) {
    LGX_CHECK((lk ? launch_planes<true, true, false> : launch_planes<false, true, false>)(
      st, map, S, b, y, norm, partials, counter, s));
  } else {
    LGX_CHECK((lk ? launch_planes<true, true, true> : launch_planes<false, true, true>)(
      st, map, S, b, y, norm, partials, counter, s));
  }
  *done = true;
  return LGX_OK;
}

static lgx_status stencil_apply(const lgx_matrix *ac, const double *x, const double *b, double *y,
                                double *norm, double *partials, unsigned *counter,
                                cudaStream_t s) {
  lgx_matrix *a = const_cast<lgx_matrix *>(ac);
  LGX_CHECK(stencil_ensure(a, s));
  bool done = false;
  LGX_CHECK(stencil_apply_planes(a, x, b, y, norm, partials, counter, s, &done));
  if (done) return LGX_OK;
  StencilDev S = dev_of(a);
  const dim3 g = st_grid(a->st);
  const bool lk = a->st.lookup;
  if (!b) {
    if (lk) k_st_apply<true, false, false><<<g, kStBlock, 0, s>>>(S, x, nullptr, y, nullptr,
                                                                  nullptr, nullptr);
    else k_st_apply<false, false, false><<<g, kStBlock, 0, s>>>(S, x, nullptr, y, nullptr,
                                                                nullptr, nullptr);
  } else if (!norm) {
    if (lk) k_st_apply<true, true, false><<<g, kStBlock, 0, s>>>(S, x, b, y, nullptr, nullptr,
                                                                 nullptr);
    else k_st_apply<false, true, false><<<g, kStBlock, 0, s>>>(S, x, b, y, nullptr, nullptr,
                                                               nullptr);
  } else {
    if (lk) k_st_apply<true, true, true><<<g, kStBlock, 0, s>>>(S, x, b, y, norm, partials,
                                                                counter);
    else k_st_apply<false, true, true><<<g, kStBlock, 0, s>>>(S, x, b, y, norm, partials,
                                                              counter);
  }
  LGX_LAUNCH_CHECK();
  count_launch();
  return LGX_OK;
}

// One red-black SOR sweep on a stencil matrix: colour 0 then 1 (forward) or
// 1 then 0 (backward); x_in may equal x_out (in situ) or be null (zero).
lgx_status stencil_sor_sweep(const lgx_matrix *ac, double relax, int forward, int ultra,
                             const double *x_in, double *x_out, const double *b,
                             cudaStream_t s) {
  lgx_matrix *a = const_cast<lgx_matrix *>(ac);
  if (a->n == 0) return LGX_OK;
  LGX_CHECK(stencil_ensure(a, s));
  if (!a->rdiag.p) {
    LGX_CHECK(a->rdiag.alloc(a->n));
    k_st_rdiag<<<std::min<int64_t>(grid_for(a->n, 256), 16384), 256, 0, s>>>(a->n, a->diag.p,
                                                                            a->rdiag.p);
    LGX_LAUNCH_CHECK();
  }
  StencilDev S = dev_of(a);
  const dim3 g((unsigned)(((S.n2 + 1) / 2 + 31) / 32), (unsigned)((S.n1 + 7) / 8),
               (unsigned)S.n0);
  const double m1 = 1.0 - relax;
  const int relax_one = relax == 1.0;
  for (int cc = 0; cc < 2; ++cc) {
    const int colour = forward ? cc : 1 - cc;
    const double *nb = cc == 0 ? x_in : x_out;
    if (a->st.lookup)
      k_st_sor_colour<true><<<g, kStBlock, 0, s>>>(S, colour, nb, relax, m1, ultra, relax_one,
                                                   a->rdiag.p, x_in, x_out, b);
    else
      k_st_sor_colour<false><<<g, kStBlock, 0, s>>>(S, colour, nb, relax, m1, ultra, relax_one,
                                                    a->rdiag.p, x_in, x_out, b);
    LGX_LAUNCH_CHECK();
  }
  return LGX_OK;
}

lgx_status matrix_spmv(const lgx_matrix *a, const double *x, double *y, cudaStream_t s) {
  if (a->kind == LGX_MATRIX_CSR) {
    if (a->csr.storage == LGX_F64) return csr_spmv<double, double>(a->csr, a->csr.v64.p, x, y, s);
    return csr_spmv<float, double>(a->csr, a->csr.v32.p, x, y, s);
  }
  return stencil_apply(a, x, nullptr, y, nullptr, nullptr, nullptr, s);
}

lgx_status matrix_residual(const lgx_matrix *a, const double *b, const double *x, double *r,
                           double *norm, double *partials, unsigned *counter, cudaStream_t s) {
  if (a->kind == LGX_MATRIX_CSR) {
    if (a->csr.storage == LGX_F64)
      return csr_residual<double, double>(a->csr, a->csr.v64.p, b, x, r, norm, partials, counter,
                                          s);
    return csr_residual<float, double>(a->csr, a->csr.v32.p, b, x, r, norm, partials, counter, s);
  }
  return stencil_apply(a, x, b, r, norm, partials, counter, s);
}

int64_t matrix_partials(const lgx_matrix *a) {
  if (a->kind == LGX_MATRIX_CSR) return csr_partials(a->n);
  return stencil_partials(a->st);
}

__global__ void k_csr_diag(int64_t n, const int64_t *rowptr, const int32_t *col,
                           const double *v64, const float *v32, double *d) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = 0.0;
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e)
      if (col[e] == i) v = v64 ? v64[e] : (double)v32[e];
    d[i] = v;
  }
}

lgx_status matrix_diagonal(lgx_matrix *a, cudaStream_t s, const double **out) {
  if (a->kind != LGX_MATRIX_CSR) {
    LGX_CHECK(stencil_ensure(a, s));
    *out = a->diag.p;
    return LGX_OK;
  }
  if (!a->diag.p) {
    LGX_CHECK(a->diag.alloc(a->n));
    const Csr &c = a->csr;
    k_csr_diag<<<std::min<int64_t>(grid_for(a->n, 256), 8192), 256, 0, s>>>(
      a->n, c.rowptr.p, c.col.p, c.storage == LGX_F64 ? c.v64.p : nullptr,
      c.storage == LGX_F32 ? c.v32.p : nullptr, a->diag.p);
    LGX_LAUNCH_CHECK();
  }
  *out = a->diag.p;
  return LGX_OK;
}

// ---------------------------------------------------------------------------
// Stencil -> CSR (csr/create-from.hpp:37-246)
// ---------------------------------------------------------------------------
__global__ void k_st_count(StencilDev S, int zero_to_one, const double *__restrict__ raw_diag,
                           int64_t *keep, int64_t *rowlen, bool lookup) {
  __shared__ double sh_conn[48];
  const double *conn = stage_conn(S, sh_conn);
  const int p2 = blockIdx.x * blockDim.x + threadIdx.x;
  const int p1 = blockIdx.y * blockDim.y + threadIdx.y;
  const int p0 = blockIdx.z;
  if (p2 >= S.n2 || p1 >= S.n1) return;
  const int64_t i = ((int64_t)p0 * S.n1 + p1) * S.n2 + p2;
  double cv[6];
  int64_t cj[6];
  bool has[6];
  if (lookup) st_row<true>(S, conn, p0, p1, p2, i, cv, cj, has);
  else st_row<false>(S, conn, p0, p1, p2, i, cv, cj, has);
  const bool kept = zero_to_one || S.diag[i] != 0.0;
  keep[i] = kept;
  int64_t c = 1;
  for (int e = 0; e < 6; ++e) c += has[e] && cv[e] != 0.0;
  rowlen[i] = kept ? c : 0;
}

__global__ void k_st_fill(StencilDev S, bool lookup, const int64_t *rowid_incl,
                          const int64_t *rowptr_by_cell, int64_t *rowptr, int32_t *col,
                          double *val, int64_t *cmap) {
  __shared__ double sh_conn[48];
  const double *conn = stage_conn(S, sh_conn);
  const int p2 = blockIdx.x * blockDim.x + threadIdx.x;
  const int p1 = blockIdx.y * blockDim.y + threadIdx.y;
  const int p0 = blockIdx.z;
  if (p2 >= S.n2 || p1 >= S.n1) return;
  const int64_t i = ((int64_t)p0 * S.n1 + p1) * S.n2 + p2;
  // rowid_incl: offsets array of the keep flags (rowid_incl[i] = rows before i)
  const bool kept = rowid_incl[i + 1] != rowid_incl[i];
  if (cmap) cmap[i] = kept ? rowid_incl[i] : -1;
  if (!kept) return;
  const int64_t r = rowid_incl[i];
  int64_t pos = rowptr_by_cell[i];
  rowptr[r] = pos;
  double cv[6];
  int64_t cj[6];
  bool has[6];
  if (lookup) st_row<true>(S, conn, p0, p1, p2, i, cv, cj, has);
  else st_row<false>(S, conn, p0, p1, p2, i, cv, cj, has);
  for (int e = 0; e < 3; ++e)
    if (has[e] && cv[e] != 0.0) {
      col[pos] = (int32_t)rowid_incl[cj[e]];
      val[pos++] = -cv[e];
    }
  col[pos] = (int32_t)r;
  val[pos++] = S.diag[i];
  for (int e = 3; e < 6; ++e)
    if (has[e] && cv[e] != 0.0) {
      col[pos] = (int32_t)rowid_incl[cj[e]];
      val[pos++] = -cv[e];
    }
}

}  // namespace lgx

using namespace lgx;

extern "C" {

// henry < 0: SymmetricDiffusionLookupProvider; else HenryDiffusionLookupProvider
// with that constant and the gaseous materials in gaseous_mask
static lgx_status stencil_create(const int64_t dims[3], const double q[3], const double coeffs[4],
                                 const uint8_t *d_mat, const double *d_k, double sol_start,
                                 double sol_end, int zero_to_one, lgx_stream stream,
                                 lgx_matrix **out, const double *d_k1 = nullptr,
                                 const double *d_k2 = nullptr, double henry = -1.0,
                                 unsigned gaseous_mask = 0) {
  if (!dims || !q || !out) return fail(LGX_ERR_INVALID, "null argument");
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1)
    return fail(LGX_ERR_INVALID, "grid dimensions must be positive");
  if (dims[0] > 65535) return fail(LGX_ERR_INVALID, "axis 0 is limited to 65535 cells");
  const int64_t n = dims[0] * dims[1] * dims[2];
  if (n > INT32_MAX) return fail(LGX_ERR_INVALID, "grid too large for 32-bit indices");
  auto *m = new lgx_matrix();
  m->kind = d_mat ? LGX_MATRIX_STENCIL_LOOKUP : LGX_MATRIX_STENCIL_VALUE;
  m->n = n;
  m->symmetric = 1;
  StencilDesc &st = m->st;
  for (int d = 0; d < 3; ++d) {
    st.dims[d] = dims[d];
    st.q[d] = q[d];
  }
  st.sol_start = sol_start;
  st.sol_end = sol_end;
  st.zero_to_one = zero_to_one;
  st.lookup = d_mat != nullptr;
  st.values = d_k1 != nullptr;
  lgx_status s = LGX_OK;
  if (d_mat) {
    for (int c = 0; c < 4; ++c) st.coeffs[c] = coeffs[c];
    // lookup-wright.hpp:18-60: diffusion factor hm(c_a, c_b), or with the
    // Henry provider hm(c_a f_b, c_b f_a) (f = henry for gaseous materials);
    // lookup-wright.hpp:73-85: conn[d][a*4+b] = factor * q_d
    for (int f = 0; f < 16; ++f) {
      double a = coeffs[f / 4], b = coeffs[f % 4];
      if (henry >= 0.0) {
        const double fa = (gaseous_mask >> (f / 4)) & 1u ? henry : 1.0;
        const double fb = (gaseous_mask >> (f % 4)) & 1u ? henry : 1.0;
        a = coeffs[f / 4] * fb;
        b = coeffs[f % 4] * fa;
      }
      const double p = a * b;
      st.dfac[f] = p != 0.0 ? (p + p) / (a + b) : 0.0;
    }
    for (int d = 0; d < 3; ++d)
      for (int f = 0; f < 16; ++f) st.conn[d * 16 + f] = st.dfac[f] * q[d];
    s = m->mat.alloc(n);
    if (s == LGX_OK &&
        cudaMemcpyAsync(m->mat.p, d_mat, n, cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
      s = fail(LGX_ERR_CUDA, "copying materials failed");
  } else {
    s = m->k.alloc(4 * n);  // k | face0 | face1 | face2
    if (s == LGX_OK && cudaMemcpyAsync(m->k.p, d_k, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                       stream) != cudaSuccess)
      s = fail(LGX_ERR_CUDA, "copying conductivities failed");
  }
  if (s == LGX_OK) s = stencil_ensure(m, stream, d_k1, d_k2);
  if (s != LGX_OK) {
    delete m;
    return s;
  }
  // stored non-zeros of the assembled matrix (zero connections included)
  int64_t nnz = n;
  for (int d = 0; d < 3; ++d) nnz += 2 * (dims[d] - 1) * (n / dims[d]);
  m->nnz = nnz;
  *out = m;
  return LGX_OK;
}

lgx_status lgx_box_axis_quotients(const lgx_box_info *box, double q[3]) {
  if (!box || !q) return fail(LGX_ERR_INVALID, "null argument");
  double h[3];
  for (int d = 0; d < 3; ++d) {
    if (box->cells[d] < 1) return fail(LGX_ERR_INVALID, "cell counts must be positive");
    if (!(box->lengths[d] > 0.0) || !std::isfinite(box->lengths[d]))
      return fail(LGX_ERR_INVALID, "axis lengths must be positive and finite");
    h[d] = box->lengths[d] / (double)box->cells[d];
  }
  // the axis area (the other axes' spacings multiplied from the lowest axis)
  // over the axis's own spacing
  for (int d = 0; d < 3; ++d) {
    double area = 1.0;
    for (int e = 0; e < 3; ++e)
      if (e != d) area = area * h[e];
    q[d] = area / h[d];
  }
  return LGX_OK;
}

lgx_status lgx_stencil_create_lookup(const int64_t dims[3], const double q[3],
                                     const double coeffs[4], const uint8_t *d_mat,
                                     double sol_start, double sol_end, int zero_to_one,
                                     lgx_stream stream, lgx_matrix **out) {
  if (!d_mat || !coeffs) return fail(LGX_ERR_INVALID, "null materials");
  return stencil_create(dims, q, coeffs, d_mat, nullptr, sol_start, sol_end, zero_to_one, stream,
                        out);
}

lgx_status lgx_stencil_create_lookup_henry(const int64_t dims[3], const double q[3],
                                           const double coeffs[4], uint8_t gaseous_materials,
                                           double henry_constant, const uint8_t *d_mat,
                                           double sol_start, double sol_end, int zero_to_one,
                                           lgx_stream stream, lgx_matrix **out) {
  if (!d_mat || !coeffs) return fail(LGX_ERR_INVALID, "null materials");
  if (!(henry_constant >= 0.0)) return fail(LGX_ERR_INVALID, "the Henry constant must be >= 0");
  return stencil_create(dims, q, coeffs, d_mat, nullptr, sol_start, sol_end, zero_to_one, stream,
                        out, nullptr, nullptr, henry_constant, gaseous_materials);
}

lgx_status lgx_stencil_create_value(const int64_t dims[3], const double q[3], const double *d_k,
                                    double sol_start, double sol_end, int zero_to_one,
                                    lgx_stream stream, lgx_matrix **out) {
  if (!d_k) return fail(LGX_ERR_INVALID, "null conductivities");
  return stencil_create(dims, q, nullptr, nullptr, d_k, sol_start, sol_end, zero_to_one, stream,
                        out);
}

lgx_status lgx_stencil_create_values(const int64_t dims[3], const double q[3], const double *d_k0,
                                     const double *d_k1, const double *d_k2, double sol_start,
                                     double sol_end, int zero_to_one, lgx_stream stream,
                                     lgx_matrix **out) {
  if (!d_k0 || !d_k1 || !d_k2) return fail(LGX_ERR_INVALID, "null conductivities");
  return stencil_create(dims, q, nullptr, nullptr, d_k0, sol_start, sol_end, zero_to_one, stream,
                        out, d_k1, d_k2);
}

lgx_status lgx_stencil_engine_set(int engine) {
  if (engine != 0 && engine != 1) return fail(LGX_ERR_INVALID, "stencil engine must be 0 or 1");
  g_stencil_engine.store(engine, std::memory_order_relaxed);
  return LGX_OK;
}

int lgx_stencil_engine_get(void) { return g_stencil_engine.load(std::memory_order_relaxed); }

lgx_status lgx_spmv(const lgx_matrix *a, const double *d_x, double *d_y, lgx_stream stream) {
  if (!a || (a->n > 0 && (!d_x || !d_y))) return fail(LGX_ERR_INVALID, "null argument");
  return matrix_spmv(a, d_x, d_y, stream);
}

lgx_status lgx_spmv_f32(const lgx_matrix *a, const float *d_x, float *d_y, lgx_stream stream) {
  if (!a || (a->n > 0 && (!d_x || !d_y))) return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind != LGX_MATRIX_CSR || a->csr.storage != LGX_F32)
    return fail(LGX_ERR_UNSUPPORTED, "lgx_spmv_f32 needs a float-stored CSR matrix");
  return csr_spmv<float, float>(a->csr, a->csr.v32.p, d_x, d_y, stream);
}

lgx_status lgx_residual(const lgx_matrix *a, const double *d_b, const double *d_x, double *d_r,
                        double *d_norm2sq, lgx_stream stream) {
  if (!a || (a->n > 0 && (!d_b || !d_x || !d_r))) return fail(LGX_ERR_INVALID, "null argument");
  DBuf<double> partials;
  DBuf<unsigned> counter;
  if (d_norm2sq) {
    LGX_CHECK(partials.alloc(matrix_partials(a)));
    LGX_CHECK(counter.alloc(1));
    LGX_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(unsigned), stream));
  }
  LGX_CHECK(matrix_residual(a, d_b, d_x, d_r, d_norm2sq, partials.p, counter.p, stream));
  if (d_norm2sq) LGX_CUDA(cudaStreamSynchronize(stream));
  return LGX_OK;
}

lgx_status lgx_diagonal(const lgx_matrix *a, double *d_diag, lgx_stream stream) {
  if (!a || (a->n > 0 && !d_diag)) return fail(LGX_ERR_INVALID, "null argument");
  const double *d = nullptr;
  LGX_CHECK(matrix_diagonal(const_cast<lgx_matrix *>(a), stream, &d));
  if (a->n)
    LGX_CUDA(cudaMemcpyAsync(d_diag, d, sizeof(double) * a->n, cudaMemcpyDeviceToDevice, stream));
  return LGX_OK;
}

lgx_status lgx_stencil_effective_diffusion(const lgx_matrix *a, const double lengths[3],
                                           uint8_t none_materials, const double *d_sol,
                                           const int64_t *d_compress_map, lgx_stream stream,
                                           double *h_eff, double *h_area_part) {
  if (!a || !lengths || !d_sol || !h_eff) return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind == LGX_MATRIX_CSR) return fail(LGX_ERR_UNSUPPORTED, "not a stencil matrix");
  const StencilDesc &st = a->st;
  if (st.values)
    return fail(LGX_ERR_UNSUPPORTED, "the values valuator has no diffusion coefficient");
  if (st.dims[0] < 2) return fail(LGX_ERR_INVALID, "the flow axis needs two planes");
  const int64_t other = st.dims[1] * st.dims[2], mid = st.dims[0] / 2;
  DBuf<double> out;
  LGX_CHECK(out.alloc(2));
  const cudaStream_t s = (cudaStream_t)stream;
  StDfac dfac;
  for (int f = 0; f < 16; ++f) dfac.v[f] = st.dfac[f];
  k_st_effdiff<<<1, kEffThreads, 0, s>>>(other, mid * other, st.lookup ? a->mat.p : nullptr,
                                         st.lookup ? nullptr : a->k.p, dfac,
                                         (unsigned)none_materials, d_sol, d_compress_map, out.p);
  LGX_LAUNCH_CHECK();
  count_launch();
  double h[2] = {0.0, 0.0};
  LGX_CUDA(cudaMemcpyAsync(h, out.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  const double area_part = h[1] / (double)other * 0.5;
  double eff = h[0];
  eff *= st.q[0];
  eff /= area_part * (lengths[1] * lengths[2]);
  eff *= lengths[0];
  *h_eff = eff / (st.sol_end - st.sol_start);
  if (h_area_part) *h_area_part = area_part;
  return LGX_OK;
}

lgx_status lgx_stencil_rhs(const lgx_matrix *a, double *d_b, lgx_stream stream) {
  if (!a || !d_b) return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind == LGX_MATRIX_CSR) return fail(LGX_ERR_UNSUPPORTED, "not a stencil matrix");
  const StencilDesc &st = a->st;
  DBuf<double> cellv;
  const double *cv = a->k.p;
  if (st.lookup) {
    LGX_CHECK(cellv.alloc(a->n));
    k_st_cellvalue<<<std::min<int64_t>(grid_for(a->n, 256), 8192), 256, 0, stream>>>(
      a->n, a->mat.p, st.coeffs[0], st.coeffs[1], st.coeffs[2], st.coeffs[3], cellv.p);
    LGX_LAUNCH_CHECK();
    cv = cellv.p;
  }
  k_st_rhs<<<st_grid(st), kStBlock, 0, stream>>>((int)st.dims[0], (int)st.dims[1],
                                                 (int)st.dims[2], cv, 2.0 * st.q[0], st.sol_start,
                                                 st.sol_end, d_b);
  LGX_LAUNCH_CHECK();
  LGX_CUDA(cudaStreamSynchronize(stream));
  return LGX_OK;
}

lgx_status lgx_stencil_to_csr(const lgx_matrix *ac, int64_t *d_compress_map, lgx_stream stream,
                              lgx_matrix **out) {
  if (!ac || !out) return fail(LGX_ERR_INVALID, "null argument");
  if (ac->kind == LGX_MATRIX_CSR) return fail(LGX_ERR_UNSUPPORTED, "not a stencil matrix");
  lgx_matrix *a = const_cast<lgx_matrix *>(ac);
  LGX_CHECK(stencil_ensure(a, stream));
  const int64_t n = a->n;
  DBuf<int64_t> keep, rowlen, rowid, rptr_cell;
  LGX_CHECK(keep.alloc(n));
  LGX_CHECK(rowlen.alloc(n));
  LGX_CHECK(rowid.alloc(n + 1));
  LGX_CHECK(rptr_cell.alloc(n + 1));
  StencilDev S = dev_of(a);
  const dim3 g = st_grid(a->st);
  k_st_count<<<g, kStBlock, 0, stream>>>(S, a->st.zero_to_one, a->diag.p, keep.p, rowlen.p,
                                         a->st.lookup != 0);
  LGX_LAUNCH_CHECK();
  LGX_CHECK(inclusive_offsets(n, keep.p, rowid.p, stream));
  LGX_CHECK(inclusive_offsets(n, rowlen.p, rptr_cell.p, stream));
  int64_t rows = 0, nnz = 0;
  LGX_CUDA(cudaMemcpyAsync(&rows, rowid.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, stream));
  LGX_CUDA(cudaMemcpyAsync(&nnz, rptr_cell.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost,
                           stream));
  LGX_CUDA(cudaStreamSynchronize(stream));
  DBuf<int64_t> rowptr;
  DBuf<int32_t> col;
  DBuf<double> val;
  LGX_CHECK(rowptr.alloc(rows + 1));
  LGX_CHECK(col.alloc(nnz));
  LGX_CHECK(val.alloc(nnz));
  k_st_fill<<<g, kStBlock, 0, stream>>>(S, a->st.lookup != 0, rowid.p, rptr_cell.p, rowptr.p,
                                        col.p, val.p, d_compress_map);
  LGX_LAUNCH_CHECK();
  LGX_CUDA(cudaMemcpyAsync(rowptr.p + rows, &nnz, sizeof(int64_t), cudaMemcpyHostToDevice,
                           stream));
  return lgx_csr_create(rows, nnz, rowptr.p, col.p, val.p, 1, LGX_F64, stream, out);
}

}  // extern "C"
