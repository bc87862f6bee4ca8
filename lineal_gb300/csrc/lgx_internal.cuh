// Internal definitions shared by the lineal_gb300 CUDA sources.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "lineal_gb300.h"

namespace lgx {

// ---- value types ---------------------------------------------------------
// Stored matrix values are double, float or (precision form) bfloat16 with a
// per-row float scale.  cvt<XT>(v) widens a stored value to the arithmetic
// type.
using bf16 = __nv_bfloat16;
template <typename XT, typename VT>
__host__ __device__ __forceinline__ XT cvt(VT v) {
  return static_cast<XT>(v);
}
template <>
__host__ __device__ __forceinline__ float cvt<float, bf16>(bf16 v) {
  return __bfloat162float(v);
}
template <typename VT>
inline constexpr bool kIsBf16 = false;
template <>
inline constexpr bool kIsBf16<bf16> = true;


// ---- error handling -----------------------------------------------------
void set_error(const std::string &msg);
lgx_status fail(lgx_status s, const std::string &msg);
lgx_status cuda_fail(cudaError_t e, const char *what);

#define LGX_CUDA(...)                                                          \
  do {                                                                         \
    cudaError_t lgx_e_ = (__VA_ARGS__);                                        \
    if (lgx_e_ != cudaSuccess) return ::lgx::cuda_fail(lgx_e_, #__VA_ARGS__); \
  } while (0)
#define LGX_CHECK(...)                           \
  do {                                           \
    lgx_status lgx_s_ = (__VA_ARGS__);           \
    if (lgx_s_ != LGX_OK) return lgx_s_;         \
  } while (0)
void count_launch();
// adds the kernel nodes of a replayed graph to the launch count
void count_launches(uint64_t k);
uint64_t launch_count();
// Every kernel launch site is followed by this check, which also counts the
// launch (lgx_kernel_launches).
#define LGX_LAUNCH_CHECK()     \
  do {                         \
    ::lgx::count_launch();     \
    LGX_CUDA(cudaGetLastError()); \
  } while (0)

// ---- device buffers -----------------------------------------------------
template <typename T>
struct DBuf {
  T *p = nullptr;
  int64_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  lgx_status alloc(int64_t count) {
    release();
    if (count <= 0) count = 1;
    cudaError_t e = cudaMalloc(&p, sizeof(T) * (size_t)count);
    if (e != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();
      return fail(LGX_ERR_NOMEM, "device allocation of " + std::to_string(sizeof(T) * count) +
                                     " bytes failed: " + cudaGetErrorString(e));
    }
    n = count;
    return LGX_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

constexpr uint32_t kUnaggregated = 0xFFFFFFFFu;
// trailing elements of every CSR column/value buffer (the staged row kernels
// copy 16-byte-aligned spans that may reach past the last entry)
constexpr int kCsrPad = 16;
constexpr uint32_t kIsolated = 0xFFFFFFFEu;

// ---- matrices -------------------------------------------------------------
struct Grid27;

struct Csr {
  int64_t n = 0, nnz = 0;
  int64_t max_row = 0;
  int64_t max_win = 0;  // most entries in any kWarpTileRows consecutive rows
  // row-engine configuration chosen by the autotuner per operation class
  // (0 products: SpMV and residual, 1 SOR sweeps) and value type (0 FP64,
  // 1 FP32, 2 BF16); -1 = the process-wide configuration
  int8_t tuned[2][3] = {{-1, -1, -1}, {-1, -1, -1}};
  int symmetric = 0;
  lgx_dtype storage = LGX_F64;
  DBuf<int64_t> rowptr;
  DBuf<int32_t> col;
  DBuf<double> v64;
  DBuf<float> v32;
  // rows of a 27- or 7-point grid matrix in colour order, stored without
  // column indices (products and sweeps use it when set; see lgx_grid.cu)
  std::shared_ptr<const Grid27> grid;
};

// Colour-permuted grid matrix: 27 points (even edge lengths, parity
// colouring c = 4 (i & 1) + 2 (j & 1) + (k & 1), B = n / 8) or 7 points (even
// n2, red-black colouring c = (i + j + k) & 1, B = n / 2); colour c in rows
// [c B, (c + 1) B), natural order inside a colour.  Row values are stored per
// stencil offset e = 9 (dz + 1) + 3 (dy + 1) + (dx + 1) -- the CSR row order
// -- offset-major (v[e S + r], S = n padded to an odd multiple of 32
// entries so that the 27 planes of one row do not sit a power of two apart),
// 0 where the neighbour lies outside the grid.
// Each array mirrors the CSR value array it was built from (src*): products
// and sweeps switch to the grid only when given that array.
struct Grid27 {
  int points = 27;  // 27 (parity colouring) or 7 (red-black colouring, block n / 2)
  int n0 = 0, n1 = 0, n2 = 0;
  int64_t n = 0, block = 0, stride = 0;
  DBuf<double> v64;
  DBuf<float> v32;
  DBuf<bf16> v16;
  const void *src64 = nullptr, *src32 = nullptr, *src16 = nullptr;
  // tensor maps of the float and FP64 values (CUtensorMaps, encoded on
  // first use)
  alignas(64) mutable unsigned char vmap32[128] = {};
  alignas(64) mutable unsigned char vmap64[128] = {};
  mutable const void *vmap32_key = nullptr, *vmap64_key = nullptr;
};

// Csr::tuned index of a value type
template <typename VT>
constexpr int tune_value_index() {
  return sizeof(VT) == 8 ? 0 : sizeof(VT) == 4 ? 1 : 2;
}

struct StencilDesc {
  int64_t dims[3];
  double q[3];
  double coeffs[4];
  double conn[48];
  double dfac[16];  // lookup: diffusion factor of materials a -> b at [4 a + b]
  double sol_start, sol_end;
  int zero_to_one;
  int lookup;
  int values;  // values valuator: a conductivity per cell and axis
  const uint8_t *mat;
  const double *k;
};

}  // namespace lgx

struct lgx_matrix {
  int kind = LGX_MATRIX_CSR;
  int64_t n = 0;
  int64_t nnz = 0;
  int symmetric = 1;
  lgx::Csr csr;                 // CSR kinds
  lgx::StencilDesc st{};        // stencil kinds
  lgx::DBuf<uint8_t> mat;       // stencil lookup materials (owned copy)
  lgx::DBuf<double> k;          // stencil value conductivities (owned copy)
  lgx::DBuf<double> diag;       // cached diagonal (lazily computed)
  lgx::DBuf<double> rdiag;      // stencil SOR: correctly rounded 1 / diagonal, 0 where the
                                // sweep divides directly (lazily computed)
  int64_t grid_dims[3] = {0, 0, 0};  // CSR kinds: grid operator on this grid
  int grid_points = 0;                // 27 or 7 points; 0: unknown
};

// Colour-permuted copy of a CSR matrix used by the multicolour smoothers.
// Row r' of the permuted matrix is row perm[r'] of the original; its entries
// keep the original column order (columns mapped through iperm) so that the
// row sums are formed in exactly the order of the original row.
struct lgx_colouring {
  int64_t n = 0;
  int32_t ncolours = 0;
  std::vector<int64_t> offsets;  // host: colour c occupies rows [offsets[c], offsets[c+1])
  lgx::DBuf<int32_t> colour;     // natural order
  lgx::DBuf<int32_t> perm;       // permuted -> natural
  lgx::DBuf<int32_t> iperm;      // natural -> permuted
  lgx::Csr pcsr;                 // permuted matrix (values in the source storage type)
  lgx::DBuf<float> pv32;         // float copy of the permuted values (float cycles)
  lgx::DBuf<lgx::bf16> pv16;     // bfloat16 values a_ij / a_ii (bf16 float cycles)
  lgx::DBuf<float> pscale;       // per-row scale of pv16: the diagonal a_ii
  lgx::DBuf<double> rdiag;       // FP64 values: 1 / a_rr correctly rounded, or 0 where
                                 // the SOR row must divide (permuted order)
  lgx::DBuf<double> pdiag;       // the stored diagonal a_rr, widened (permuted order)
  lgx::DBuf<double> work_b, work_x;  // natural<->permuted staging for the public sweep API
  bool stencil_rb = false;       // red-black colouring of a stencil matrix: the sweeps run
                                 // matrix-free in natural order (no permuted copy)
};

namespace lgx {

// ---- kernels exposed across translation units --------------------------
// Deterministic two-stage reductions.  `partials` needs reduce_blocks(n)
// doubles; `counter` one zero-initialised unsigned int.
constexpr int kReduceThreads = 256;
int reduce_blocks(int64_t n);

lgx_status csr_from_device(int64_t n, int64_t nnz, const int64_t *rowptr, const int32_t *col,
                           const double *val, int symmetric, lgx_dtype storage,
                           cudaStream_t s, Csr &out);
lgx_status csr_compute_max_row(Csr &a, cudaStream_t s);
// rows per tile of the warp-tile row engine; Csr::max_win is measured over
// windows of this many rows
constexpr int kWarpTileRows = 32;
// sets a.max_win from the row offsets (for matrices whose rows were permuted)
lgx_status csr_compute_max_window(Csr &a, cudaStream_t s);

// y = A x for CSR with value type VT and vector type XT (accumulation in XT)
template <typename VT, typename XT>
lgx_status csr_spmv(const Csr &a, const VT *val, const XT *x, XT *y, cudaStream_t s);
// r = b - A x; if norm != nullptr, norm[0] = ||r||^2 (double, deterministic)
// scale: per-row factor of bfloat16 values (value = scale[row] * stored)
template <typename VT, typename XT>
lgx_status csr_residual(const Csr &a, const VT *val, const XT *b, const XT *x, XT *r,
                        double *norm, double *partials, unsigned *counter, cudaStream_t s,
                        const float *scale = nullptr);

// grid rows without column indices (lgx_grid.cu): each runs when
// `a` carries a grid mirroring `val` (*done), else leaves the work to the
// CSR kernels
template <typename VT, typename XT>
lgx_status grid_spmv(const Csr &a, const VT *val, const XT *x, XT *y, cudaStream_t s, bool *done);
template <typename VT, typename XT>
lgx_status grid_residual(const Csr &a, const VT *val, const XT *b, const XT *x, XT *r,
                         const float *scale, cudaStream_t s, bool *done);
// r_out: the rows' residuals b - A x with their new x are written there as
// well (the last colour of a forward sweep; float values and vectors only)
template <typename VT, typename XT>
lgx_status grid_sor_rows(const Csr &a, const VT *val, int64_t rb, int64_t re, const XT *b, XT *x,
                         double relax, int ultra, const double *rdiag, int relax_one,
                         int from_zero, int64_t visit_end, const float *scale, cudaStream_t s,
                         bool *done, XT *r_out = nullptr);
// whether grid_sor_rows takes r_out on this matrix (7-point grid rows, float)
bool grid_sweep_residual(const Csr &a);
// the residual of rows [rb, re) only
template <typename VT, typename XT>
lgx_status grid_residual_rows(const Csr &a, const VT *val, const XT *b, const XT *x, XT *r,
                              int64_t rb, int64_t re, cudaStream_t s, bool *done);

lgx_status stencil_spmv(const StencilDesc &st, const double *x, double *y, cudaStream_t s);
lgx_status stencil_residual(const StencilDesc &st, const double *b, const double *x, double *r,
                            double *norm, double *partials, unsigned *counter, cudaStream_t s);
lgx_status stencil_diagonal(const StencilDesc &st, double *d, cudaStream_t s);
// red-black SOR sweep of a stencil matrix in natural order (lgx_spmv.cu)
lgx_status stencil_sor_sweep(const lgx_matrix *a, double relax, int forward, int ultra,
                             const double *x_in, double *x_out, const double *b, cudaStream_t s);
lgx_status matrix_diagonal(lgx_matrix *a, cudaStream_t s, const double **out);

// Generic matrix application for the Krylov drivers (CSR or stencil).
lgx_status matrix_spmv(const lgx_matrix *a, const double *x, double *y, cudaStream_t s);
lgx_status matrix_residual(const lgx_matrix *a, const double *b, const double *x, double *r,
                           double *norm, double *partials, unsigned *counter, cudaStream_t s);

lgx_status dot(int64_t n, const double *a, const double *b, double *out, double *partials,
               unsigned *counter, cudaStream_t s);

// colouring helpers
lgx_status colouring_build(const Csr &a, const int32_t *d_colour, int32_t ncolours,
                           cudaStream_t s, lgx_colouring &out);
lgx_status colouring_jp(const Csr &a, uint64_t seed, cudaStream_t s, DBuf<int32_t> &colour,
                        int32_t &ncolours);
// One multicolour sweep on the permuted matrix (vectors in permuted order,
// in place).  VT value type, XT vector/arithmetic type.
// from_zero: the sweep starts from x = 0 (x need not be cleared); scale: the
// per-row factor of bfloat16 values.  r_last / res_from (forward sweeps):
// when the last colour runs on float 7-point grid rows, its rows' residuals
// b - A x are written to r_last as well and *res_from is that colour's
// first row (else c.n): the caller's residual then needs rows
// [0, *res_from) only.
template <typename VT, typename XT>
lgx_status mc_sor_sweep(const lgx_colouring &c, const VT *val, double relax, int forward,
                        int ultra, const XT *b, XT *x, cudaStream_t s, int from_zero = 0,
                        const float *scale = nullptr, XT *r_last = nullptr,
                        int64_t *res_from = nullptr);
lgx_status colouring_make_bf16(lgx_colouring &c, cudaStream_t s);
// gives c.pcsr a Grid27 when it is the parity-coloured 27-point (points 27)
// or red-black 7-point (points 7) operator on `dims` (checked on the device;
// *attached tells whether it was)
lgx_status grid27_attach(lgx_colouring &c, const int64_t dims[3], int points, cudaStream_t s,
                         bool *attached);

lgx_status jacobi_csr(const Csr &a, double relax, const double *x_in, double *x_out,
                      const double *b, cudaStream_t s);
lgx_status jacobi_diag_zero(int64_t n, const double *d, double relax, const double *b, double *x,
                            cudaStream_t s);
lgx_status colouring_make_f32(lgx_colouring &c, cudaStream_t s);
lgx_status colouring_sweep_natural(lgx_colouring &c, double relax, int forward, int ultra,
                                   const double *x_in, double *x_out, const double *b,
                                   cudaStream_t s);

// permutation gathers
template <typename T, typename U>
lgx_status gather(int64_t n, const int32_t *idx, const T *src, U *dst, cudaStream_t s);
template <typename T, typename U>
lgx_status scatter(int64_t n, const int32_t *idx, const T *src, U *dst, cudaStream_t s);

inline unsigned grid_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

lgx_status inclusive_offsets(int64_t n, const int64_t *in, int64_t *out, cudaStream_t s);
lgx_status check_device_error(cudaStream_t s);
// allocates the column/value arrays of a CSR with the trailing padding that
// the staged row kernels rely on
lgx_status csr_alloc_arrays(Csr &a, int64_t nnz, lgx_dtype storage);
// partial-sum slots needed by the fused reductions of the row-block kernels
int64_t csr_partials(int64_t n);
int64_t matrix_partials(const lgx_matrix *a);
// faces (value kinds) and the cached diagonal; k1/k2: the axis-1/2
// conductivities of a values stencil, read by the first call only
lgx_status stencil_ensure(lgx_matrix *a, cudaStream_t s, const double *k1 = nullptr,
                          const double *k2 = nullptr);

// ---- programmatic dependent launch ---------------------------------------
// Kernels of the solve chains are launched with the programmatic-stream-
// serialization attribute: a kernel may be scheduled while its predecessor in
// the stream drains, runs its prologue (barrier set-up, bulk copies of the
// constant matrix data), and calls pdl_wait() before it touches anything the
// predecessor wrote; griddepcontrol.wait returns once the predecessor has
// completed and its memory is visible.  pdl_trigger() lets the successor be
// scheduled as soon as every CTA of this grid has started.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
// false when LGX_PDL=0 (plain stream ordering, for comparison)
bool pdl_enabled();
// FP64 row launches over at most this many rows also use programmatic
// dependent launch (small launches are latency-bound; large FP64 ones lose
// occupancy to the early-scheduled successor).  LGX_PDL_FP64_ROWS overrides.
int64_t pdl_fp64_rows();

// want: the caller's choice for this launch.  Measured at 256^3: the float
// V-cycle gains (mixed solve 382 -> 376 ms) while the FP64 chain, whose row
// kernels are FP64-pipe bound, loses (536 -> 550 ms); FP64 chains therefore
// launch without the attribute.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(bool want, void (*kernel)(KArgs...), dim3 grid, dim3 block,
                              size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = want && pdl_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// ---- device helpers ------------------------------------------------------
// a / d rounded to nearest from y = RN(1/d): q0 = a*y is within 1.5 ulp of
// a/d, one correction q1 = q0 + (a - d*q0)*y makes it faithful, and a second
// one with the then exact residual gives the correctly rounded quotient
// (P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990: a faithful quotient
// corrected once with the correctly rounded reciprocal rounds correctly).
// Five FP64 operations instead of a full division.  Valid while a and d stay
// within [2^-400, 2^400] in magnitude; the caller checks a, the reciprocal
// table marks d.
__device__ __forceinline__ double div_by_recip(double a, double d, double y) {
  const double q0 = a * y;
  const double r0 = fma(-d, q0, a);
  const double q1 = fma(r0, y, q0);
  const double r1 = fma(-d, q1, a);
  return fma(r1, y, q1);
}

// integer tests on the bit pattern, which keep these tests off the FP64
// pipe.  The bits leave through an asm move: written with plain integer
// arithmetic, the compiler recognises each test as a floating-point
// comparison (v != 0, |v| < 2^400, isfinite) and emits it on the FP64 pipe
// -- nine FP64 instructions per cell in the stencil SOR sweep (ncu opcode
// counts), where 12 are its arithmetic.
__device__ __forceinline__ void double_words(double v, unsigned &lo, unsigned &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(v));
}
__device__ __forceinline__ int exponent_field(double v) {
  unsigned lo, hi;
  double_words(v, lo, hi);
  return (int)((hi >> 20) & 0x7ffu);
}
__device__ __forceinline__ bool exponent_within_400(double v) {
  const int e = exponent_field(v);
  return e > 1023 - 400 && e < 1023 + 400;
}
__device__ __forceinline__ bool nonzero_bits(double v) {
  unsigned lo, hi;
  double_words(v, lo, hi);
  return ((hi << 1) | lo) != 0u;
}


template <int T>
__device__ __forceinline__ double block_sum(double v, double *sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
#pragma unroll
  for (int s = T / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Deterministic grid reduction.  Every block calls it with its threads'
// values; block `bid` of `nblocks` stores its (fixed-shape tree) sum in
// partials[bid]; the last block to arrive sums the partials in index order
// (fixed strided split + tree), stores the total in *total (thread 0) and
// re-arms the counter.  Returns true in that last block only.  Requires
// blockDim.x == T (a power of two).
template <int T>
__device__ __forceinline__ bool grid_reduce(double v, unsigned bid, unsigned nblocks,
                                            double *partials, unsigned *counter, double *total) {
  __shared__ double sh[T];
  __shared__ bool last;
  const double bs = block_sum<T>(v, sh);
  if (threadIdx.x == 0) {
    partials[bid] = bs;
    __threadfence();
    const unsigned done = atomicAdd(counter, 1u);
    last = (done == nblocks - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc = 0.0;
  for (unsigned b = threadIdx.x; b < nblocks; b += T) acc += ((volatile double *)partials)[b];
  const double t = block_sum<T>(acc, sh);
  if (threadIdx.x == 0) {
    *total = t;
    *counter = 0;
  }
  return true;
}

}  // namespace lgx
