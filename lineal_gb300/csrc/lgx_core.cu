// Core of the lineal_gb300 library: error reporting, matrix handles, CSR
// construction, synthetic operators, deterministic reductions and vector ops.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <memory>
#include <map>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "lgx_internal.cuh"

namespace lgx {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(uint64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

int sm_count() {
  static int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

// Row-engine configuration (see launch_rows).  FP64 SpMV / SOR sweep at
// 256^3 (27-point, 449M nnz), ms:
//   CTA tiles kind 0 1.55 / 2.63, kind 1 1.37 / 1.98, kind 2 1.45 / 2.33;
//   warp tiles 3: 1.08 / 1.69, 4: 1.38 / 2.48, 5: 1.16 / 1.80, 6: 1.37 / 2.30
// Default 3; LGX_ROWS_CONFIG or lgx_row_engine_set choose another.
static std::atomic<int> g_rows_config{[] {
  const char *e = std::getenv("LGX_ROWS_CONFIG");
  const int v = e ? std::atoi(e) : 3;
  return (v >= 0 && v <= 7) ? v : 3;
}()};

int rows_config() { return g_rows_config.load(std::memory_order_relaxed); }

bool pdl_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("LGX_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

int64_t pdl_fp64_rows() {
  static const int64_t rows = [] {
    const char *e = std::getenv("LGX_PDL_FP64_ROWS");
    return e ? (int64_t)std::atoll(e) : (int64_t)262144;
  }();
  return rows;
}

int *device_error_flag() {
  static int *p = [] {
    int *q = nullptr;
    if (cudaMalloc(&q, sizeof(int)) != cudaSuccess) return (int *)nullptr;
    cudaMemset(q, 0, sizeof(int));
    cudaDeviceSynchronize();
    return q;
  }();
  return p;
}

lgx_status check_device_error(cudaStream_t s) {
  int *p = device_error_flag();
  if (!p) return fail(LGX_ERR_NOMEM, "device error flag not allocated");
  int h = 0;
  LGX_CUDA(cudaMemcpyAsync(&h, p, sizeof(int), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  if (h) {
    LGX_CUDA(cudaMemsetAsync(p, 0, sizeof(int), s));
    return fail(LGX_ERR_CUDA, "a device wait on a shared-memory copy timed out");
  }
  return LGX_OK;
}

void set_error(const std::string &msg) { g_last_error = msg; }

lgx_status fail(lgx_status s, const std::string &msg) {
  g_last_error = msg;
  return s;
}

lgx_status cuda_fail(cudaError_t e, const char *what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? LGX_ERR_NOMEM : LGX_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// CSR construction
// ---------------------------------------------------------------------------
__global__ void k_f64_to_f32(int64_t n, const double *src, float *dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

__global__ void k_f32_to_f64(int64_t n, const float *src, double *dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

// validates sortedness / diagonal presence and records the longest row
__global__ void k_csr_check(int64_t n, int64_t nnz, const int64_t *rowptr, const int32_t *col,
                            unsigned long long *max_row, unsigned long long *max_win, int *bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = rowptr[i], e = rowptr[i + 1];
    if (b < 0 || e < b || e > nnz) {
      atomicOr(bad, 1);
      continue;
    }
    atomicMax(max_row, (unsigned long long)(e - b));
    const int64_t we = rowptr[i + kWarpTileRows < n ? i + kWarpTileRows : n];
    if (we >= b) atomicMax(max_win, (unsigned long long)(we - b));
    int has_diag = 0;
    for (int64_t k = b; k < e; ++k) {
      const int32_t c = col[k];
      if (c < 0 || c >= n) atomicOr(bad, 2);
      if (k > b && col[k - 1] >= c) atomicOr(bad, 4);
      has_diag |= (c == i);
    }
    if (!has_diag) atomicOr(bad, 8);
  }
}

lgx_status csr_from_device(int64_t n, int64_t nnz, const int64_t *rowptr, const int32_t *col,
                           const double *val, int symmetric, lgx_dtype storage, cudaStream_t s,
                           Csr &out) {
  if (n < 0 || nnz < 0 || n > INT32_MAX) return fail(LGX_ERR_INVALID, "invalid CSR sizes");
  out.n = n;
  out.nnz = nnz;
  out.symmetric = symmetric;
  out.storage = storage;
  LGX_CHECK(out.rowptr.alloc(n + 3));  // +2: staged row-offset spans
  LGX_CHECK(csr_alloc_arrays(out, nnz, storage));
  LGX_CUDA(cudaMemcpyAsync(out.rowptr.p, rowptr, sizeof(int64_t) * (n + 1),
                           cudaMemcpyDeviceToDevice, s));
  if (nnz) LGX_CUDA(cudaMemcpyAsync(out.col.p, col, sizeof(int32_t) * nnz,
                                    cudaMemcpyDeviceToDevice, s));
  if (storage == LGX_F64) {
    if (nnz) LGX_CUDA(cudaMemcpyAsync(out.v64.p, val, sizeof(double) * nnz,
                                      cudaMemcpyDeviceToDevice, s));
  } else {
    if (nnz) {
      k_f64_to_f32<<<std::min<int64_t>(grid_for(nnz, 256), 4096), 256, 0, s>>>(nnz, val,
                                                                               out.v32.p);
      LGX_LAUNCH_CHECK();
    }
  }
  return csr_compute_max_row(out, s);
}

lgx_status csr_alloc_arrays(Csr &a, int64_t nnz, lgx_dtype storage) {
  LGX_CHECK(a.col.alloc(nnz + kCsrPad));
  if (storage == LGX_F64) {
    LGX_CHECK(a.v64.alloc(nnz + kCsrPad));
  } else {
    LGX_CHECK(a.v32.alloc(nnz + kCsrPad));
  }
  return LGX_OK;
}

lgx_status csr_compute_max_row(Csr &a, cudaStream_t s) {
  DBuf<unsigned long long> mx;
  DBuf<int> bad;
  LGX_CHECK(mx.alloc(2));
  LGX_CHECK(bad.alloc(1));
  LGX_CUDA(cudaMemsetAsync(mx.p, 0, 2 * sizeof(unsigned long long), s));
  LGX_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  if (a.n) {
    k_csr_check<<<std::min<int64_t>(grid_for(a.n, 256), 4096), 256, 0, s>>>(
      a.n, a.nnz, a.rowptr.p, a.col.p, mx.p, mx.p + 1, bad.p);
    LGX_LAUNCH_CHECK();
  }
  unsigned long long h_mx[2] = {0, 0};
  int h_bad = 0;
  LGX_CUDA(cudaMemcpyAsync(h_mx, mx.p, sizeof(h_mx), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaMemcpyAsync(&h_bad, bad.p, sizeof(h_bad), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  if (h_bad & 1) return fail(LGX_ERR_INVALID, "CSR row offsets are not monotone");
  if (h_bad & 2) return fail(LGX_ERR_INVALID, "CSR column index out of range");
  if (h_bad & 4) return fail(LGX_ERR_INVALID, "CSR columns are not strictly ascending");
  if (h_bad & 8) return fail(LGX_ERR_INVALID, "CSR row without stored diagonal");
  a.max_row = (int64_t)h_mx[0];
  a.max_win = (int64_t)h_mx[1];
  return LGX_OK;
}

// the block's maximum first, one atomic per block (one per row on a single
// address serialised 16.8M atomics at 256^3: 8 ms)
__global__ void __launch_bounds__(256) k_csr_window(int64_t n, const int64_t *rowptr,
                                                    unsigned long long *max_win) {
  __shared__ unsigned long long part[8];
  unsigned long long m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = rowptr[i];
    const int64_t we = rowptr[i + kWarpTileRows < n ? i + kWarpTileRows : n];
    m = (unsigned long long)(we - b) > m ? (unsigned long long)(we - b) : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long q = __shfl_xor_sync(0xffffffffu, m, o);
    m = q > m ? q : m;
  }
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = part[w] > m ? part[w] : m;
    atomicMax(max_win, m);
  }
}

lgx_status csr_compute_max_window(Csr &a, cudaStream_t s) {
  DBuf<unsigned long long> mx;
  LGX_CHECK(mx.alloc(1));
  LGX_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), s));
  if (a.n) {
    k_csr_window<<<std::min<int64_t>(grid_for(a.n, 256), 4096), 256, 0, s>>>(a.n, a.rowptr.p,
                                                                              mx.p);
    LGX_LAUNCH_CHECK();
  }
  unsigned long long h = 0;
  LGX_CUDA(cudaMemcpyAsync(&h, mx.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  a.max_win = (int64_t)h;
  return LGX_OK;
}

// ---------------------------------------------------------------------------
// Deterministic reductions: every block reduces a fixed strided subset, the
// last block to finish sums the per-block partials in index order.
// ---------------------------------------------------------------------------
int reduce_blocks(int64_t n) {
  int64_t b = (n + kReduceThreads * 8 - 1) / (kReduceThreads * 8);
  if (b < 1) b = 1;
  if (b > 1216) b = 1216;
  return (int)b;
}

__device__ __forceinline__ bool finish_reduction(double v, double *partials, unsigned *counter,
                                                 double *total) {
  return grid_reduce<kReduceThreads>(v, blockIdx.x, gridDim.x, partials, counter, total);
}

__global__ void k_dot(int64_t n, const double *a, const double *b, double *out, double *partials,
                      unsigned *counter) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s = fma(a[i], b[i], s);
  double t;
  if (finish_reduction(s, partials, counter, &t) && threadIdx.x == 0) out[0] = t;
}

__global__ void k_maxabs(int64_t n, const double *a, double *out, double *partials,
                         unsigned *counter) {
  __shared__ double sh[kReduceThreads];
  __shared__ bool last;
  double m = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    m = fmax(m, fabs(a[i]));
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int s = kReduceThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = sh[0];
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double r = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) r = fmax(r, ((volatile double *)partials)[b]);
    out[0] = r;
    *counter = 0;
  }
}

lgx_status dot(int64_t n, const double *a, const double *b, double *out, double *partials,
               unsigned *counter, cudaStream_t s) {
  k_dot<<<reduce_blocks(n), kReduceThreads, 0, s>>>(n, a, b, out, partials, counter);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

// Scratch of the public reductions (lgx_dot, lgx_norm2sq, lgx_max_norm): one
// set per stream, allocated on the stream's first call and kept for the life
// of the process (1216 partial sums and an arrival counter, 9.7 KB), so that
// later calls neither allocate nor free -- cudaFree waits for the whole
// device.  Calls on one stream run in order and share its set; the last block
// of every completed reduction leaves the counter at zero.  Streams are told
// apart by device and stream id (cudaStreamGetId: ids are not reused while
// the process runs), so two streams never share a set.
struct ReduceScratch {
  DBuf<double> partials;
  DBuf<unsigned> counter;
};
static std::mutex g_reduce_scratch_mutex;
static std::map<std::pair<int, unsigned long long>, std::unique_ptr<ReduceScratch>>
  g_reduce_scratch;

static lgx_status reduce_scratch(cudaStream_t s, ReduceScratch **out) {
  int dev = 0;
  LGX_CUDA(cudaGetDevice(&dev));
  unsigned long long id = 0;
  LGX_CUDA(cudaStreamGetId(s, &id));
  std::lock_guard<std::mutex> lock(g_reduce_scratch_mutex);
  auto &slot = g_reduce_scratch[{dev, id}];
  if (!slot) {
    auto rs = std::make_unique<ReduceScratch>();
    LGX_CHECK(rs->partials.alloc(reduce_blocks(INT64_MAX)));
    LGX_CHECK(rs->counter.alloc(1));
    LGX_CUDA(cudaMemsetAsync(rs->counter.p, 0, sizeof(unsigned), s));
    slot = std::move(rs);
  }
  *out = slot.get();
  return LGX_OK;
}

// Scratch of lgx_dot_static: one partial sum per block of k_dot and the
// block-arrival counter, in the module's static device memory (8 KB + 8 B).
// The counter must be zero when a call starts: static device memory is
// zero-initialised when the module loads, and every completed k_dot leaves
// its counter at zero again (the last block resets it).
constexpr int kDotStaticPartials = 1024;
struct DotStaticScratch {
  double partials[kDotStaticPartials];
  unsigned counter;
};
static __device__ __align__(256) DotStaticScratch g_dot_static_scratch;

// Device address of g_dot_static_scratch, looked up once per device (with
// that device current) on the first lgx_dot_static call there.
constexpr int kDotStaticMaxDevices = 64;
static std::mutex g_dot_static_mutex;
static DotStaticScratch *g_dot_static_ptr[kDotStaticMaxDevices] = {};

static lgx_status dot_static_scratch(DotStaticScratch **out) {
  int dev = 0;
  LGX_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kDotStaticMaxDevices)
    return fail(LGX_ERR_UNSUPPORTED, "lgx_dot_static: device ordinal " + std::to_string(dev) +
                                       " beyond the " + std::to_string(kDotStaticMaxDevices) +
                                       " devices it keeps scratch addresses for");
  std::lock_guard<std::mutex> lock(g_dot_static_mutex);
  if (!g_dot_static_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_dot_static_scratch);
    if (e != cudaSuccess)
      return fail(LGX_ERR_CUDA, std::string("lgx_dot_static: cudaGetSymbolAddress failed: ") +
                                  cudaGetErrorString(e));
    g_dot_static_ptr[dev] = static_cast<DotStaticScratch *>(p);
  }
  *out = g_dot_static_ptr[dev];
  return LGX_OK;
}

__global__ void k_axpy(int64_t n, double alpha, const double *x, double *y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = fma(x[i], alpha, y[i]);
}

// out = alpha x + beta y with the products and the sum rounded one by one
// (no contraction into an fma): the rounding of lineal's expression trees
// add / subtract / scale (component-wise/vector-expression.hpp:67-91)
__global__ void k_lincomb(int64_t n, double alpha, const double *x, double beta, const double *y,
                          double *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double ax = __dmul_rn(alpha, x[i]);
    out[i] = y ? __dadd_rn(ax, __dmul_rn(beta, y[i])) : ax;
  }
}

__global__ void k_fill(int64_t n, double value, double *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = value;
}

template <typename T, typename U>
__global__ void k_gather(int64_t n, const int32_t *idx, const T *src, U *dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (U)src[idx[i]];
}
template <typename T, typename U>
__global__ void k_scatter(int64_t n, const int32_t *idx, const T *src, U *dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[idx[i]] = (U)src[i];
}

template <typename T, typename U>
lgx_status gather(int64_t n, const int32_t *idx, const T *src, U *dst, cudaStream_t s) {
  if (n == 0) return LGX_OK;
  k_gather<T, U><<<std::min<int64_t>(grid_for(n, 256), 8192), 256, 0, s>>>(n, idx, src, dst);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}
template <typename T, typename U>
lgx_status scatter(int64_t n, const int32_t *idx, const T *src, U *dst, cudaStream_t s) {
  if (n == 0) return LGX_OK;
  k_scatter<T, U><<<std::min<int64_t>(grid_for(n, 256), 8192), 256, 0, s>>>(n, idx, src, dst);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}
template lgx_status gather<double, double>(int64_t, const int32_t *, const double *, double *,
                                           cudaStream_t);
template lgx_status gather<double, float>(int64_t, const int32_t *, const double *, float *,
                                          cudaStream_t);
template lgx_status scatter<double, double>(int64_t, const int32_t *, const double *, double *,
                                            cudaStream_t);
template lgx_status scatter<float, double>(int64_t, const int32_t *, const float *, double *,
                                           cudaStream_t);
template lgx_status gather<float, float>(int64_t, const int32_t *, const float *, float *,
                                        cudaStream_t);

// ---------------------------------------------------------------------------
// Synthetic structured operators (7- and 27-point).  The arithmetic uses
// explicitly rounded operations so that no multiply-add is contracted and the
// values equal a plain IEEE evaluation on the host.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double hmean(double a, double b) {
  const double p = __dmul_rn(a, b);
  return p != 0.0 ? __ddiv_rn(__dadd_rn(p, p), __dadd_rn(a, b)) : 0.0;
}

__global__ void k_gen_count(int64_t n0, int64_t n1, int64_t n2, int npts, int64_t *rowlen) {
  const int64_t n = n0 * n1 * n2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p0 = i / (n1 * n2), p1 = (i / n2) % n1, p2 = i % n2;
    const int64_t c0 = 1 + (p0 > 0) + (p0 + 1 < n0);
    const int64_t c1 = 1 + (p1 > 0) + (p1 + 1 < n1);
    const int64_t c2 = 1 + (p2 > 0) + (p2 + 1 < n2);
    if (npts == 27) {
      rowlen[i] = c0 * c1 * c2;
    } else {
      rowlen[i] = 1 + (c0 - 1) + (c1 - 1) + (c2 - 1);
    }
  }
}

__global__ void k_gen_fill(int64_t n0, int64_t n1, int64_t n2, int npts, const double *k,
                           const int64_t *rowptr, int32_t *col, double *val) {
  const int64_t n = n0 * n1 * n2;
  const double w[4] = {0.0, 1.0, 0.5, 0.25};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p0 = i / (n1 * n2), p1 = (i / n2) % n1, p2 = i % n2;
    int64_t pos = rowptr[i];
    const double ki = k[i];
    double diag = 0.0;
    if (p0 == 0) diag = __dadd_rn(diag, __dmul_rn(2.0, ki));
    if (p0 + 1 == n0) diag = __dadd_rn(diag, __dmul_rn(2.0, ki));
    int64_t dpos = -1;
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b)
        for (int c = -1; c <= 1; ++c) {
          const int m = abs(a) + abs(b) + abs(c);
          if (npts == 7 && m > 1) continue;
          if (p0 + a < 0 || p0 + a >= n0 || p1 + b < 0 || p1 + b >= n1 || p2 + c < 0 ||
              p2 + c >= n2)
            continue;
          const int64_t j = i + a * n1 * n2 + b * n2 + c;
          col[pos] = (int32_t)j;
          if (m == 0) {
            dpos = pos;
            val[pos] = 0.0;
          } else {
            const double cc = __dmul_rn(hmean(ki, k[j]), w[m]);
            val[pos] = -cc;
            diag = __dadd_rn(diag, cc);
          }
          ++pos;
        }
    if (diag == 0.0) diag = 1.0;
    val[dpos] = diag;
  }
}

__global__ void k_scan_block(int64_t n, const int64_t *in, int64_t *out, int64_t *block_sums) {
  // exclusive scan of `in` into out[1..n] (out[0] = 0) in chunks of 1024
  __shared__ int64_t sh[1024];
  const int64_t base = (int64_t)blockIdx.x * 1024;
  const int64_t i = base + threadIdx.x;
  sh[threadIdx.x] = i < n ? in[i] : 0;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int64_t t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i + 1] = sh[threadIdx.x];
  if (threadIdx.x == 1023) block_sums[blockIdx.x] = sh[1023];
}

__global__ void k_scan_add(int64_t n, int64_t *out, const int64_t *block_offsets) {
  const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i + 1] += block_offsets[blockIdx.x];
  if (i == 0) out[0] = 0;
}

// out[0] = 0, out[i+1] = sum_{j<=i} in[j]; recursive over chunks of 1024.
lgx_status inclusive_offsets(int64_t n, const int64_t *in, int64_t *out, cudaStream_t s) {
  if (n == 0) {
    LGX_CUDA(cudaMemsetAsync(out, 0, sizeof(int64_t), s));
    return LGX_OK;
  }
  const int64_t nb = (n + 1023) / 1024;
  DBuf<int64_t> bs, bo;
  LGX_CHECK(bs.alloc(nb));
  LGX_CHECK(bo.alloc(nb + 1));
  k_scan_block<<<(unsigned)nb, 1024, 0, s>>>(n, in, out, bs.p);
  LGX_LAUNCH_CHECK();
  if (nb > 1) {
    LGX_CHECK(inclusive_offsets(nb, bs.p, bo.p, s));
  } else {
    LGX_CUDA(cudaMemsetAsync(bo.p, 0, sizeof(int64_t), s));
  }
  k_scan_add<<<(unsigned)nb, 1024, 0, s>>>(n, out, bo.p);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

static lgx_status gen_structured(const int64_t dims[3], const double *d_k, int npts,
                                 lgx_dtype storage, cudaStream_t s, lgx_matrix **out) {
  if (!dims || !d_k || !out) return fail(LGX_ERR_INVALID, "null argument");
  const int64_t n = dims[0] * dims[1] * dims[2];
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1 || n > INT32_MAX)
    return fail(LGX_ERR_INVALID, "invalid grid dimensions");
  DBuf<int64_t> rowlen, rowptr;
  LGX_CHECK(rowlen.alloc(n));
  LGX_CHECK(rowptr.alloc(n + 3));  // +2: staged row-offset spans
  const unsigned g = (unsigned)std::min<int64_t>(grid_for(n, 256), 65535);
  k_gen_count<<<g, 256, 0, s>>>(dims[0], dims[1], dims[2], npts, rowlen.p);
  LGX_LAUNCH_CHECK();
  LGX_CHECK(inclusive_offsets(n, rowlen.p, rowptr.p, s));
  int64_t nnz = 0;
  LGX_CUDA(cudaMemcpyAsync(&nnz, rowptr.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  rowlen.release();
  auto *m = new lgx_matrix();
  m->kind = LGX_MATRIX_CSR;
  m->n = n;
  m->nnz = nnz;
  m->symmetric = 1;
  Csr &c = m->csr;
  c.n = n;
  c.nnz = nnz;
  c.symmetric = 1;
  c.storage = storage;
  c.rowptr = std::move(rowptr);
  lgx_status st = c.col.alloc(nnz + kCsrPad);
  DBuf<double> v64;
  if (st == LGX_OK) st = v64.alloc(nnz + kCsrPad);
  if (st != LGX_OK) {
    delete m;
    return st;
  }
  k_gen_fill<<<g, 256, 0, s>>>(dims[0], dims[1], dims[2], npts, d_k, c.rowptr.p, c.col.p, v64.p);
  if (cudaError_t e = cudaGetLastError(); e != cudaSuccess) {
    delete m;
    return cuda_fail(e, "k_gen_fill");
  }
  if (storage == LGX_F64) {
    c.v64 = std::move(v64);
  } else {
    st = c.v32.alloc(nnz + kCsrPad);
    if (st != LGX_OK) {
      delete m;
      return st;
    }
    k_f64_to_f32<<<4096, 256, 0, s>>>(nnz, v64.p, c.v32.p);
    cudaStreamSynchronize(s);
  }
  c.max_row = npts;
  c.max_win = (int64_t)npts * kWarpTileRows;
  *out = m;
  return LGX_OK;
}

}  // namespace lgx

using namespace lgx;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *lgx_status_string(lgx_status s) {
  switch (s) {
    case LGX_OK: return "ok";
    case LGX_ERR_INVALID: return "invalid argument";
    case LGX_ERR_CUDA: return "CUDA error";
    case LGX_ERR_NOMEM: return "out of device memory";
    case LGX_ERR_BREAKDOWN: return "Krylov breakdown";
    case LGX_ERR_NONFINITE: return "non-finite value";
    case LGX_ERR_NOT_SPD: return "matrix not positive definite";
    case LGX_ERR_UNSUPPORTED: return "unsupported operation";
    case LGX_ERR_NOT_CONVERGED: return "not converged";
  }
  return "unknown status";
}

const char *lgx_last_error(void) { return g_last_error.c_str(); }

const char *lgx_version(void) { return "lineal_gb300 0.1 (sm_103a)"; }

uint64_t lgx_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

lgx_status lgx_csr_create(int64_t n, int64_t nnz, const int64_t *d_rowptr, const int32_t *d_col,
                          const double *d_val, int symmetric, lgx_dtype storage,
                          lgx_stream stream, lgx_matrix **out) {
  if (!out || (n > 0 && (!d_rowptr || (nnz > 0 && (!d_col || !d_val)))))
    return fail(LGX_ERR_INVALID, "null argument");
  auto *m = new lgx_matrix();
  m->kind = LGX_MATRIX_CSR;
  m->n = n;
  m->nnz = nnz;
  m->symmetric = symmetric;
  lgx_status st =
    csr_from_device(n, nnz, d_rowptr, d_col, d_val, symmetric, storage, stream, m->csr);
  if (st != LGX_OK) {
    delete m;
    return st;
  }
  *out = m;
  return LGX_OK;
}

lgx_status lgx_csr_create_host(int64_t n, int64_t nnz, const int64_t *h_rowptr,
                               const int32_t *h_col, const double *h_val, int symmetric,
                               lgx_dtype storage, lgx_matrix **out) {
  if (!out || (n > 0 && !h_rowptr) || (nnz > 0 && (!h_col || !h_val)))
    return fail(LGX_ERR_INVALID, "null argument");
  DBuf<int64_t> rp;
  DBuf<int32_t> c;
  DBuf<double> v;
  LGX_CHECK(rp.alloc(n + 1));
  LGX_CHECK(c.alloc(nnz));
  LGX_CHECK(v.alloc(nnz));
  LGX_CUDA(cudaMemcpy(rp.p, h_rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
  if (nnz) {
    LGX_CUDA(cudaMemcpy(c.p, h_col, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice));
    LGX_CUDA(cudaMemcpy(v.p, h_val, sizeof(double) * nnz, cudaMemcpyHostToDevice));
  }
  return lgx_csr_create(n, nnz, rp.p, c.p, v.p, symmetric, storage, nullptr, out);
}

lgx_status lgx_csr_download(const lgx_matrix *a, int64_t *h_rowptr, int32_t *h_col,
                            double *h_val, lgx_stream stream) {
  if (!a || a->kind != LGX_MATRIX_CSR) return fail(LGX_ERR_INVALID, "not a CSR matrix");
  const Csr &c = a->csr;
  if (h_rowptr)
    LGX_CUDA(cudaMemcpyAsync(h_rowptr, c.rowptr.p, sizeof(int64_t) * (c.n + 1),
                             cudaMemcpyDeviceToHost, stream));
  if (h_col && c.nnz)
    LGX_CUDA(cudaMemcpyAsync(h_col, c.col.p, sizeof(int32_t) * c.nnz, cudaMemcpyDeviceToHost,
                             stream));
  if (h_val && c.nnz) {
    if (c.storage == LGX_F64) {
      LGX_CUDA(cudaMemcpyAsync(h_val, c.v64.p, sizeof(double) * c.nnz, cudaMemcpyDeviceToHost,
                               stream));
    } else {
      DBuf<double> tmp;
      LGX_CHECK(tmp.alloc(c.nnz));
      k_f32_to_f64<<<4096, 256, 0, stream>>>(c.nnz, c.v32.p, tmp.p);
      LGX_LAUNCH_CHECK();
      LGX_CUDA(cudaMemcpyAsync(h_val, tmp.p, sizeof(double) * c.nnz, cudaMemcpyDeviceToHost,
                               stream));
      LGX_CUDA(cudaStreamSynchronize(stream));
    }
  }
  LGX_CUDA(cudaStreamSynchronize(stream));
  return LGX_OK;
}

lgx_status lgx_matrix_destroy(lgx_matrix *a) {
  delete a;
  return LGX_OK;
}

lgx_status lgx_matrix_info(const lgx_matrix *a, int *kind, int64_t *n, int64_t *nnz,
                           int *symmetric) {
  if (!a) return fail(LGX_ERR_INVALID, "null matrix");
  if (kind) *kind = a->kind;
  if (n) *n = a->n;
  if (nnz) *nnz = a->nnz;
  if (symmetric) *symmetric = a->symmetric;
  return LGX_OK;
}

lgx_status lgx_gen_27pt(const int64_t dims[3], const double *d_k, lgx_dtype storage,
                        lgx_stream stream, lgx_matrix **out) {
  LGX_CHECK(gen_structured(dims, d_k, 27, storage, stream, out));
  for (int d = 0; d < 3; ++d) (*out)->grid_dims[d] = dims[d];
  (*out)->grid_points = 27;
  return LGX_OK;
}

static lgx_status csr_set_grid(lgx_matrix *a, const int64_t dims[3], int points) {
  if (!a || !dims) return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind != LGX_MATRIX_CSR) return fail(LGX_ERR_INVALID, "not a CSR matrix");
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1 || dims[0] * dims[1] * dims[2] != a->n)
    return fail(LGX_ERR_INVALID, "grid does not have one cell per row");
  for (int d = 0; d < 3; ++d) a->grid_dims[d] = dims[d];
  a->grid_points = points;
  return LGX_OK;
}

lgx_status lgx_csr_set_grid27(lgx_matrix *a, const int64_t dims[3]) {
  return csr_set_grid(a, dims, 27);
}

lgx_status lgx_csr_set_grid7(lgx_matrix *a, const int64_t dims[3]) {
  return csr_set_grid(a, dims, 7);
}

lgx_status lgx_gen_7pt(const int64_t dims[3], const double *d_k, lgx_dtype storage,
                       lgx_stream stream, lgx_matrix **out) {
  LGX_CHECK(gen_structured(dims, d_k, 7, storage, stream, out));
  for (int d = 0; d < 3; ++d) (*out)->grid_dims[d] = dims[d];
  (*out)->grid_points = 7;
  return LGX_OK;
}

lgx_status lgx_dot(int64_t n, const double *d_a, const double *d_b, double *d_out,
                   lgx_stream stream) {
  if (n < 0 || (n > 0 && (!d_a || !d_b)) || !d_out) return fail(LGX_ERR_INVALID, "bad argument");
  ReduceScratch *rs = nullptr;
  LGX_CHECK(reduce_scratch(stream, &rs));
  LGX_CHECK(dot(n, d_a, d_b, d_out, rs->partials.p, rs->counter.p, stream));
  LGX_CUDA(cudaStreamSynchronize(stream));
  return LGX_OK;
}

lgx_status lgx_row_engine_set(int config) {
  if (config < 0 || config > 7)
    return fail(LGX_ERR_INVALID, "row engine configuration must be in [0, 7]");
  g_rows_config.store(config, std::memory_order_relaxed);
  return LGX_OK;
}

int lgx_row_engine_get(void) { return rows_config(); }

lgx_status lgx_dot_static(int64_t n, const double *d_a, const double *d_b, double *d_out,
                          lgx_stream stream) {
  if (n < 0 || (n > 0 && (!d_a || !d_b)) || !d_out) return fail(LGX_ERR_INVALID, "bad argument");
  // same grid as lgx_dot (so the same result); its partial sums must fit the
  // static scratch
  if (reduce_blocks(n) > kDotStaticPartials)
    return fail(LGX_ERR_INVALID,
                "lgx_dot_static: n = " + std::to_string(n) + " exceeds the maximum of " +
                  std::to_string((int64_t)kDotStaticPartials * kReduceThreads * 8) +
                  " elements its static scratch holds; use lgx_dot");
  DotStaticScratch *sc = nullptr;
  LGX_CHECK(dot_static_scratch(&sc));
  return dot(n, d_a, d_b, d_out, sc->partials, &sc->counter, stream);
}

lgx_status lgx_norm2sq(int64_t n, const double *d_a, double *d_out, lgx_stream stream) {
  return lgx_dot(n, d_a, d_a, d_out, stream);
}

lgx_status lgx_max_norm(int64_t n, const double *d_a, double *d_out, lgx_stream stream) {
  if (n < 0 || (n > 0 && !d_a) || !d_out) return fail(LGX_ERR_INVALID, "bad argument");
  ReduceScratch *rs = nullptr;
  LGX_CHECK(reduce_scratch(stream, &rs));
  k_maxabs<<<reduce_blocks(n), kReduceThreads, 0, stream>>>(n, d_a, d_out, rs->partials.p,
                                                             rs->counter.p);
  LGX_LAUNCH_CHECK();
  LGX_CUDA(cudaStreamSynchronize(stream));
  return LGX_OK;
}

lgx_status lgx_axpy(int64_t n, double alpha, const double *d_x, double *d_y, lgx_stream stream) {
  if (n < 0 || (n > 0 && (!d_x || !d_y))) return fail(LGX_ERR_INVALID, "bad argument");
  if (n == 0) return LGX_OK;
  k_axpy<<<std::min<int64_t>(grid_for(n, 256), 8192), 256, 0, stream>>>(n, alpha, d_x, d_y);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

lgx_status lgx_lincomb(int64_t n, double alpha, const double *d_x, double beta,
                       const double *d_y, double *d_out, lgx_stream stream) {
  if (n < 0 || (n > 0 && (!d_x || !d_out))) return fail(LGX_ERR_INVALID, "bad argument");
  if (n == 0) return LGX_OK;
  k_lincomb<<<std::min<int64_t>(grid_for(n, 256), 8192), 256, 0, stream>>>(n, alpha, d_x, beta,
                                                                           d_y, d_out);
  LGX_LAUNCH_CHECK();
  count_launch();
  return LGX_OK;
}

lgx_status lgx_fill(int64_t n, double value, double *d_out, lgx_stream stream) {
  if (n < 0 || (n > 0 && !d_out)) return fail(LGX_ERR_INVALID, "bad argument");
  if (n == 0) return LGX_OK;
  k_fill<<<std::min<int64_t>(grid_for(n, 256), 8192), 256, 0, stream>>>(n, value, d_out);
  LGX_LAUNCH_CHECK();
  count_launch();
  return LGX_OK;
}

}  // extern "C"
