// Persistent CSR row engine with TMA bulk staging.
//
// A CSR tile of R consecutive rows owns one contiguous segment of the column
// and value arrays.  Each CTA walks its tiles (t = blockIdx.x, +gridDim.x, ...)
// with two shared-memory stages: while the threads compute tile j from stage
// j&1 (one thread per row, the row's products in storage order), thread 0 has
// already issued the bulk copies (cp.async.bulk global->shared, completion
// counted on an mbarrier) of tile j+1 into the other stage.  The copies are
// whole 16-byte-aligned spans, so the segment's first entry sits at a small
// offset inside the stage.  Column and value buffers of every CSR in this
// library carry kCsrPad trailing elements, so the aligned span never leaves
// the allocation.
//
// Every wait on an mbarrier is bounded (about one second of SM clock); on
// timeout the kernel records an error in the library's device error flag,
// waits once more (bounded) for its own copies and returns.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "lgx_internal.cuh"

namespace lgx {

constexpr int kTileRows = 256;     // threads per CTA, maximum rows per tile

template <typename VT>
struct TileCap {
  // entries per stage: 2 stages x (4 + sizeof(VT)) bytes x CAP <= 208 KB
  static constexpr int value = sizeof(VT) == 8 ? 8192 : 12288;
};

// per stage: row offsets (kTileRows + 4) * 8 bytes, columns (CAP + 8) * 4
// bytes, values (CAP + 8) * sizeof(VT) bytes (an aligned span exceeds its
// segment by at most 6 elements); then per stage a bounds record and a barrier
template <typename VT>
__host__ __device__ constexpr size_t stage_bytes() {
  return (size_t)(kTileRows + 4) * 8 + (size_t)(TileCap<VT>::value + 8) * 4 +
         (size_t)(TileCap<VT>::value + 8) * sizeof(VT);
}
template <typename VT>
__host__ __device__ constexpr size_t tile_smem_bytes() {
  return 2 * stage_bytes<VT>() + 2 * 32 + 64;
}

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         uint64_t *bar) {
  asm volatile(
    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
      "r"(smem_u32(dst)),
    "l"(src), "r"(bytes), "r"(smem_u32(bar))
    : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned phase) {
  unsigned ok;
  asm volatile(
    "{\n\t.reg .pred p;\n\t"
    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
    "selp.u32 %0, 1, 0, p;\n\t}"
    : "=r"(ok)
    : "r"(smem_u32(bar)), "r"(phase)
    : "memory");
  return ok != 0;
}

// bounded wait: true when the phase completed
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned phase) {
  const long long start = clock64();
  while (!mbar_try_wait(bar, phase)) {
    if (clock64() - start > (1ll << 31)) return false;
  }
  return true;
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

template <typename VT>
struct Stage {
  int64_t *rp;   // kTileRows + 4 row offsets, 16-byte aligned
  int32_t *col;  // CAP + 8 entries, 16-byte aligned
  VT *val;       // CAP + 8 entries, 16-byte aligned
};

// What thread 0 knows about a tile when it issues its copies; read by the
// other threads after the barrier that follows the issue.
struct TileRec {
  int64_t r0, r1, e0, e1;
};

// Issue the bulk copies of tile rows [r0, r1): row offsets r0..r1 and the
// segment [e0, e1) of columns and values, each as a 16-byte-aligned span.
template <typename VT>
__device__ __forceinline__ void issue_tile(const int64_t *rowptr, const int32_t *col,
                                           const VT *val, const TileRec &t, Stage<VT> st,
                                           uint64_t *bar) {
  constexpr int64_t CA = 16 / 4, VA = 16 / (int64_t)sizeof(VT);
  const int64_t p0 = t.r0 & ~1ll, p1 = (t.r1 + 2) & ~1ll;
  const int64_t c0 = t.e0 & ~(CA - 1), c1 = (t.e1 + CA - 1) & ~(CA - 1);
  const int64_t v0 = t.e0 & ~(VA - 1), v1 = (t.e1 + VA - 1) & ~(VA - 1);
  const unsigned pb = (unsigned)((p1 - p0) * 8), cb = (unsigned)((c1 - c0) * 4),
                 vb = (unsigned)((v1 - v0) * sizeof(VT));
  fence_proxy_async();
  mbar_expect_tx(bar, pb + cb + vb);
  bulk_g2s(st.rp, rowptr + p0, pb, bar);
  if (cb) bulk_g2s(st.col, col + c0, cb, bar);
  if (vb) bulk_g2s(st.val, val + v0, vb, bar);
}

// Op interface:
//   __device__ double row(int64_t row, const int32_t *c, const VT *v, int len) const;
//     (returns the row's contribution to an optional sum)
//   static constexpr bool kReduce;  __device__ void finish(double total) const;
//   double *partials; unsigned *counter;  (when kReduce)
template <typename VT, class Op>
__global__ void __launch_bounds__(kTileRows)
  k_rows(int64_t rb, int64_t re, int rows_per_tile, const int64_t *__restrict__ rowptr,
         const int32_t *__restrict__ col, const VT *__restrict__ val, Op op, int *err) {
  constexpr int CAP = TileCap<VT>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  static_assert((CAP + 8) * 4 % 16 == 0 && (CAP + 8) * sizeof(VT) % 16 == 0);
  // stage s starts at smem_raw + s * stage_bytes (computed, not indexed, so
  // the pointers stay in registers)
  auto stage = [&](int s) {
    unsigned char *p = smem_raw + (size_t)s * stage_bytes<VT>();
    Stage<VT> r;
    r.rp = reinterpret_cast<int64_t *>(p);
    r.col = reinterpret_cast<int32_t *>(p + (size_t)(kTileRows + 4) * 8);
    r.val = reinterpret_cast<VT *>(p + (size_t)(kTileRows + 4) * 8 + (size_t)(CAP + 8) * 4);
    return r;
  };
  TileRec *rec = reinterpret_cast<TileRec *>(smem_raw + 2 * stage_bytes<VT>());
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + 2 * stage_bytes<VT>() + 2 * 32);
  const int64_t nrows = re - rb;
  const int64_t ntiles = (nrows + rows_per_tile - 1) / rows_per_tile;
  const int64_t G = gridDim.x;

  auto bounds = [&](int64_t t) {
    TileRec r;
    r.r0 = rb + t * rows_per_tile;
    r.r1 = min(r.r0 + rows_per_tile, re);
    r.e0 = rowptr[r.r0];
    r.e1 = rowptr[r.r1];
    return r;
  };

  // thread 0 = producer: issues tile t+G while tile t is computed, and loads
  // the bounds of tile t+2G one iteration ahead of their use
  TileRec ahead{};
  int64_t t = blockIdx.x;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    if (t < ntiles) {
      rec[0] = bounds(t);
      if (rec[0].e1 - rec[0].e0 <= CAP)
        issue_tile<VT>(rowptr, col, val, rec[0], stage(0), &bar[0]);
    }
    if (t + G < ntiles) ahead = bounds(t + G);
  }
  __syncthreads();

  unsigned phase[2] = {0u, 0u};
  double contrib = 0.0;
  bool ok = true;
  for (int64_t j = 0; t < ntiles; ++j, t += G) {
    const int s = (int)(j & 1);
    if (threadIdx.x == 0 && t + G < ntiles) {
      (s ? rec[0] : rec[1]) = ahead;
      if (ahead.e1 - ahead.e0 <= CAP)
        issue_tile<VT>(rowptr, col, val, ahead, stage(s ^ 1), &bar[s ^ 1]);
      if (t + 2 * G < ntiles) ahead = bounds(t + 2 * G);
    }
    const TileRec cur = s ? rec[1] : rec[0];
    const int64_t row = cur.r0 + threadIdx.x;
    if (cur.e1 - cur.e0 <= CAP) {
      const bool waited = mbar_wait_bounded(&bar[s], phase[s]);
      // uniform decision: every thread leaves the loop if any wait gave up
      if (__syncthreads_or(!waited)) {
        ok = false;
        break;
      }
      phase[s] ^= 1u;
      constexpr int64_t CA = 4, VA = 16 / (int64_t)sizeof(VT);
      const int64_t p0 = cur.r0 & ~1ll, c0 = cur.e0 & ~(CA - 1), v0 = cur.e0 & ~(VA - 1);
      if (row < cur.r1) {
        const Stage<VT> sg = stage(s);
        const int64_t b = sg.rp[row - p0], e = sg.rp[row + 1 - p0];
        contrib += op.row(row, sg.col + (b - c0), sg.val + (b - v0), (int)(e - b));
      }
    } else if (row < cur.r1) {
      const int64_t b = rowptr[row], e = rowptr[row + 1];
      contrib += op.row(row, col + b, val + b, (int)(e - b));
    }
    __syncthreads();
  }
  if (!ok) {
    // a copy did not complete in time: report, drain the copies still in
    // flight (bounded) and leave
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      for (int s = 0; s < 2; ++s) (void)mbar_wait_bounded(&bar[s], phase[s]);
    }
    return;
  }
  if constexpr (Op::kReduce) {
    double total;
    if (grid_reduce<kTileRows>(contrib, blockIdx.x, gridDim.x, op.partials, op.counter, &total) &&
        threadIdx.x == 0)
      op.finish(total);
  }
}

int sm_count();
// device int set by kernels whose bounded waits gave up (0 = no error)
int *device_error_flag();

// rows per tile so that every tile's segment fits one stage
template <typename VT>
inline int rows_per_tile(int64_t max_row) {
  if (max_row <= 0) return kTileRows;
  const int64_t r = TileCap<VT>::value / max_row;
  if (r < 1) return 1;  // rows longer than a stage run on the unstaged path
  return (int)(r < kTileRows ? r : kTileRows);
}

// CTAs for a persistent launch over `tiles` tiles
template <typename VT>
inline unsigned rows_grid(int64_t tiles) {
  const int64_t per_sm = 1;  // one CTA per SM: the two stages use ~200 KB
  const int64_t g = (int64_t)sm_count() * per_sm;
  return (unsigned)(tiles < g ? (tiles > 0 ? tiles : 1) : g);
}

// sets the dynamic shared memory limit once per kernel instantiation
template <typename VT, class Op>
inline cudaError_t rows_prepare() {
  static cudaError_t e = cudaFuncSetAttribute(k_rows<VT, Op>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)tile_smem_bytes<VT>());
  return e;
}

template <typename VT, class Op>
inline lgx_status launch_rows(int64_t rb, int64_t re, int64_t max_row, const int64_t *rowptr,
                              const int32_t *col, const VT *val, const Op &op, cudaStream_t s) {
  if (re <= rb) return LGX_OK;
  LGX_CUDA(rows_prepare<VT, Op>());
  const int rpt = rows_per_tile<VT>(max_row);
  const int64_t tiles = (re - rb + rpt - 1) / rpt;
  k_rows<VT, Op><<<rows_grid<VT>(tiles), kTileRows, tile_smem_bytes<VT>(), s>>>(
    rb, re, rpt, rowptr, col, val, op, device_error_flag());
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

// grid size of a reducing launch (the partial buffer needs that many slots)
template <typename VT>
inline int64_t rows_partials(int64_t nrows, int64_t max_row) {
  const int rpt = rows_per_tile<VT>(max_row);
  return rows_grid<VT>((nrows + rpt - 1) / rpt);
}

// ---- row operations ---------------------------------------------------------
// sum_k fma(a_k, x[c_k], init) in storage order.  The column and x loads of
// up to 32 entries are issued together ahead of the dependent FMA chain, so a
// 27-point row costs one round of gather latency.
template <typename VT, typename XT>
__device__ __forceinline__ XT row_dot(const int32_t *c, const VT *v, int len,
                                      const XT *__restrict__ x, XT sum) {
  for (int k = 0; k < len; k += 32) {
    const int m = len - k < 32 ? len - k : 32;
    XT xv[32];
#pragma unroll
    for (int u = 0; u < 32; ++u)
      if (u < m) xv[u] = __ldg(x + c[k + u]);
#pragma unroll
    for (int u = 0; u < 32; ++u)
      if (u < m) sum = fma((XT)v[k + u], xv[u], sum);
  }
  return sum;
}

}  // namespace lgx
