// Persistent CSR row engine with TMA bulk staging.
//
// A CSR tile of R consecutive rows owns one contiguous segment of the column
// and value arrays.  Each CTA walks its tiles (t = blockIdx.x, +gridDim.x, ...)
// and stages each tile's row offsets, columns and values into shared memory
// with bulk copies (cp.async.bulk global->shared, completion counted on an
// mbarrier); then one thread per row computes the row from shared memory,
// the row's products in storage order.  Copy and compute overlap either
// inside a CTA (two stages: tile j+1 is in flight while tile j is computed)
// or between the two CTAs resident on an SM (one stage each); RowCfg lists
// the configurations.  The copies are whole 16-byte-aligned spans, so the
// segment's first entry sits at a small offset inside the stage.  Column and
// value buffers of every CSR in this library carry kCsrPad trailing
// elements, so the aligned span never leaves the allocation.
//
// Every wait on an mbarrier is bounded (about one second of SM clock); on
// timeout the kernel records an error in the library's device error flag,
// waits once more (bounded) for its own copies and returns.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <type_traits>

#include "lgx_internal.cuh"

namespace lgx {

constexpr int kTileRows = 256;     // threads per CTA, maximum rows per tile

// Engine configurations (the tuning space of the row kernels):
//   kind 0: two stages of CAP entries, one CTA per SM (prefetch overlap
//           inside the CTA);
//   kind 1: one stage, two CTAs per SM (the other CTA overlaps the copy);
//   kind 2: two smaller stages, two CTAs per SM.
template <typename VT, int KIND>
struct RowCfg {
  static constexpr int stages = KIND == 1 ? 1 : 2;
  static constexpr int ctas_per_sm = KIND == 0 ? 1 : 2;
  static constexpr int cap = KIND == 2 ? (sizeof(VT) == 8 ? 4096 : 6144)
                                       : (sizeof(VT) == 8 ? 8192 : 12288);
  // entries gathered per round of a row (register budget: 255 registers per
  // thread at one CTA per SM, 128 at two)
  static constexpr int gather = KIND == 0 ? 32 : 16;
};
// upper bound of the CTAs per SM of every row-engine configuration:
// reduction partials of row kernels are sized sm_count() * kRowsMaxCtasPerSm
constexpr int kRowsMaxCtasPerSm = 16;

// per stage: row offsets (kTileRows + 4) * 8 bytes, columns (CAP + 8) * 4
// bytes, values (CAP + 8) * sizeof(VT) bytes (an aligned span exceeds its
// segment by at most 6 elements); then per stage a bounds record and a barrier
template <typename VT, int KIND>
__host__ __device__ constexpr size_t stage_bytes() {
  return (size_t)(kTileRows + 4) * 8 + (size_t)(RowCfg<VT, KIND>::cap + 8) * 4 +
         (size_t)(RowCfg<VT, KIND>::cap + 8) * sizeof(VT);
}
template <typename VT, int KIND>
__host__ __device__ constexpr size_t tile_smem_bytes() {
  return RowCfg<VT, KIND>::stages * stage_bytes<VT, KIND>() + 2 * 32 + 64;
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
//   using X = <type of the gathered vector entries>;
//   template <int W> __device__ double row(int64_t row, const int32_t *c, const VT *v,
//                                          int len) const;
//     (returns the row's contribution to an optional sum; W = entries whose
//     gathers are issued together)
//   static constexpr bool kReduce;  __device__ void finish(double total) const;
//   double *partials; unsigned *counter;  (when kReduce)
template <typename VT, class Op, int KIND>
__global__ void __launch_bounds__(kTileRows, RowCfg<VT, KIND>::ctas_per_sm)
  k_rows(int64_t rb, int64_t re, int rows_per_tile, const int64_t *__restrict__ rowptr,
         const int32_t *__restrict__ col, const VT *__restrict__ val, Op op, int *err) {
  constexpr int CAP = RowCfg<VT, KIND>::cap;
  constexpr int NST = RowCfg<VT, KIND>::stages;
  static_assert(RowCfg<VT, KIND>::ctas_per_sm <= kRowsMaxCtasPerSm);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  static_assert((CAP + 8) * 4 % 16 == 0 && (CAP + 8) * sizeof(VT) % 16 == 0);
  // stage s starts at smem_raw + s * stage_bytes (computed, not indexed, so
  // the pointers stay in registers)
  auto stage = [&](int s) {
    unsigned char *p = smem_raw + (size_t)s * stage_bytes<VT, KIND>();
    Stage<VT> r;
    r.rp = reinterpret_cast<int64_t *>(p);
    r.col = reinterpret_cast<int32_t *>(p + (size_t)(kTileRows + 4) * 8);
    r.val = reinterpret_cast<VT *>(p + (size_t)(kTileRows + 4) * 8 + (size_t)(CAP + 8) * 4);
    return r;
  };
  TileRec *rec = reinterpret_cast<TileRec *>(smem_raw + NST * stage_bytes<VT, KIND>());
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + NST * stage_bytes<VT, KIND>() + 2 * 32);
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

  pdl_trigger();
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
  pdl_wait();

  unsigned phase[2] = {0u, 0u};
  double contrib = 0.0;
  bool ok = true;
  for (int64_t j = 0; t < ntiles; ++j, t += G) {
    // stage of tile j; with a single stage the next tile is issued after the
    // current one has been consumed (end of the iteration)
    const int s = NST == 2 ? (int)(j & 1) : 0;
    if (NST == 2 && threadIdx.x == 0 && t + G < ntiles) {
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
        contrib += op.template row<RowCfg<VT, KIND>::gather>(row, sg.col + (b - c0), sg.val + (b - v0),
                                                             (int)(e - b));
      }
    } else if (row < cur.r1) {
      const int64_t b = rowptr[row], e = rowptr[row + 1];
      contrib += op.template row<RowCfg<VT, KIND>::gather>(row, col + b, val + b, (int)(e - b));
    }
    __syncthreads();
    if (NST == 1 && threadIdx.x == 0 && t + G < ntiles) {
      rec[0] = ahead;
      if (ahead.e1 - ahead.e0 <= CAP) issue_tile<VT>(rowptr, col, val, ahead, stage(0), &bar[0]);
      if (t + 2 * G < ntiles) ahead = bounds(t + 2 * G);
    }
    if (NST == 1) __syncthreads();
  }
  if (!ok) {
    // a copy did not complete in time: report, drain the copies still in
    // flight (bounded) and leave
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      for (int s = 0; s < NST; ++s) (void)mbar_wait_bounded(&bar[s], phase[s]);
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
template <typename VT, int KIND>
inline int rows_per_tile(int64_t max_row) {
  if (max_row <= 0) return kTileRows;
  const int64_t r = RowCfg<VT, KIND>::cap / max_row;
  if (r < 1) return 1;  // rows longer than a stage run on the unstaged path
  return (int)(r < kTileRows ? r : kTileRows);
}

// ---- warp-tile engine ---------------------------------------------------------
// Every warp owns its own tiles of kWarpTileRows (32) consecutive rows and its
// own S shared-memory stages and mbarriers: lane 0 issues the bulk copies of
// the warp's next tiles while the lanes compute the current one (lane = row),
// and no barrier couples the warps of a CTA, so the SM always holds warps in
// every phase (copy in flight, gathers in flight, FMA chain).  A stage holds
// the tile's row offsets and up to `capw` entries; capw >= Csr::max_win (the
// most entries in any 32 consecutive rows), so every tile fits.  Tiles are
// dealt round-robin over all warps of the grid (tile = warp id + j * warps),
// which keeps the active rows, and so the x gathers, in a compact window.
// dynamic shared memory limit of a warp-tile CTA (227 KB per CTA minus room
// for the static reduction buffers, up to 2 KB + 16 B)
constexpr int kWrowsSmemMax = 224 * 1024;

__host__ __device__ constexpr size_t wstage_bytes(int capw, size_t vsize) {
  return (size_t)(kWarpTileRows + 4) * 8 + (size_t)(capw + 8) * 4 + (size_t)(capw + 8) * vsize;
}
// per CTA: WPC * S barriers and WPC * S "unstaged" flags, then the stages
__host__ __device__ constexpr size_t wheader_bytes(int wpc, int nst) {
  return (((size_t)wpc * nst * 12) + 15) & ~(size_t)15;
}
__host__ __device__ constexpr size_t wsmem_bytes(int wpc, int nst, int capw, size_t vsize) {
  return wheader_bytes(wpc, nst) + (size_t)wpc * nst * wstage_bytes(capw, vsize);
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// XT = the type of the gathered x values (Op::X)
// MB = CTAs per SM the registers are capped for (0: the default of WPC)
template <int WPC, typename XT, int MB = 0>
struct WrowsBounds {
  // 4 warps per CTA: registers <= 65536 / (5 * 128) so that five CTAs (20
  // warps) fit an SM, and 8 double (16 float) gathers per round to stay
  // within them; 8 warps per CTA: two CTAs (16 warps), 16 gathers per round;
  // MB = 7 (4 warps): seven CTAs (28 warps) where shared memory allows it
  // (float and bfloat16 stages), 16 float (8 double) gathers per round
  // within 73 registers
  static constexpr int min_blocks = MB ? MB : (WPC == 4 ? 5 : 2);
  static constexpr int gather = (WPC == 4 && sizeof(XT) == 8) ? 8 : 16;
};

template <typename VT, class Op, int WPC, int S, int MB = 0>
__global__ void __launch_bounds__(WPC * 32, WrowsBounds<WPC, typename Op::X, MB>::min_blocks)
  k_wrows(int64_t rb, int64_t re, int capw, const int64_t *__restrict__ rowptr,
          const int32_t *__restrict__ col, const VT *__restrict__ val, Op op, int *err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int W = WrowsBounds<WPC, typename Op::X, MB>::gather;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t sb = wstage_bytes(capw, sizeof(VT));
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw) + warp * S;
  int *unstaged = reinterpret_cast<int *>(smem_raw + (size_t)WPC * S * 8) + warp * S;
  unsigned char *base = smem_raw + wheader_bytes(WPC, S) + (size_t)warp * S * sb;
  auto stage = [&](int s) {
    unsigned char *p = base + (size_t)s * sb;
    Stage<VT> r;
    r.rp = reinterpret_cast<int64_t *>(p);
    r.col = reinterpret_cast<int32_t *>(p + (size_t)(kWarpTileRows + 4) * 8);
    r.val = reinterpret_cast<VT *>(p + (size_t)(kWarpTileRows + 4) * 8 + (size_t)(capw + 8) * 4);
    return r;
  };
  const int64_t ntiles = (re - rb + kWarpTileRows - 1) / kWarpTileRows;
  const int64_t GW = (int64_t)gridDim.x * WPC;
  int64_t t = (int64_t)blockIdx.x * WPC + warp;
  auto bounds = [&](int64_t tt) {
    TileRec r;
    r.r0 = rb + tt * kWarpTileRows;
    r.r1 = min(r.r0 + kWarpTileRows, re);
    r.e0 = rowptr[r.r0];
    r.e1 = rowptr[r.r1];
    return r;
  };
  // lane 0: stage s receives tile `tr` (bulk copies, or an empty arrival that
  // sends the lanes to global memory when the tile does not fit)
  auto issue = [&](const TileRec &tr, int s) {
    if (tr.e1 - tr.e0 <= capw) {
      unstaged[s] = 0;
      issue_tile<VT>(rowptr, col, val, tr, stage(s), &bar[s]);
    } else {
      unstaged[s] = 1;
      mbar_arrive(&bar[s]);
    }
  };

  pdl_trigger();
  TileRec ahead{};
  unsigned pending = 0;  // stages with an issued, not yet consumed tile
  if (lane == 0) {
    for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
    for (int s = 0; s < S; ++s) {
      if (t + s * GW < ntiles) {
        issue(bounds(t + s * GW), s);
        pending |= 1u << s;
      }
    }
    if (t + S * GW < ntiles) ahead = bounds(t + S * GW);
  }
  __syncwarp();
  // the matrix copies above only read constant data; vectors come after
  pdl_wait();

  unsigned phase = 0;
  double contrib = 0.0;
  bool ok = true;
  for (int64_t j = 0; t < ntiles; ++j, t += GW) {
    const int s = S == 1 ? 0 : (int)(j % S);
    const bool waited = mbar_wait_bounded(&bar[s], (phase >> s) & 1u);
    if (__any_sync(0xffffffffu, !waited)) {
      ok = false;
      break;
    }
    phase ^= 1u << s;
    pending &= ~(1u << s);
    const int64_t r0 = rb + t * kWarpTileRows;
    const int64_t row = r0 + lane;
    const int64_t r1 = min(r0 + kWarpTileRows, re);
    if (!unstaged[s]) {
      constexpr int64_t CA = 4, VA = 16 / (int64_t)sizeof(VT);
      const Stage<VT> sg = stage(s);
      const int64_t p0 = r0 & ~1ll;
      const int64_t e0 = sg.rp[r0 - p0];
      const int64_t c0 = e0 & ~(CA - 1), v0 = e0 & ~(VA - 1);
      if (row < r1) {
        const int64_t b = sg.rp[row - p0], e = sg.rp[row + 1 - p0];
        contrib += op.template row<W>(row, sg.col + (b - c0), sg.val + (b - v0), (int)(e - b));
      }
    } else if (row < r1) {
      const int64_t b = rowptr[row], e = rowptr[row + 1];
      contrib += op.template row<W>(row, col + b, val + b, (int)(e - b));
    }
    __syncwarp();
    if (lane == 0 && t + S * GW < ntiles) {
      issue(ahead, s);
      pending |= 1u << s;
      if (t + (S + 1) * GW < ntiles) ahead = bounds(t + (S + 1) * GW);
    }
  }
  if (!ok) {
    // a copy did not complete in time: report, drain this warp's copies still
    // in flight (bounded) and join the CTA's exit
    if (lane == 0) {
      atomicExch(err, 1);
      for (int s = 0; s < S; ++s)
        if (pending & (1u << s)) (void)mbar_wait_bounded(&bar[s], (phase >> s) & 1u);
    }
    __syncwarp();
  }
  if constexpr (Op::kReduce) {
    double total;
    if (grid_reduce<WPC * 32>(contrib, blockIdx.x, gridDim.x, op.partials, op.counter, &total) &&
        threadIdx.x == 0)
      op.finish(total);
  }
}

// engine configuration used by launch_rows (LGX_ROWS_CONFIG selects another
// entry of the tuning space): 0-2 CTA tiles (RowCfg kinds); warp tiles with
// 3: 4 warps x 1 stage, 4: 4 warps x 2 stages, 5: 8 warps x 1 stage,
// 6: 8 warps x 2 stages per CTA, 7: 4 warps x 1 stage with registers capped
// for seven CTAs per SM
int rows_config();

template <typename VT, class Op, int WPC, int S, int MB = 0>
inline lgx_status launch_wrows(int64_t rb, int64_t re, const Csr &a, const VT *val, const Op &op,
                               cudaStream_t s, bool *done) {
  *done = false;
  const int64_t mw = a.max_win > 4 ? a.max_win : 4;
  if (mw > (1 << 20)) return LGX_OK;
  const int capw = (int)((mw + 7) & ~7ll);  // 16-byte value spans also for 2-byte values
  const size_t smem = wsmem_bytes(WPC, S, capw, sizeof(VT));
  if (smem > (size_t)kWrowsSmemMax) return LGX_OK;  // too long rows: CTA tiles
  static const cudaError_t attr = cudaFuncSetAttribute(
    k_wrows<VT, Op, WPC, S, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, kWrowsSmemMax);
  LGX_CUDA(attr);
  // occupancy of the last shared-memory size asked for (one query per
  // matrix shape instead of one per launch): smem in the high, CTAs per SM
  // in the low 32 bits
  static std::atomic<uint64_t> occ_cache{0};
  int per_sm = 0;
  const uint64_t cached = occ_cache.load(std::memory_order_relaxed);
  if (cached >> 32 == (uint64_t)smem) {
    per_sm = (int)(uint32_t)cached;
  } else {
    LGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wrows<VT, Op, WPC, S, MB>,
                                                           WPC * 32, smem));
    occ_cache.store(((uint64_t)smem << 32) | (uint32_t)per_sm, std::memory_order_relaxed);
  }
  if (per_sm < 1) return LGX_OK;
  if (per_sm > kRowsMaxCtasPerSm) per_sm = kRowsMaxCtasPerSm;
  const int64_t tiles = (re - rb + kWarpTileRows - 1) / kWarpTileRows;
  const int64_t need = (tiles + WPC - 1) / WPC;
  const int64_t g = (int64_t)sm_count() * per_sm;
  const unsigned grid = (unsigned)(need < g ? (need > 0 ? need : 1) : g);
  const bool pdl = sizeof(typename Op::X) == 4 || re - rb <= pdl_fp64_rows();
  LGX_CUDA(launch_pdl(pdl, k_wrows<VT, Op, WPC, S, MB>, dim3(grid),
                      dim3(WPC * 32), smem, s, rb, re, capw,
                      (const int64_t *)a.rowptr.p, (const int32_t *)a.col.p, val, op,
                      device_error_flag()));
  count_launch();
  *done = true;
  return LGX_OK;
}

template <typename VT, class Op, int KIND>
inline lgx_status launch_rows_cfg(int64_t rb, int64_t re, int64_t max_row, const int64_t *rowptr,
                                  const int32_t *col, const VT *val, const Op &op,
                                  cudaStream_t s) {
  static const cudaError_t attr = cudaFuncSetAttribute(
    k_rows<VT, Op, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
    (int)tile_smem_bytes<VT, KIND>());
  LGX_CUDA(attr);
  const int rpt = rows_per_tile<VT, KIND>(max_row);
  const int64_t tiles = (re - rb + rpt - 1) / rpt;
  const int64_t g = (int64_t)sm_count() * RowCfg<VT, KIND>::ctas_per_sm;
  const unsigned grid = (unsigned)(tiles < g ? (tiles > 0 ? tiles : 1) : g);
  const bool pdl = sizeof(typename Op::X) == 4 || re - rb <= pdl_fp64_rows();
  LGX_CUDA(launch_pdl(pdl, k_rows<VT, Op, KIND>, dim3(grid),
                      dim3(kTileRows),
                      tile_smem_bytes<VT, KIND>(), s, rb, re, rpt, rowptr, col, val, op,
                      device_error_flag()));
  count_launch();
  return LGX_OK;
}

// autotuner slot of an operation: Op::kTuneClass when declared (SOR sweeps
// declare 1), else 0 (products)
template <class Op, class = void>
struct TuneClass {
  static constexpr int value = 0;
};
template <class Op>
struct TuneClass<Op, std::void_t<decltype(Op::kTuneClass)>> {
  static constexpr int value = Op::kTuneClass;
};

// rows [rb, re) of `a` (values `val`) through the engine configuration the
// autotuner chose for this matrix and operation, else the process-wide one
template <typename VT, class Op>
inline lgx_status launch_rows(int64_t rb, int64_t re, const Csr &a, const VT *val, const Op &op,
                              cudaStream_t s) {
  if (re <= rb) return LGX_OK;
  bool done = false;
  const int tuned = a.tuned[TuneClass<Op>::value][tune_value_index<VT>()];
  const int cfg = tuned >= 0 ? tuned : rows_config();
  switch (cfg) {
    case 3: LGX_CHECK((launch_wrows<VT, Op, 4, 1>(rb, re, a, val, op, s, &done))); break;
    case 4: LGX_CHECK((launch_wrows<VT, Op, 4, 2>(rb, re, a, val, op, s, &done))); break;
    case 5: LGX_CHECK((launch_wrows<VT, Op, 8, 1>(rb, re, a, val, op, s, &done))); break;
    case 6: LGX_CHECK((launch_wrows<VT, Op, 8, 2>(rb, re, a, val, op, s, &done))); break;
    case 7: LGX_CHECK((launch_wrows<VT, Op, 4, 1, 7>(rb, re, a, val, op, s, &done))); break;
    default: break;
  }
  if (done) return LGX_OK;
  switch (cfg) {
    case 0:
      return launch_rows_cfg<VT, Op, 0>(rb, re, a.max_row, a.rowptr.p, a.col.p, val, op, s);
    case 2:
      return launch_rows_cfg<VT, Op, 2>(rb, re, a.max_row, a.rowptr.p, a.col.p, val, op, s);
    default:
      return launch_rows_cfg<VT, Op, 1>(rb, re, a.max_row, a.rowptr.p, a.col.p, val, op, s);
  }
}

// ---- row operations ---------------------------------------------------------
// sum_k fma(a_k, x[c_k], init) in storage order.  The column and x loads of
// up to W entries are issued together ahead of the dependent FMA chain, so a
// 27-point row costs one (W = 32) or two (W = 16) rounds of gather latency.
template <int W, typename VT, typename XT>
__device__ __forceinline__ XT row_dot(const int32_t *c, const VT *v, int len,
                                      const XT *__restrict__ x, XT sum) {
  for (int k = 0; k < len; k += W) {
    const int m = len - k < W ? len - k : W;
    XT xv[W];
#pragma unroll
    for (int u = 0; u < W; ++u)
      if (u < m) xv[u] = __ldg(x + c[k + u]);
#pragma unroll
    for (int u = 0; u < W; ++u)
      if (u < m) sum = fma(cvt<XT>(v[k + u]), xv[u], sum);
  }
  return sum;
}

}  // namespace lgx
