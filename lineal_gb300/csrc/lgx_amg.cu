// Aggregation AMG on the device: strength of connection, greedy aggregation
// per partition, aggregate-map merge, Galerkin coarse matrices, the level
// hierarchy, a dense FP64 coarsest solver and the V-cycle.
//
// Reference: include/lineal/linear-solver/multigrid/ (dependency/criterion.hpp,
// aggregation/base.hpp, aggregation/independent.hpp,
// aggregate-map/multithread.hpp, transport/matrix-shared.hpp,
// transport/vector-shared.hpp, hierarchy/wright.hpp, solver.hpp).
#include <cuda_runtime.h>

#include <cfloat>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "lgx_amg.cuh"
#include "lgx_internal.cuh"

namespace lgx {

// ===========================================================================
// Strength of connection (dependency/criterion.hpp:35-78) with the
// NegativeOffdiagonalTransform (graph/weight-transform.hpp:28-38): edge
// weight w_ij = -a_ij, vertex weight a_jj.  strength = max(w_ij,0) * w' /
// a_jj with w' = max(w_ij,0) for value-symmetric matrices, else the reverse
// edge's max(w_ji,0) (0 if absent); an edge is strong iff strength >
// theta * max strength of the row.  The arithmetic runs in the matrix value
// type (GraphWeight = matrix Value).  depends is written for the row's own
// edges, influences for their reverse edges (each slot has one writer).
// ===========================================================================
__device__ __forceinline__ int64_t find_col(const int64_t *rowptr, const int32_t *col,
                                            int64_t row, int32_t c) {
  int64_t lo = rowptr[row], hi = rowptr[row + 1];
  const int64_t end = hi;
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (col[mid] < c) lo = mid + 1; else hi = mid;
  }
  return (lo < end && col[lo] == c) ? lo : -1;
}

__global__ void k_iota(int64_t n, int32_t *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int32_t)i;
}

// the diagonal of every row; rd (FP64 values): 1 / d correctly rounded, or
// 0 where |d| lies outside [2^-400, 2^400] (or is not finite) and the
// quotients divide
template <typename VT>
__global__ void k_row_diag(int64_t n, const int64_t *rowptr, const int32_t *col, const VT *val,
                           VT *diag, double *rd) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = find_col(rowptr, col, i, (int32_t)i);
    const VT d = k >= 0 ? val[k] : VT(0);
    diag[i] = d;
    if (rd) rd[i] = exponent_within_400((double)d) ? 1.0 / (double)d : 0.0;
  }
}

template <typename VT>
__device__ __forceinline__ VT edge_strength(int64_t i, int64_t e, const int64_t *rowptr,
                                            const int32_t *col, const VT *val, const VT *diag,
                                            int symmetric) {
  const int32_t j = col[e];
  const VT w = -val[e];
  const VT nn = w > VT(0) ? w : VT(0);
  VT opp;
  if (symmetric) {
    opp = nn;
  } else {
    const int64_t r = find_col(rowptr, col, j, (int32_t)i);
    const VT wr = r >= 0 ? -val[r] : VT(0);
    opp = r >= 0 ? (wr > VT(0) ? wr : VT(0)) : VT(0);
  }
  return nn * opp / diag[j];
}

// the same quotient through the reciprocal table rd (FP64: the correctly
// rounded quotient in five FP64 operations where rd marks d and the
// numerator lies in range; otherwise the division)
template <typename VT>
__device__ __forceinline__ VT edge_strength_rd(int64_t i, int64_t e, const int64_t *rowptr,
                                               const int32_t *col, const VT *val, const VT *diag,
                                               const double *rd, int symmetric) {
  if constexpr (sizeof(VT) != 8) {
    return edge_strength(i, e, rowptr, col, val, diag, symmetric);
  } else {
    const int32_t j = col[e];
    const VT w = -val[e];
    const VT nn = w > VT(0) ? w : VT(0);
    VT opp;
    if (symmetric) {
      opp = nn;
    } else {
      const int64_t r = find_col(rowptr, col, j, (int32_t)i);
      const VT wr = r >= 0 ? -val[r] : VT(0);
      opp = r >= 0 ? (wr > VT(0) ? wr : VT(0)) : VT(0);
    }
    const double num = nn * opp, y = rd[j];
    return (nonzero_bits(y) && exponent_within_400(num)) ? div_by_recip(num, diag[j], y)
                                                         : num / diag[j];
  }
}

// Strength flags of every row, one warp per row and a lane per entry: the
// row's largest off-diagonal strength, then per edge dep = s > theta * max,
// the reverse entry's inf flag (found by binary search in the head's row),
// and iso when no edge is strong.  The entries' searches run side by side
// (a thread per row walked 27 searches one after another: 19.6 ms at 256^3);
// a warp walks a contiguous run of rows;
// the row maximum is reduced with the sequential comparison (s > m), so it
// is the sequential maximum.
template <typename VT>
__global__ void k_strength_warp(int64_t n, const int64_t *rowptr, const int32_t *col,
                                const VT *val, const VT *diag, const double *rd, int symmetric,
                                VT theta, uint8_t *dep, uint8_t *inf, uint8_t *iso) {
  const int lane = threadIdx.x & 31;
  // each warp a contiguous run of rows: consecutive rows search mostly the
  // same neighbour rows, which then come from L1
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t per = (n + nw - 1) / nw;
  const int64_t i0 = w * per, i1 = i0 + per < n ? i0 + per : n;
  for (int64_t i = i0; i < i1; ++i) {
    const int64_t b = rowptr[i], e = rowptr[i + 1];
    VT maxs = VT(0);
    // a lane's first two strengths stay in registers for the second pass (the
    // FP64 division in each is what bounds this kernel on GB300)
    VT keep0 = VT(0), keep1 = VT(0);
    for (int64_t k = b + lane, m = 0; k < e; k += 32, ++m) {
      if (col[k] == i) continue;
      const VT sk = edge_strength_rd(i, k, rowptr, col, val, diag, rd, symmetric);
      if (m == 0) keep0 = sk;
      else if (m == 1) keep1 = sk;
      if (sk > maxs) maxs = sk;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const VT other = __shfl_xor_sync(0xffffffffu, maxs, o);
      if (other > maxs) maxs = other;
    }
    const VT lb = theta * maxs;
    bool any = false;
    for (int64_t k = b + lane, m = 0; k < e; k += 32, ++m) {
      const int32_t j = col[k];
      if (j == i) {
        dep[k] = 0;
        continue;
      }
      const VT sk = m == 0   ? keep0
                    : m == 1 ? keep1
                             : edge_strength_rd(i, k, rowptr, col, val, diag, rd, symmetric);
      const bool cond = sk > lb;
      any = any || cond;
      dep[k] = cond;
      const int64_t r = find_col(rowptr, col, j, (int32_t)i);
      if (r >= 0) inf[r] = cond;
    }
    any = __any_sync(0xffffffffu, any);
    if (lane == 0) iso[i] = !any;
  }
}

__global__ void k_fill_u8(int64_t n, uint8_t *p, uint8_t v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

lgx_status strength(const Csr &a, double theta, uint8_t *dep, uint8_t *inf, uint8_t *iso,
                    cudaStream_t s) {
  const int64_t n = a.n;
  if (n == 0) return LGX_OK;
  const unsigned g = (unsigned)std::min<int64_t>(grid_for(n, 128), 65535);
  const unsigned gw = (unsigned)std::min<int64_t>(grid_for(n, 8), 16384);  // warp per row
  // diagonal entries of the diagonal itself carry no influence flag
  k_fill_u8<<<std::min<int64_t>(grid_for(a.nnz, 256), 16384), 256, 0, s>>>(a.nnz, inf, 0);
  LGX_LAUNCH_CHECK();
  if (a.storage == LGX_F64) {
    DBuf<double> d, rd;
    LGX_CHECK(d.alloc(n));
    LGX_CHECK(rd.alloc(n));
    k_row_diag<double><<<g, 128, 0, s>>>(n, a.rowptr.p, a.col.p, a.v64.p, d.p, rd.p);
    LGX_LAUNCH_CHECK();
    k_strength_warp<double><<<gw, 256, 0, s>>>(n, a.rowptr.p, a.col.p, a.v64.p, d.p, rd.p,
                                               a.symmetric, theta, dep, inf, iso);
    LGX_LAUNCH_CHECK();
    LGX_CUDA(cudaStreamSynchronize(s));
  } else {
    DBuf<float> d;
    LGX_CHECK(d.alloc(n));
    k_row_diag<float><<<g, 128, 0, s>>>(n, a.rowptr.p, a.col.p, a.v32.p, d.p, nullptr);
    LGX_LAUNCH_CHECK();
    k_strength_warp<float><<<gw, 256, 0, s>>>(n, a.rowptr.p, a.col.p, a.v32.p, d.p, nullptr,
                                              a.symmetric, (float)theta, dep, inf, iso);
    LGX_LAUNCH_CHECK();
    LGX_CUDA(cudaStreamSynchronize(s));
  }
  return LGX_OK;
}

// ===========================================================================
// Greedy aggregation, one warp per contiguous partition
// (aggregation/base.hpp:28-711 via independent.hpp:47-216).  The subgraph of
// a partition keeps only edges whose head lies inside it.
//
// The reference algorithm is sequential within a partition; here the 32 lanes
// of a warp share each of its steps while producing the same decisions:
//  - the front (AggregateFront, base.hpp:28-74) is an unordered set with a
//    position index; the reference iterates it in ascending vertex order, so
//    every selection below takes the smallest vertex ids explicitly;
//  - grow_aggregate (base.hpp:532-585) evaluates every front vertex in
//    parallel.  Its sequential scan keeps the vertices whose key equals the
//    maximum key, where the key is (two-way count, connectivity, front
//    neighbours) if any front vertex has a two-way connection and
//    (one-way count, ...) otherwise, and then adds the smallest `room` ids;
//  - round_aggregate (base.hpp:601-636) adds the smallest id that passes;
//  - add_help (base.hpp:263-287) handles the edges of a vertex in parallel;
//    its effects (connected-aggregate set, front set) do not depend on the
//    edge order, and "connected" is an O(1) flag per local aggregate.
// All scratch lives in n-sized arrays indexed by vertex (or by local
// aggregate id), so partition p owns the slots [pb, pe).
// ===========================================================================
struct AggDev {
  const int64_t *rowptr;
  const int32_t *col;
  const uint8_t *dep, *inf, *iso;
  uint32_t *agg;
  int64_t n, nparts;
  int32_t min_size, max_size;
  int aggressive;
  int32_t *front;       // front members (unordered), slots [pb, pe)
  int32_t *front_pos;   // position in `front` by vertex, -1 when absent
  int32_t *conn;        // connected local aggregate ids, slots [pb, pe)
  uint8_t *conn_flag;   // by local aggregate id, slot pb + ag
  int32_t *blocks;      // aggregate k of partition p: [(pb + k) * max, ...)
  int32_t *block_len;   // aggregate k of partition p: slot pb + k
  int32_t *eval;        // per front position: 4 ints of evaluation results
  int64_t *pcount;      // aggregates per partition
  int64_t *stats;       // 5 counters (atomic adds)
  int32_t cap;          // k_aggregate_cta: front and connected-list capacity
};

__device__ __forceinline__ int64_t part_begin(int64_t n, int64_t p, int64_t k) {
  const int64_t base = n / p, rem = n % p;
  return k * base + (k < rem ? k : rem);
}

constexpr unsigned kFull = 0xffffffffu;

struct AggWarp {
  const AggDev &D;
  int64_t pb, pe;
  int lane;
  // warp-uniform state
  int64_t front_len = 0, conn_len = 0, counter = 0;
  int64_t st[5] = {0, 0, 0, 0, 0};

  __device__ AggWarp(const AggDev &d, int64_t b, int64_t e) : D(d), pb(b), pe(e) {
    lane = threadIdx.x & 31;
  }
  __device__ bool in_range(int64_t v) const { return v >= pb && v < pe; }
  __device__ int32_t &blen(uint32_t ag) const { return D.block_len[pb + ag]; }
  __device__ int32_t *block(uint32_t ag) const {
    return D.blocks + (pb + (int64_t)ag) * D.max_size;
  }

  // AggregateManager::add_help: v joins aggregate ag; its in-range
  // neighbours update the connected set and the front.
  __device__ void add_help(int64_t v, uint32_t ag, int64_t &size) {
    ++size;
    if (lane == 0) {
      D.agg[v] = ag;
      block(ag)[blen(ag)++] = (int32_t)v;
    }
    __syncwarp();
    const int64_t eb = D.rowptr[v], ee = D.rowptr[v + 1];
    for (int64_t e0 = eb; e0 < ee; e0 += 32) {
      const int64_t e = e0 + lane;
      bool want_conn = false, want_front = false;
      uint32_t ta = kUnaggregated;
      int64_t t = -1;
      if (e < ee) {
        t = D.col[e];
        if (t != v && in_range(t)) {
          ta = D.agg[t];
          want_conn = ta < kIsolated && !D.conn_flag[pb + ta];
          want_front = ta == kUnaggregated && D.front_pos[t] < 0;
        }
      }
      // several lanes may name the same aggregate: the lowest lane records it
      const unsigned cmask = __ballot_sync(kFull, want_conn);
      bool leader = false;
      if (want_conn) {
        const unsigned same = __match_any_sync(cmask, ta);
        leader = (__ffs(same) - 1) == lane;
      }
      const unsigned lmask = __ballot_sync(kFull, leader);
      const unsigned below = (1u << lane) - 1u;
      if (leader) {
        const int64_t pos = conn_len + __popc(lmask & below);
        D.conn[pb + pos] = (int32_t)ta;
        D.conn_flag[pb + ta] = 1;
      }
      conn_len += __popc(lmask);
      const unsigned fmask = __ballot_sync(kFull, want_front);
      if (want_front) {
        const int64_t pos = front_len + __popc(fmask & below);
        D.front[pb + pos] = (int32_t)t;
        D.front_pos[t] = (int32_t)pos;
      }
      front_len += __popc(fmask);
      __syncwarp();
    }
  }

  __device__ void front_erase(int64_t v) {
    if (lane == 0) {
      const int32_t pos = D.front_pos[v];
      if (pos >= 0) {
        const int32_t last = D.front[pb + front_len - 1];
        D.front[pb + pos] = last;
        D.front_pos[last] = pos;
        D.front_pos[v] = -1;
      }
    }
    __syncwarp();
    --front_len;
  }

  __device__ void helpers_clear() {
    for (int64_t i = lane; i < front_len; i += 32) D.front_pos[D.front[pb + i]] = -1;
    for (int64_t i = lane; i < conn_len; i += 32) D.conn_flag[pb + D.conn[pb + i]] = 0;
    front_len = 0;
    conn_len = 0;
    __syncwarp();
  }

  // Per in-range edge of front vertex vtx calls f(edge, head, head aggregate,
  // head in front, head aggregate connected).  Edges are loaded eight at a
  // time with independent loads so the dependent chain col -> agg ->
  // connected-flag costs one round of latency per batch.
  template <class F>
  __device__ __forceinline__ void edges(int64_t vtx, F &&f) const {
    const int64_t eb = D.rowptr[vtx], ee = D.rowptr[vtx + 1];
    for (int64_t e0 = eb; e0 < ee; e0 += 8) {
      int64_t t[8];
      bool ok[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int64_t e = e0 + u;
        t[u] = e < ee ? (int64_t)D.col[e] : vtx;
        ok[u] = e < ee && t[u] != vtx && in_range(t[u]);
      }
      uint32_t ha[8];
      bool fr[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        ha[u] = ok[u] ? D.agg[t[u]] : kUnaggregated;
        fr[u] = ok[u] && D.front_pos[t[u]] >= 0;
      }
      bool cf[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) cf[u] = ok[u] && ha[u] < kIsolated && D.conn_flag[pb + ha[u]];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (ok[u]) f(e0 + u, t[u], ha[u], fr[u], cf[u]);
    }
  }

  // smallest vertex id > floor among the lane's front positions with mark set
  __device__ int64_t warp_min_marked(int64_t floor) const {
    int64_t best = INT64_MAX;
    for (int64_t i = lane; i < front_len; i += 32) {
      if (!D.eval[4 * (pb + i) + 3]) continue;
      const int64_t v = D.front[pb + i];
      if (v > floor && v < best) best = v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const int64_t other = __shfl_xor_sync(kFull, best, o);
      best = other < best ? other : best;
    }
    return best;
  }

  // grow_aggregate (base.hpp:532-585)
  __device__ void grow(uint32_t ag, int64_t &size) {
    while (size < D.min_size) {
      // evaluate every front vertex: eval = (cons2, cons1, con, nbs); adj
      // (full off-diagonal count) is re-read from the row offsets
      bool any2 = false;
      for (int64_t i = lane; i < front_len; i += 32) {
        const int64_t vtx = D.front[pb + i];
        int32_t *ev = D.eval + 4 * (pb + i);
        if (D.iso[vtx]) {
          ev[0] = ev[1] = 0;
          ev[3] = 0;
          continue;
        }
        int32_t con = 0, nbs = 0, c2 = 0, c1 = 0;
        edges(vtx, [&](int64_t e, int64_t, uint32_t ha, bool in_front, bool connected) {
          const bool dep = D.dep[e], inf = D.inf[e];
          con += connected;
          nbs += in_front;
          c2 += (ha == ag) && (inf && dep);
          c1 += (ha == ag) && (!inf && dep);
        });
        ev[0] = c2;
        ev[1] = c1;
        ev[2] = con;
        ev[3] = nbs;
        any2 = any2 || c2 > 0;
      }
      __syncwarp();
      const bool mode2 = __any_sync(kFull, any2);
      // maximum key among eligible vertices
      int32_t k0 = 0, kn = 0;
      double kc = 0.0;
      bool have = false;
      for (int64_t i = lane; i < front_len; i += 32) {
        const int64_t vtx = D.front[pb + i];
        if (D.iso[vtx]) continue;
        const int32_t *ev = D.eval + 4 * (pb + i);
        const int32_t c = mode2 ? ev[0] : ev[1];
        if (c <= 0) continue;
        const int64_t adj = (D.rowptr[vtx + 1] - D.rowptr[vtx]) - 1;
        const double con = (double)ev[2] / (double)adj;
        if (!have || c > k0 || (c == k0 && (con > kc || (con == kc && ev[3] > kn)))) {
          k0 = c;
          kc = con;
          kn = ev[3];
          have = true;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const int32_t o0 = __shfl_xor_sync(kFull, k0, o);
        const double oc = __shfl_xor_sync(kFull, kc, o);
        const int32_t on = __shfl_xor_sync(kFull, kn, o);
        const bool oh = __shfl_xor_sync(kFull, have, o);
        if (oh && (!have || o0 > k0 || (o0 == k0 && (oc > kc || (oc == kc && on > kn))))) {
          k0 = o0;
          kc = oc;
          kn = on;
          have = true;
        }
      }
      if (!have) break;  // no candidates (warp-uniform after the reduction)
      // mark the vertices whose key equals the maximum (eval[3] reused as mark)
      for (int64_t i = lane; i < front_len; i += 32) {
        const int64_t vtx = D.front[pb + i];
        int32_t *ev = D.eval + 4 * (pb + i);
        bool m = false;
        if (!D.iso[vtx]) {
          const int32_t c = mode2 ? ev[0] : ev[1];
          if (c > 0) {
            const int64_t adj = (D.rowptr[vtx + 1] - D.rowptr[vtx]) - 1;
            const double con = (double)ev[2] / (double)adj;
            m = c == k0 && con == kc && ev[3] == kn;
          }
        }
        ev[3] = m;
      }
      __syncwarp();
      // add the smallest `room` candidates in ascending order
      const int64_t room = D.max_size - size;
      int64_t floor = -1;
      int64_t picked[64];
      int64_t npick = 0;
      for (int64_t k = 0; k < room; ++k) {
        const int64_t v = warp_min_marked(floor);
        if (v == INT64_MAX) break;
        picked[npick++] = v;
        floor = v;
      }
      for (int64_t k = 0; k < npick; ++k) {
        front_erase(picked[k]);
        add_help(picked[k], ag, size);
      }
    }
  }

  // round_aggregate (base.hpp:601-636)
  __device__ void round(uint32_t ag, int64_t &size) {
    while (size < D.max_size) {
      int64_t best = INT64_MAX;
      for (int64_t i = lane; i < front_len; i += 32) {
        const int64_t vtx = D.front[pb + i];
        if (D.iso[vtx] || vtx >= best) continue;
        int32_t cons = 0, unagg = 0, inagg = 0;
        edges(vtx, [&](int64_t e, int64_t, uint32_t ha, bool, bool) {
          cons += (ha == ag) && D.dep[e];
          unagg += ha == kUnaggregated;
          inagg += ha == ag;
        });
        if (cons == 0 || unagg >= inagg) continue;
        best = vtx;
      }
      for (int o = 16; o > 0; o >>= 1) {
        const int64_t other = __shfl_xor_sync(kFull, best, o);
        best = other < best ? other : best;
      }
      if (best == INT64_MAX) break;
      front_erase(best);
      add_help(best, ag, size);
    }
  }

  // handle_vertex (base.hpp:638-677)
  __device__ void handle(int64_t seed) {
    if (D.agg[seed] != kUnaggregated) return;
    if (D.iso[seed]) {
      if (lane == 0) D.agg[seed] = kIsolated;
      __syncwarp();
      ++st[4];
      return;
    }
    const uint32_t ag = (uint32_t)counter;
    int64_t size = 0;
    add_help(seed, ag, size);
    grow(ag, size);
    round(ag, size);
    if (size == 1 && D.max_size > 1) {
      // find_merge_aggregate (base.hpp:487-503): first strong in-range edge
      // (ascending column) whose head lies in an aggregate with room
      uint32_t target = kUnaggregated;
      const int64_t eb = D.rowptr[seed], ee = D.rowptr[seed + 1];
      for (int64_t e0 = eb; e0 < ee && target == kUnaggregated; e0 += 32) {
        const int64_t e = e0 + lane;
        bool ok = false;
        uint32_t ta = kUnaggregated;
        if (e < ee) {
          const int64_t t = D.col[e];
          if (t != seed && in_range(t) && (D.dep[e] || D.inf[e])) {
            ta = D.agg[t];
            ok = ta < kIsolated && blen(ta) < D.max_size;
          }
        }
        const unsigned m = __ballot_sync(kFull, ok);
        if (m) target = __shfl_sync(kFull, ta, __ffs(m) - 1);
      }
      if (target != kUnaggregated) {
        if (lane == 0) {
          blen(ag) = 0;
          D.agg[seed] = target;
          block(target)[blen(target)++] = (int32_t)seed;
        }
        __syncwarp();
        ++st[3];
        helpers_clear();
        return;
      }
      if (D.aggressive) {
        if (lane == 0) {
          blen(ag) = 0;
          D.agg[seed] = kIsolated;
        }
        __syncwarp();
        ++st[4];
        helpers_clear();
        return;
      }
      ++st[2];
    } else {
      ++st[1];
    }
    ++counter;
    helpers_clear();
  }
};

constexpr int kAggWarpsPerBlock = 4;

__global__ void __launch_bounds__(32 * kAggWarpsPerBlock) k_aggregate(AggDev D) {
  const int64_t p = (int64_t)blockIdx.x * kAggWarpsPerBlock + (threadIdx.x >> 5);
  if (p >= D.nparts) return;  // whole warps leave together
  const int64_t pb = part_begin(D.n, D.nparts, p), pe = part_begin(D.n, D.nparts, p + 1);
  const int lane = threadIdx.x & 31;
  for (int64_t v = pb + lane; v < pe; v += 32) D.block_len[v] = 0;
  __syncwarp();
  AggWarp W(D, pb, pe);
  for (int64_t v = pb; v < pe; ++v) W.handle(v);
  if (lane == 0) {
    D.pcount[p] = W.counter;
    W.st[0] = W.counter;
    for (int k = 0; k < 5; ++k)
      if (W.st[k]) atomicAdd((unsigned long long *)&D.stats[k], (unsigned long long)W.st[k]);
  }
}

// ---------------------------------------------------------------------------
// The same aggregation with one CTA per partition and the partition's
// mutable state in shared memory, for levels with few, large partitions (the
// coarse levels: 8 to a few hundred partitions of 5k-70k vertices, rows of
// ~20 entries).  The aggregates of a partition form one sequential chain of
// dependent steps, so the kernel shortens the steps:
//  - warp 0 runs the warp kernel's sequential steps (add a vertex, update
//    the front and connected set, choose, pick) on shared memory: the
//    aggregate ids (16 bits per vertex), front and connected flags (one bit
//    per vertex / local aggregate), the front list with each member's row
//    offset and length (loaded once, when it joins), the connected list;
//  - each evaluation of the front (grow_aggregate's counts, round_
//    aggregate's test) is spread over the CTA, one warp per member, so the
//    members' rows load at once and each count is one warp reduction;
//    warps 1.. wait between evaluations at a named barrier that warp 0
//    releases;
//  - choices are integer reductions (redux.sync) over 32-bit vertex ids
//    and a 64-bit key.
// Measured at 256^3 against the warp kernel: levels 1-3 (174, 17, 8
// partitions) 153 / 754 / 268 ms before, with 60 % of it evaluating fronts
// of ~13 members one row per lane.  Decisions are the warp kernel's:
// counts are order-free sums, selections take the smallest vertex ids, a
// member's position is found by search, and every aggregate's vertices are
// added in the same order.  Capacities: local aggregate ids below 0xFFFE,
// rows below 65536 entries (counts are packed in 16-bit halves), front and
// connected lists within `cap` entries; a partition that exceeds one sets
// `overflow` and the host redoes the level with the warp kernel.
// ---------------------------------------------------------------------------
constexpr int kAggCtaThreads = 256;
constexpr int kAggCtaCapMax = 4096;
constexpr int kAggCtaCapMin = 256;
constexpr uint16_t kSUnagg = 0xFFFF, kSIso = 0xFFFE;
constexpr int kCmdGrow = 0, kCmdRound = 1, kCmdDone = 2;

__host__ __device__ inline int64_t agg_align16(int64_t b) { return (b + 15) / 16 * 16; }
__host__ __device__ inline int64_t agg_bit_words(int64_t P) { return (P + 31) / 32; }
// shared bytes of a partition of P vertices with list capacity cap (a
// multiple of 8): aggregate ids, two bit sets, then per list entry the row
// offset (8), member, row length, two counters (4 each), connected id (2)
__host__ __device__ inline int64_t agg_cta_base(int64_t P) {
  return agg_align16(2 * P) + agg_align16(8 * agg_bit_words(P));
}
__host__ __device__ inline int64_t agg_cta_bytes(int64_t P, int64_t cap) {
  return agg_cta_base(P) + 30 * cap;
}

struct AggCtaCtl {
  int32_t cmd, nfront, bad;
  uint32_t ag;
};

__device__ __forceinline__ void agg_cta_sync() {
  __syncwarp();
  asm volatile("bar.sync 1, %0;" ::"r"(kAggCtaThreads) : "memory");
}

struct AggCta {
  const AggDev &D;
  AggCtaCtl *ctl;
  int64_t pb, pe;
  int lane;
  int32_t cap;
  uint16_t *sagg;   // by local vertex: local aggregate id, kSUnagg, kSIso
  uint32_t *inF;    // by local vertex: front member
  uint32_t *cF;     // by local aggregate id: connected
  int64_t *fbeg;    // per front position: row offset of the member
  int32_t *front;   // per front position: member (vertex id); unordered
  int32_t *flen;    // per front position: row length, 0 for isolated members
  uint32_t *cntA, *cntB;  // per front position: packed 16-bit counts / mark
  uint16_t *conn;   // connected local aggregate ids
  // warp 0's state (warp-uniform)
  int64_t front_len = 0, conn_len = 0, counter = 0;
  int64_t st[5] = {0, 0, 0, 0, 0};
  bool bad = false;

  __device__ AggCta(const AggDev &d, AggCtaCtl *c, int64_t b, int64_t e, unsigned char *smem)
      : D(d), ctl(c), pb(b), pe(e) {
    lane = threadIdx.x & 31;
    cap = d.cap;
    const int64_t P = e - b;
    unsigned char *q = smem;
    sagg = (uint16_t *)q;
    q += agg_align16(2 * P);
    inF = (uint32_t *)q;
    cF = inF + agg_bit_words(P);
    q += agg_align16(8 * agg_bit_words(P));
    fbeg = (int64_t *)q;
    q += 8 * (int64_t)cap;
    front = (int32_t *)q;
    flen = front + cap;
    cntA = (uint32_t *)(flen + cap);
    cntB = cntA + cap;
    q += 16 * (int64_t)cap;
    conn = (uint16_t *)q;
  }
  __device__ bool in_range(int64_t v) const { return v >= pb && v < pe; }
  __device__ int32_t &blen(uint32_t ag) const { return D.block_len[pb + ag]; }
  __device__ int32_t *block(uint32_t ag) const {
    return D.blocks + (pb + (int64_t)ag) * D.max_size;
  }
  __device__ uint32_t agg_of(int64_t v) const {
    const uint16_t a = sagg[v - pb];
    return a == kSUnagg ? kUnaggregated : a == kSIso ? kIsolated : (uint32_t)a;
  }
  __device__ void set_agg(int64_t v, uint32_t a) const {
    sagg[v - pb] = a == kUnaggregated ? kSUnagg : a == kIsolated ? kSIso : (uint16_t)a;
  }
  __device__ bool in_front(int64_t v) const {
    const int64_t u = v - pb;
    return (inF[u >> 5] >> (u & 31)) & 1u;
  }
  __device__ void front_flag(int64_t v, bool on) const {
    const int64_t u = v - pb;
    if (on) atomicOr(&inF[u >> 5], 1u << (u & 31));
    else atomicAnd(&inF[u >> 5], ~(1u << (u & 31)));
  }
  __device__ bool connected(uint32_t ag) const { return (cF[ag >> 5] >> (ag & 31)) & 1u; }
  __device__ void conn_flag(uint32_t ag, bool on) const {
    if (on) atomicOr(&cF[ag >> 5], 1u << (ag & 31));
    else atomicAnd(&cF[ag >> 5], ~(1u << (ag & 31)));
  }

  // ---- the CTA-wide evaluation (every thread) ----
  // Warp w counts the members w, w + W, ... (W warps), two at a time with
  // their loads in flight together; the lanes cover a member's row.
  __device__ void eval_part() const {
    constexpr int W = kAggCtaThreads / 32;
    const int cmd = ctl->cmd;
    const int32_t nf = ctl->nfront;
    const uint32_t ag = ctl->ag;
    const int32_t warp = (int32_t)(threadIdx.x >> 5);
    for (int32_t m0 = warp; m0 < nf; m0 += 2 * W) {
      int32_t mm[2] = {m0, m0 + W};
      int64_t eb[2];
      int32_t len[2], self[2];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const bool ok = mm[j] < nf;
        eb[j] = ok ? fbeg[mm[j]] : 0;
        len[j] = ok ? flen[mm[j]] : 0;
        self[j] = ok ? front[mm[j]] : -1;
      }
      const int32_t most = len[0] > len[1] ? len[0] : len[1];
      uint32_t a[2] = {0, 0}, b[2] = {0, 0};
      for (int32_t o = lane; o - lane < most; o += 32) {
        int32_t t[2];
        uint8_t dp[2], nf_[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          t[j] = -1;
          dp[j] = nf_[j] = 0;
          if (o < len[j]) {
            const int64_t e = eb[j] + o;
            t[j] = D.col[e];
            dp[j] = D.dep[e];
            nf_[j] = cmd == kCmdGrow ? D.inf[e] : 0;
          }
        }
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          if (t[j] < 0 || t[j] == self[j] || !in_range(t[j])) continue;
          const uint32_t ha = agg_of(t[j]);
          if (cmd == kCmdGrow) {
            // (two-way, one-way) counts into the aggregate | (connected, in front)
            a[j] += (ha == ag && dp[j] && nf_[j]) | (uint32_t)(ha == ag && dp[j] && !nf_[j]) << 16;
            b[j] += (ha < kIsolated && connected(ha)) | (uint32_t)in_front(t[j]) << 16;
          } else {
            // (dependent edges into the aggregate | edges into it), unaggregated
            a[j] += (ha == ag && dp[j]) | (uint32_t)(ha == ag) << 16;
            b[j] += ha == kUnaggregated;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const uint32_t sa = __reduce_add_sync(kFull, a[j]), sb = __reduce_add_sync(kFull, b[j]);
        if (lane == 0 && mm[j] < nf) {
          cntA[mm[j]] = sa;
          cntB[mm[j]] = sb;
        }
      }
    }
  }

  // warp 0: counts of every front member into cntA / cntB, the whole CTA
  // taking part
  __device__ void eval(int cmd, uint32_t ag) {
    if (lane == 0) {
      ctl->cmd = cmd;
      ctl->nfront = (int32_t)front_len;
      ctl->ag = ag;
    }
    agg_cta_sync();  // releases the other warps
    eval_part();
    agg_cta_sync();  // every count is in
  }

  // ---- warp 0's sequential steps ----
  // AggregateManager::add_help: v (row [eb, ee)) joins aggregate ag; its
  // in-range neighbours update the connected set and the front, new front
  // members get their row offsets and lengths
  __device__ void add_help(int64_t v, uint32_t ag, int64_t &size, int64_t eb, int64_t ee) {
    // the aggregate's list holds its `size` vertices so far
    if (lane == 0) {
      set_agg(v, ag);
      block(ag)[size] = (int32_t)v;
      blen(ag) = (int32_t)(size + 1);
    }
    ++size;
    __syncwarp();
    const int64_t f0 = front_len;
    for (int64_t base = eb; base < ee; base += 128) {
      int64_t tt[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t e = base + 32 * j + lane;
        tt[j] = e < ee ? (int64_t)D.col[e] : -1;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (base + 32 * j >= ee) break;  // uniform
        const int64_t t = tt[j];
        bool want_conn = false, want_front = false;
        uint32_t ta = kUnaggregated;
        if (t >= 0 && t != v && in_range(t)) {
          ta = agg_of(t);
          want_conn = ta < kIsolated && !connected(ta);
          want_front = ta == kUnaggregated && !in_front(t);
        }
        const unsigned cmask = __ballot_sync(kFull, want_conn);
        bool leader = false;
        if (want_conn) {
          const unsigned same = __match_any_sync(cmask, ta);
          leader = (__ffs(same) - 1) == lane;
        }
        const unsigned lmask = __ballot_sync(kFull, leader);
        const unsigned fmask = __ballot_sync(kFull, want_front);
        if (conn_len + __popc(lmask) > cap || front_len + __popc(fmask) > cap) {
          bad = true;  // uniform: the counts come from ballots
          return;
        }
        const unsigned below = (1u << lane) - 1u;
        if (leader) {
          conn[conn_len + __popc(lmask & below)] = (uint16_t)ta;
          conn_flag(ta, true);
        }
        conn_len += __popc(lmask);
        if (want_front) {
          front[front_len + __popc(fmask & below)] = (int32_t)t;
          front_flag(t, true);
        }
        front_len += __popc(fmask);
        __syncwarp();
      }
    }
    bool long_row = false;
    for (int64_t q = f0 + lane; q < front_len; q += 32) {
      const int64_t t = front[q];
      const int64_t rb = D.rowptr[t], re = D.rowptr[t + 1];
      fbeg[q] = rb;
      long_row = long_row || re - rb > 65535;
      flen[q] = D.iso[t] ? 0 : (int32_t)(re - rb);
    }
    if (__any_sync(kFull, long_row)) bad = true;  // counts would not fit 16 bits
    __syncwarp();
  }

  // removes front member v; returns its row
  __device__ void front_take(int64_t v, int64_t &eb, int64_t &ee) {
    uint32_t pos1 = 0;  // position + 1
    for (int64_t i = lane; i < front_len; i += 32)
      if (front[i] == (int32_t)v) pos1 = (uint32_t)i + 1;
    pos1 = __reduce_max_sync(kFull, pos1);
    // v was picked from the front, so it is there (guarded all the same)
    if (pos1 == 0) {
      bad = true;
      eb = ee = 0;
      return;
    }
    const int64_t pos = pos1 - 1;
    eb = fbeg[pos];
    ee = eb + flen[pos];
    __syncwarp();
    if (lane == 0) {
      const int64_t last = front_len - 1;
      front[pos] = front[last];
      fbeg[pos] = fbeg[last];
      flen[pos] = flen[last];
      front_flag(v, false);
    }
    __syncwarp();
    --front_len;
  }

  __device__ void helpers_clear() {
    for (int64_t i = lane; i < front_len; i += 32) front_flag(front[i], false);
    for (int64_t i = lane; i < conn_len; i += 32) conn_flag(conn[i], false);
    front_len = 0;
    conn_len = 0;
    __syncwarp();
  }

  // smallest member id > floor among the marked positions (mark in cntA);
  // vertex ids are below 2^31
  __device__ uint32_t warp_min_marked(uint32_t floor) const {
    uint32_t best = 0xFFFFFFFFu;
    for (int64_t i = lane; i < front_len; i += 32) {
      const uint32_t v = (uint32_t)front[i];
      if (cntA[i] && (floor == 0xFFFFFFFFu || v > floor) && v < best) best = v;
    }
    return __reduce_min_sync(kFull, best);
  }

  // grow_aggregate (base.hpp:532-585).  A member's key is (count,
  // connectivity, front neighbours) with connectivity = connected / (row
  // length - 1) compared as doubles.  Here it is one 64-bit integer:
  // count << 48 | floor(connected * (2^32 - 1) / (row length - 1)) << 16 |
  // neighbours.  Distinct fractions with denominators below 2^16 differ by
  // more than 1 / (2^32 - 1), so the scaled floors order and tie exactly as
  // the fractions -- and as their correctly rounded quotients, which lie
  // much closer than that apart only when equal.  Rows without a diagonal
  // (a connected count above the denominator, or a zero denominator) are
  // left to the warp kernel.
  __device__ void grow(uint32_t ag, int64_t &size) {
    while (size < D.min_size && front_len > 0) {
      eval(kCmdGrow, ag);
      bool any2 = false;
      for (int64_t i = lane; i < front_len; i += 32) any2 = any2 || (cntA[i] & 0xFFFFu) != 0;
      const bool mode2 = __any_sync(kFull, any2);
      bool odd = false;
      uint64_t kmax = 0;
      for (int64_t i = lane; i < front_len; i += 32) {
        const uint32_t c = mode2 ? cntA[i] & 0xFFFFu : cntA[i] >> 16;
        uint64_t key = 0;
        if (c > 0) {
          const uint64_t con = cntB[i] & 0xFFFFu, nb = cntB[i] >> 16;
          const uint64_t den = (uint64_t)(flen[i] - 1);
          if (den == 0 || con > den) {
            odd = true;
          } else {
            key = (uint64_t)c << 48 | (con * 0xFFFFFFFFull / den) << 16 | nb;
          }
        }
        cntA[i] = (uint32_t)(key >> 32);
        cntB[i] = (uint32_t)key;
        kmax = key > kmax ? key : kmax;
      }
      if (__any_sync(kFull, odd)) {
        bad = true;
        return;
      }
      const uint32_t khi = __reduce_max_sync(kFull, (uint32_t)(kmax >> 32));
      const uint32_t klo =
        __reduce_max_sync(kFull, (uint32_t)(kmax >> 32) == khi ? (uint32_t)kmax : 0u);
      if (khi == 0 && klo == 0) break;  // no candidates
      // mark the members whose key equals the maximum (cntA becomes the mark)
      int64_t nmarked = 0;
      for (int64_t base = 0; base < front_len; base += 32) {
        const int64_t i = base + lane;
        bool m = false;
        if (i < front_len) {
          m = cntA[i] == khi && cntB[i] == klo;
          cntA[i] = m;
        }
        nmarked += __popc(__ballot_sync(kFull, m));
      }
      __syncwarp();
      const int64_t room = D.max_size - size;
      const int64_t npick = nmarked < room ? nmarked : room;
      uint32_t picked[64];
      uint32_t floor = 0xFFFFFFFFu;
      for (int64_t k = 0; k < npick; ++k) {
        floor = warp_min_marked(floor);
        picked[k] = floor;
      }
      for (int64_t k = 0; k < npick; ++k) {
        int64_t eb, ee;
        front_take(picked[k], eb, ee);
        if (bad) return;
        add_help(picked[k], ag, size, eb, ee);
        if (bad) return;
      }
    }
  }

  // round_aggregate (base.hpp:601-636)
  __device__ void round(uint32_t ag, int64_t &size) {
    while (size < D.max_size && front_len > 0) {
      eval(kCmdRound, ag);
      uint32_t best = 0xFFFFFFFFu;
      for (int64_t i = lane; i < front_len; i += 32) {
        const uint32_t cons = cntA[i] & 0xFFFFu, inagg = cntA[i] >> 16, unagg = cntB[i];
        if (cons == 0 || unagg >= inagg) continue;
        best = (uint32_t)front[i] < best ? (uint32_t)front[i] : best;
      }
      best = __reduce_min_sync(kFull, best);
      if (best == 0xFFFFFFFFu) break;
      int64_t eb, ee;
      front_take(best, eb, ee);
      if (bad) return;
      add_help(best, ag, size, eb, ee);
      if (bad) return;
    }
  }

  // handle_vertex (base.hpp:638-677)
  __device__ void handle(int64_t seed) {
    if (agg_of(seed) != kUnaggregated) return;
    const bool iso = D.iso[seed];
    const int64_t eb = D.rowptr[seed], ee = D.rowptr[seed + 1];
    if (iso) {
      if (lane == 0) set_agg(seed, kIsolated);
      __syncwarp();
      ++st[4];
      return;
    }
    if (counter >= (int64_t)kSIso) {
      bad = true;  // local aggregate ids must fit 16 bits
      return;
    }
    const uint32_t ag = (uint32_t)counter;
    int64_t size = 0;
    add_help(seed, ag, size, eb, ee);
    if (bad) return;
    grow(ag, size);
    if (bad) return;
    round(ag, size);
    if (bad) return;
    if (size == 1 && D.max_size > 1) {
      // find_merge_aggregate (base.hpp:487-503): first strong in-range edge
      // (ascending column) whose head lies in an aggregate with room
      uint32_t target = kUnaggregated;
      for (int64_t e0 = eb; e0 < ee && target == kUnaggregated; e0 += 32) {
        const int64_t e = e0 + lane;
        bool ok = false;
        uint32_t ta = kUnaggregated;
        if (e < ee) {
          const int64_t t = D.col[e];
          if (t != seed && in_range(t) && (D.dep[e] || D.inf[e])) {
            ta = agg_of(t);
            ok = ta < kIsolated && blen(ta) < D.max_size;
          }
        }
        const unsigned m = __ballot_sync(kFull, ok);
        if (m) target = __shfl_sync(kFull, ta, __ffs(m) - 1);
      }
      if (target != kUnaggregated) {
        if (lane == 0) {
          blen(ag) = 0;
          set_agg(seed, target);
          block(target)[blen(target)++] = (int32_t)seed;
        }
        __syncwarp();
        ++st[3];
        helpers_clear();
        return;
      }
      if (D.aggressive) {
        if (lane == 0) {
          blen(ag) = 0;
          set_agg(seed, kIsolated);
        }
        __syncwarp();
        ++st[4];
        helpers_clear();
        return;
      }
      ++st[2];
    } else {
      ++st[1];
    }
    ++counter;
    helpers_clear();
  }
};

__global__ void __launch_bounds__(kAggCtaThreads) k_aggregate_cta(AggDev D, int *overflow) {
  extern __shared__ __align__(16) unsigned char agg_smem[];
  __shared__ AggCtaCtl ctl;
  const int64_t p = blockIdx.x;
  if (p >= D.nparts) return;  // the whole block leaves together
  const int64_t pb = part_begin(D.n, D.nparts, p), pe = part_begin(D.n, D.nparts, p + 1);
  const int64_t P = pe - pb;
  AggCta S(D, &ctl, pb, pe, agg_smem);
  for (int64_t u = threadIdx.x; u < P; u += kAggCtaThreads) {
    S.sagg[u] = kSUnagg;
    D.block_len[pb + u] = 0;
  }
  for (int64_t w = threadIdx.x; w < 2 * agg_bit_words(P); w += kAggCtaThreads) S.inF[w] = 0u;
  if (threadIdx.x == 0) {
    ctl.cmd = kCmdGrow;
    ctl.bad = 0;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    for (int64_t v = pb; v < pe && !S.bad; ++v) S.handle(v);
    if (S.lane == 0) {
      ctl.cmd = kCmdDone;
      ctl.bad = S.bad;
      ctl.ag = (uint32_t)S.counter;
    }
    agg_cta_sync();  // releases the other warps for good
  } else {
    // one evaluation per round; warp 0 says when the partition is done
    for (;;) {
      agg_cta_sync();
      if (ctl.cmd == kCmdDone) break;
      S.eval_part();
      agg_cta_sync();
    }
  }
  __syncthreads();
  if (ctl.bad) {
    if (threadIdx.x == 0) atomicExch(overflow, 1);
    return;
  }
  for (int64_t u = threadIdx.x; u < P; u += kAggCtaThreads) D.agg[pb + u] = S.agg_of(pb + u);
  if (threadIdx.x == 0) {
    D.pcount[p] = S.counter;
    S.st[0] = S.counter;
    for (int k = 0; k < 5; ++k)
      if (S.st[k]) atomicAdd((unsigned long long *)&D.stats[k], (unsigned long long)S.st[k]);
  }
}

// merge (aggregate-map/multithread.hpp:107-143): aggregate ids become global
// through the per-partition offsets; the coarse-to-fine lists are laid out
// partition by partition, aggregates in creation order.
__device__ __forceinline__ int64_t part_of(int64_t n, int64_t P, int64_t v) {
  const int64_t base = n / P, rem = n % P;
  const int64_t big = rem * (base + 1);
  return v < big ? v / (base + 1) : rem + (v - big) / base;
}

// partition of global aggregate c: the last p with poff[p] <= c
__device__ __forceinline__ int64_t part_of_aggregate(const int64_t *poff, int64_t P, int64_t c) {
  int64_t lo = 0, hi = P;
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) / 2;
    if (poff[mid] <= c) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void k_agg_fix(AggDev D, const int64_t *poff) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < D.n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t a = D.agg[v];
    if (a < kIsolated) D.agg[v] = a + (uint32_t)poff[part_of(D.n, D.nparts, v)];
  }
}

__global__ void k_agg_glen(AggDev D, const int64_t *poff, int64_t nc, int64_t *glen) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = part_of_aggregate(poff, D.nparts, c);
    glen[c] = D.block_len[part_begin(D.n, D.nparts, p) + (c - poff[p])];
  }
}

__global__ void k_agg_lists(AggDev D, const int64_t *poff, int64_t nc, const int64_t *list_ptr,
                            int32_t *list) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = part_of_aggregate(poff, D.nparts, c);
    const int64_t k = part_begin(D.n, D.nparts, p) + (c - poff[p]);
    const int32_t *blk = D.blocks + k * D.max_size;
    int64_t o = list_ptr[c];
    for (int32_t m = 0; m < D.block_len[k]; ++m) list[o++] = blk[m];
  }
}

// Kernel choice.  Levels with few partitions (at most four per SM) whose
// state fits in shared memory with lists of at least kAggCtaCapMin entries
// take k_aggregate_cta, every partition of the level resident at once;
// otherwise one warp per partition (the finest level: thousands of small
// partitions).  Measured at 256^3 (levels 1-4: 175, 17, 8, 8 partitions of
// 16k, 66k, 27k, 5k vertices, rows of ~50-150 entries) the warp kernel
// takes 154 / 744 / 288 / 45 ms, three fifths of it evaluating fronts of
// ~13 members one long row per lane.  LGX_AGG_KERNEL=warp / cta forces a
// kernel (the tests run both against the oracle; a forced cta choice whose
// partitions do not fit runs the warp kernel); LGX_AGG_CTA_CAP lowers the
// list capacity so that tests reach the overflow path on small cases.
//
// Capacity of the CTA kernel's lists for a level, 0 where it does not fit:
// the shared memory of an SM is shared by the partitions it must hold at
// once (1 KB of it reserved per CTA).
static int32_t agg_cta_cap(int64_t n, int64_t nparts, int64_t smem_optin, int64_t smem_sm,
                           int64_t sms, bool forced) {
  const int64_t pmax = (n + nparts - 1) / nparts;
  const int64_t per_sm = (nparts + sms - 1) / sms;
  const int64_t budget =
    std::min<int64_t>(smem_optin, smem_sm / per_sm - 1024 - (int64_t)sizeof(AggCtaCtl));
  const int64_t avail = budget - agg_cta_base(pmax) - 16;
  int64_t cap = std::min<int64_t>(kAggCtaCapMax, avail > 0 ? avail / 30 / 8 * 8 : 0);
  if (const char *e = std::getenv("LGX_AGG_CTA_CAP")) {
    const long v = std::strtol(e, nullptr, 10);
    if (v >= 8) cap = std::min<int64_t>(cap, v / 8 * 8);
  }
  if (cap < 8 || agg_cta_bytes(pmax, cap) > budget) return 0;
  if (!forced && (cap < kAggCtaCapMin || nparts > 4 * sms)) return 0;
  return (int32_t)cap;
}

lgx_status aggregate(const Csr &a, const uint8_t *dep, const uint8_t *inf, const uint8_t *iso,
                     int32_t min_size, int32_t max_size, int64_t nparts, int aggressive,
                     cudaStream_t s, AggResult &out, uint32_t *agg_out = nullptr) {
  const int64_t n = a.n;
  if (nparts < 1) nparts = 1;
  if (nparts > n && n > 0) nparts = n;
  // the kernels keep up to max_size picks per growth step in a local array
  if (max_size < 1 || min_size < 1 || max_size > 64 || min_size > max_size)
    return fail(LGX_ERR_INVALID, "aggregate sizes must satisfy 1 <= min <= max <= 64");
  uint32_t *agg = agg_out;
  if (!agg) {
    LGX_CHECK(out.agg.alloc(n));
    agg = out.agg.p;
  }
  int dev = 0, sms = 1, smem_optin = 0, smem_sm = 0;
  LGX_CUDA(cudaGetDevice(&dev));
  LGX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  LGX_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  LGX_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  const char *force = std::getenv("LGX_AGG_KERNEL");
  const bool want_warp = force && std::strcmp(force, "warp") == 0;
  const bool forced_cta = force && std::strcmp(force, "cta") == 0;
  const int32_t cap =
    n > 0 && !want_warp ? agg_cta_cap(n, nparts, smem_optin, smem_sm, sms, forced_cta) : 0;
  DBuf<int32_t> front, front_pos, conn, blocks, blen, eval;
  DBuf<uint8_t> conn_flag;
  DBuf<int64_t> pcount, poff, stats, glen;
  LGX_CHECK(blocks.alloc(n * max_size));
  LGX_CHECK(blen.alloc(n));
  LGX_CHECK(pcount.alloc(nparts));
  LGX_CHECK(poff.alloc(nparts + 1));
  LGX_CHECK(stats.alloc(5));
  LGX_CUDA(cudaMemsetAsync(stats.p, 0, sizeof(int64_t) * 5, s));
  LGX_CUDA(cudaMemsetAsync(pcount.p, 0, sizeof(int64_t) * nparts, s));
  AggDev D{a.rowptr.p, a.col.p,  dep,      inf,        iso,     agg,    n,
           nparts,     min_size, max_size, aggressive, nullptr, nullptr, nullptr,
           nullptr,    blocks.p, blen.p,   nullptr,    pcount.p, stats.p, cap};
  bool done = n == 0;
  if (cap > 0) {
    const int bytes = (int)agg_cta_bytes((n + nparts - 1) / nparts, cap);
    DBuf<int> overflow;
    LGX_CHECK(overflow.alloc(1));
    LGX_CUDA(cudaMemsetAsync(overflow.p, 0, sizeof(int), s));
    LGX_CUDA(cudaFuncSetAttribute(k_aggregate_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  bytes));
    k_aggregate_cta<<<(unsigned)nparts, kAggCtaThreads, bytes, s>>>(D, overflow.p);
    LGX_LAUNCH_CHECK();
    int of = 0;
    LGX_CUDA(cudaMemcpyAsync(&of, overflow.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    LGX_CUDA(cudaStreamSynchronize(s));
    done = of == 0;
    // a partition outgrew a capacity: the warp kernel redoes the level
    if (!done) LGX_CUDA(cudaMemsetAsync(stats.p, 0, sizeof(int64_t) * 5, s));
  }
  if (!done) {
    LGX_CHECK(front.alloc(n));
    LGX_CHECK(front_pos.alloc(n));
    LGX_CHECK(conn.alloc(n));
    LGX_CHECK(conn_flag.alloc(n));
    LGX_CHECK(eval.alloc(4 * n));
    LGX_CUDA(cudaMemsetAsync(agg, 0xFF, sizeof(uint32_t) * n, s));
    LGX_CUDA(cudaMemsetAsync(front_pos.p, 0xFF, sizeof(int32_t) * n, s));
    LGX_CUDA(cudaMemsetAsync(conn_flag.p, 0, n, s));
    D.front = front.p;
    D.front_pos = front_pos.p;
    D.conn = conn.p;
    D.conn_flag = conn_flag.p;
    D.eval = eval.p;
    k_aggregate<<<grid_for(nparts, kAggWarpsPerBlock), 32 * kAggWarpsPerBlock, 0, s>>>(D);
    LGX_LAUNCH_CHECK();
  }
  if (std::getenv("LGX_VERBOSE") && n > 0)
    std::fprintf(stderr, "[lgx setup] aggregation of %lld rows in %lld partitions: %s\n",
                 (long long)n, (long long)nparts,
                 cap > 0 ? (done ? "CTA kernel" : "CTA kernel overflowed, warp kernel")
                         : "warp kernel");
  LGX_CHECK(inclusive_offsets(nparts, pcount.p, poff.p, s));
  int64_t nc = 0;
  LGX_CUDA(cudaMemcpyAsync(&nc, poff.p + nparts, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaMemcpyAsync(out.stats, stats.p, sizeof(int64_t) * 5, cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  out.ncoarse = nc;
  LGX_CHECK(glen.alloc(nc));
  LGX_CHECK(out.list_ptr.alloc(nc + 1));
  if (n > 0) {
    k_agg_fix<<<std::min<int64_t>(grid_for(n, 256), 16384), 256, 0, s>>>(D, poff.p);
    LGX_LAUNCH_CHECK();
  }
  if (nc > 0) {
    k_agg_glen<<<std::min<int64_t>(grid_for(nc, 256), 16384), 256, 0, s>>>(D, poff.p, nc, glen.p);
    LGX_LAUNCH_CHECK();
  }
  LGX_CHECK(inclusive_offsets(nc, glen.p, out.list_ptr.p, s));
  int64_t total = 0;
  LGX_CUDA(cudaMemcpyAsync(&total, out.list_ptr.p + nc, sizeof(int64_t), cudaMemcpyDeviceToHost,
                           s));
  LGX_CUDA(cudaStreamSynchronize(s));
  LGX_CHECK(out.list.alloc(total));
  if (n > 0 && nc > 0) {
    k_agg_lists<<<std::min<int64_t>(grid_for(nc, 256), 16384), 256, 0, s>>>(
      D, poff.p, nc, out.list_ptr.p, out.list.p);
    LGX_LAUNCH_CHECK();
  }
  LGX_CUDA(cudaStreamSynchronize(s));
  return LGX_OK;
}

// ===========================================================================
// Galerkin coarse matrix (transport/matrix-shared.hpp:85-183, non-unique
// builder csr/shared.hpp:730-764): coarse row I gathers the fine rows of
// aggregate I in list order, columns ascending; each value is first cast to
// the coarse value type, then accumulated in double per coarse column in
// first-encounter order; the row is sorted by column; entries in isolated
// columns are dropped.  One thread per coarse row, scratch slots at the
// offsets of the row's fine entries.
// ===========================================================================
template <typename VT>
__global__ void k_galerkin_upper(int64_t nc, const int64_t *rowptr, const int64_t *list_ptr,
                                 const int32_t *list, int64_t *upper) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    int64_t u = 0;
    for (int64_t k = list_ptr[c]; k < list_ptr[c + 1]; ++k)
      u += rowptr[list[k] + 1] - rowptr[list[k]];
    upper[c] = u;
  }
}

// flagged_only: the rows that k_galerkin_warp left (count -1)
template <typename VT>
__global__ void k_galerkin_accumulate(int64_t nc, const int64_t *rowptr, const int32_t *col,
                                      const VT *val, const uint32_t *agg, const int64_t *list_ptr,
                                      const int32_t *list, int coarse_f32, const int64_t *soff,
                                      int32_t *scol, double *sval, int64_t *count,
                                      int flagged_only) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    if (flagged_only && count[c] != -1) continue;
    int32_t *cc = scol + soff[c];
    double *vv = sval + soff[c];
    int64_t m = 0;
    for (int64_t k = list_ptr[c]; k < list_ptr[c + 1]; ++k) {
      const int64_t i = list[k];
      for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e) {
        const uint32_t J = agg[col[e]];
        if (J >= kIsolated) continue;
        const double v = coarse_f32 ? (double)(float)val[e] : (double)val[e];
        int64_t f = 0;
        while (f < m && cc[f] != (int32_t)J) ++f;
        if (f == m) {
          cc[m] = (int32_t)J;
          vv[m] = v;
          ++m;
        } else {
          vv[f] = __dadd_rn(vv[f], v);
        }
      }
    }
    // insertion sort by column
    for (int64_t x = 1; x < m; ++x) {
      const int32_t c0 = cc[x];
      const double v0 = vv[x];
      int64_t y = x - 1;
      while (y >= 0 && cc[y] > c0) {
        cc[y + 1] = cc[y];
        vv[y + 1] = vv[y];
        --y;
      }
      cc[y + 1] = c0;
      vv[y + 1] = v0;
    }
    count[c] = m;
  }
}

// The same accumulation with one warp per coarse row: the row's fine entries
// (at most kGalCap, in encounter order: list order, then storage order) are
// staged in shared memory as (coarse column, value cast to the coarse type);
// an entry is its column's head when no earlier entry has that column and
// links to the next entry of its column; each head sums its column's values
// along the links, in encounter order (the sequential sum of the per-thread
// kernel), and is written at its rank among the heads by column.  All loads of a row go out in two rounds (the list rows' offsets,
// then every entry's column, value and aggregate), where the thread-per-row
// kernel walks its scratch in global memory entry by entry.  Rows with more
// entries get count -1 and are left to k_galerkin_accumulate (flagged).
constexpr int kGalCap = 512;
constexpr int kGalWarps = 4;
constexpr int kGalMaxList = 64;  // aggregates hold at most 64 rows

template <typename VT>
__global__ void __launch_bounds__(32 * kGalWarps)
  k_galerkin_warp(int64_t nc, const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                  const VT *__restrict__ val, const uint32_t *__restrict__ agg,
                  const int64_t *__restrict__ list_ptr, const int32_t *__restrict__ list,
                  int coarse_f32, const int64_t *__restrict__ soff, int32_t *scol, double *sval,
                  int64_t *count) {
  __shared__ int32_t sJ[kGalWarps][kGalCap];
  __shared__ double sV[kGalWarps][kGalCap];
  __shared__ uint32_t sHead[kGalWarps][kGalCap / 32];
  __shared__ int16_t sNext[kGalWarps][kGalCap], sHeadList[kGalWarps][kGalCap];
  __shared__ int64_t sRow[kGalWarps][kGalMaxList];
  __shared__ int32_t sPfx[kGalWarps][kGalMaxList + 1];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t *J = sJ[w];
  double *V = sV[w];
  uint32_t *H = sHead[w];
  int16_t *NX = sNext[w], *HL = sHeadList[w];
  int64_t *RB = sRow[w];
  int32_t *PF = sPfx[w];
  const int64_t nwarps = (int64_t)gridDim.x * kGalWarps;
  for (int64_t c = (int64_t)blockIdx.x * kGalWarps + w; c < nc; c += nwarps) {
    const int64_t n = soff[c + 1] - soff[c];
    const int64_t l0 = list_ptr[c], nl = list_ptr[c + 1] - l0;
    if (n > kGalCap || nl > kGalMaxList) {
      if (lane == 0) count[c] = -1;
      continue;
    }
    // the list rows' offsets and their prefix sums
    int32_t run = 0;
    for (int64_t b0 = 0; b0 < nl; b0 += 32) {
      const int64_t k = b0 + lane;
      int32_t len = 0;
      if (k < nl) {
        const int64_t i = list[l0 + k];
        const int64_t rb = rowptr[i];
        RB[k] = rb;
        len = (int32_t)(rowptr[i + 1] - rb);
      }
      int32_t x = len;
      for (int d = 1; d < 32; d <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
      }
      if (k < nl) PF[k + 1] = run + x;
      run += __shfl_sync(0xffffffffu, x, 31);
    }
    if (lane == 0) PF[0] = 0;
    __syncwarp();
    // stage every entry: item p of list row k sits at PF[k] + offset
    for (int32_t p = lane; p < (int32_t)n; p += 32) {
      int32_t lo = 0, hi = (int32_t)nl - 1;
      while (lo < hi) {
        const int32_t mid = (lo + hi + 1) >> 1;
        if (PF[mid] <= p) lo = mid;
        else hi = mid - 1;
      }
      const int64_t e = RB[lo] + (p - PF[lo]);
      const uint32_t jc = agg[col[e]];
      const VT vr = val[e];
      J[p] = jc >= kIsolated ? -1 : (int32_t)jc;
      V[p] = coarse_f32 ? (double)(float)vr : (double)vr;
    }
    __syncwarp();
    // links (integer work only): an entry is its column's head when no
    // earlier entry has the column; NX[q] = the next entry with q's column
    // (each scan stops at its first match)
    for (int32_t q0 = 0; q0 < (int32_t)n; q0 += 32) {
      const int32_t q = q0 + lane;
      bool head = false;
      if (q < (int32_t)n) {
        const int32_t jq = J[q];
        int32_t nx = -1;
        if (jq >= 0) {
          head = true;
          for (int32_t t = 0; t < q; ++t)
            if (J[t] == jq) {
              head = false;
              break;
            }
          for (int32_t t = q + 1; t < (int32_t)n; ++t)
            if (J[t] == jq) {
              nx = t;
              break;
            }
        }
        NX[q] = nx;
      }
      const unsigned m = __ballot_sync(0xffffffffu, head);
      if (lane == 0) H[q0 >> 5] = m;
    }
    __syncwarp();
    // the heads in entry order
    int32_t nh = 0;
    for (int32_t wd = 0; wd < ((int32_t)n + 31) / 32; ++wd) {
      const unsigned m = H[wd];
      if ((m >> lane) & 1u) HL[nh + __popc(m & ((1u << lane) - 1u))] = (int16_t)(wd * 32 + lane);
      nh += __popc(m);
    }
    __syncwarp();
    // one head per lane: its rank among the heads by column, and its
    // column's sum in encounter order along the links (the FP64 adds run
    // only along the chains: a warp-wide FP64 instruction costs the pipe the
    // same however few lanes it has)
    for (int32_t k = lane; k < nh; k += 32) {
      const int32_t q = HL[k], jq = J[q];
      int32_t rank = 0;
      for (int32_t u = 0; u < nh; ++u) rank += J[HL[u]] < jq;
      double sum = V[q];
      for (int32_t t = NX[q]; t >= 0; t = NX[t]) sum = __dadd_rn(sum, V[t]);
      scol[soff[c] + rank] = jq;
      sval[soff[c] + rank] = sum;
    }
    const int32_t heads = nh;
    if (lane == 0) count[c] = heads;
    __syncwarp();
  }
}

__global__ void k_galerkin_emit(int64_t nc, const int64_t *soff, const int32_t *scol,
                                const double *sval, const int64_t *rowptr_c, int32_t *col_c,
                                double *val_c, int coarse_f32) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = rowptr_c[c], m = rowptr_c[c + 1] - o;
    for (int64_t k = 0; k < m; ++k) {
      col_c[o + k] = scol[soff[c] + k];
      const double v = sval[soff[c] + k];
      val_c[o + k] = coarse_f32 ? (double)(float)v : v;
    }
  }
}

lgx_status galerkin(const Csr &a, const AggResult &ag, int coarse_f32, cudaStream_t s, Csr &out) {
  const int64_t nc = ag.ncoarse;
  DBuf<int64_t> upper, soff, count, rowptr_c;
  LGX_CHECK(upper.alloc(nc));
  LGX_CHECK(soff.alloc(nc + 1));
  LGX_CHECK(count.alloc(nc));
  LGX_CHECK(rowptr_c.alloc(nc + 1));
  const unsigned g = (unsigned)std::min<int64_t>(grid_for(nc, 128), 65535);
  if (nc > 0) {
    k_galerkin_upper<double><<<g, 128, 0, s>>>(nc, a.rowptr.p, ag.list_ptr.p, ag.list.p, upper.p);
    LGX_LAUNCH_CHECK();
  }
  LGX_CHECK(inclusive_offsets(nc, upper.p, soff.p, s));
  int64_t total = 0;
  LGX_CUDA(cudaMemcpyAsync(&total, soff.p + nc, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  DBuf<int32_t> scol;
  DBuf<double> sval;
  LGX_CHECK(scol.alloc(total));
  LGX_CHECK(sval.alloc(total));
  if (nc > 0) {
    // warp per coarse row, then the thread-per-row kernel for the rows too
    // long for its shared memory (LGX_GALERKIN_WARP=0: thread per row only)
    static const bool warp_on = [] {
      const char *e = std::getenv("LGX_GALERKIN_WARP");
      return !(e && e[0] == '0');
    }();
    const unsigned gw = (unsigned)std::min<int64_t>(grid_for(nc, kGalWarps), 16 * 152);
    if (a.storage == LGX_F64) {
      if (warp_on)
        k_galerkin_warp<double><<<gw, 32 * kGalWarps, 0, s>>>(
          nc, a.rowptr.p, a.col.p, a.v64.p, ag.agg.p, ag.list_ptr.p, ag.list.p, coarse_f32,
          soff.p, scol.p, sval.p, count.p);
      k_galerkin_accumulate<double><<<g, 128, 0, s>>>(nc, a.rowptr.p, a.col.p, a.v64.p, ag.agg.p,
                                                      ag.list_ptr.p, ag.list.p, coarse_f32, soff.p,
                                                      scol.p, sval.p, count.p, warp_on);
    } else {
      if (warp_on)
        k_galerkin_warp<float><<<gw, 32 * kGalWarps, 0, s>>>(
          nc, a.rowptr.p, a.col.p, a.v32.p, ag.agg.p, ag.list_ptr.p, ag.list.p, coarse_f32,
          soff.p, scol.p, sval.p, count.p);
      k_galerkin_accumulate<float><<<g, 128, 0, s>>>(nc, a.rowptr.p, a.col.p, a.v32.p, ag.agg.p,
                                                     ag.list_ptr.p, ag.list.p, coarse_f32, soff.p,
                                                     scol.p, sval.p, count.p, warp_on);
    }
    LGX_LAUNCH_CHECK();
  }
  LGX_CHECK(inclusive_offsets(nc, count.p, rowptr_c.p, s));
  int64_t nnz_c = 0;
  LGX_CUDA(cudaMemcpyAsync(&nnz_c, rowptr_c.p + nc, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  DBuf<int32_t> col_c;
  DBuf<double> val_c;
  LGX_CHECK(col_c.alloc(nnz_c));
  LGX_CHECK(val_c.alloc(nnz_c));
  if (nc > 0) {
    k_galerkin_emit<<<g, 128, 0, s>>>(nc, soff.p, scol.p, sval.p, rowptr_c.p, col_c.p, val_c.p,
                                      coarse_f32);
    LGX_LAUNCH_CHECK();
  }
  return csr_from_device(nc, nnz_c, rowptr_c.p, col_c.p, val_c.p, a.symmetric,
                         coarse_f32 ? LGX_F32 : a.storage, s, out);
}

// ===========================================================================
// Dense FP64 coarsest solver.  The coarsest matrix (at most a few thousand
// rows) is inverted once by Gauss-Jordan elimination without pivoting (SPD);
// each cycle then applies the inverse with one dense matrix-vector product,
// which replaces the sequential forward/backward substitution of
// cholesky/solver.hpp:42-50 by a fully parallel kernel.
// ===========================================================================
__global__ void k_dense_from_csr(int64_t n, const int64_t *rowptr, const int32_t *col,
                                 const double *v64, const float *v32, double *d) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double *row = d + i * n;
    for (int64_t j = 0; j < n; ++j) row[j] = 0.0;
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e)
      row[col[e]] = v64 ? v64[e] : (double)v32[e];
  }
}

// step k, part 1: pivot row scaled into prow, column factors into pcol.
// LuSolver's unpivoted elimination (lu/decomposition.hpp:31-122) needs a
// usable pivot: non-zero, finite and not below 64 eps times the largest
// entry of its row (every block forms the row maximum itself).
__global__ void __launch_bounds__(256)
  k_gj_pivot(int64_t n, int64_t k, double *a, double *prow, double *pcol, int *bad) {
  const double p = a[k * n + k];
  __shared__ double red[256];
  double m = 0.0;
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) m = fmax(m, fabs(a[k * n + j]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  const double rowmax = red[0];
  if (!(p != 0.0 && isfinite(p)) || fabs(p) < 64.0 * DBL_EPSILON * rowmax) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(bad, 1);
    return;
  }
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    prow[j] = j == k ? 1.0 / p : a[k * n + j] / p;
    pcol[j] = a[j * n + k];
  }
}

// step k, part 2: rank-one update of all rows
__global__ void k_gj_update(int64_t n, int64_t k, double *a, const double *prow,
                            const double *pcol, const int *bad) {
  if (*bad) return;
  const int64_t total = n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / n, j = t % n;
    if (i == k) {
      a[t] = prow[j];
    } else {
      const double f = pcol[i];
      a[t] = j == k ? -f * prow[k] : fma(-f, prow[j], a[t]);
    }
  }
}

// ---- dense FP64 Cholesky of the coarsest matrix (CholeskySolver,
// cholesky/decomposition.hpp:52-107, on the dense matrix): A = L L^T in the
// lower triangle, right-looking, one column per step; every pivot must be
// positive.  The inverse applied per V-cycle is then formed from the factor
// by two triangular solves with all n columns of the identity at once:
// L^-1 (forward substitution), then A^-1 = L^-T L^-1 (backward).
__global__ void __launch_bounds__(256) k_chol_column(int64_t n, int64_t k, double *a, int *bad) {
  const double d = a[k * n + k];
  if (!(d > 0.0) || !isfinite(d)) {
    if (threadIdx.x == 0) atomicOr(bad, 1);
    return;
  }
  const double lkk = sqrt(d);
  for (int64_t i = k + 1 + threadIdx.x; i < n; i += blockDim.x) a[i * n + k] = a[i * n + k] / lkk;
  if (threadIdx.x == 0) a[k * n + k] = lkk;
}

// trailing update of the lower triangle: a_ij -= l_ik l_jk for k < j <= i
__global__ void k_chol_update(int64_t n, int64_t k, double *a, const int *bad) {
  if (*bad) return;
  const int64_t m = n - k - 1;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * m;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = k + 1 + t / m, j = k + 1 + t % m;
    if (j > i) continue;
    a[i * n + j] = fma(-a[i * n + k], a[j * n + k], a[i * n + j]);
  }
}

// The two triangular solves with all n columns of the identity, column by
// column of L so that every step is one parallel rank-one update (a row of
// dependent sums per thread would be a chain of n loads):
//  forward,  X = L^-1: step k scales row k by 1 / l_kk, then row i > k
//            subtracts l_ik times row k;
//  backward, X = L^-T X: step k (from n - 1 down) scales row k by 1 / l_kk,
//            then row i < k subtracts l_ki times row k.
// Each scaling is its own launch so the update reads the finished row.
__global__ void k_tri_scale(int64_t n, int64_t k, const double *l, double *x) {
  const double d = l[k * n + k];
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    x[k * n + c] = x[k * n + c] / d;
}

// rows [r0, r1) of x: x_ic -= f(i) x_kc with f(i) = l_ik (forward) or l_ki
// (transposed, backward)
__global__ void k_tri_update(int64_t n, int64_t k, int64_t r0, int64_t r1, int transposed,
                             const double *l, double *x) {
  const int64_t rows = r1 - r0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = r0 + t / n, c = t % n;
    const double f = transposed ? l[k * n + i] : l[i * n + k];
    x[i * n + c] = fma(-f, x[k * n + c], x[i * n + c]);
  }
}

__global__ void k_set_identity(int64_t n, double *x) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n;
       t += (int64_t)gridDim.x * blockDim.x)
    x[t] = (t / n == t % n) ? 1.0 : 0.0;
}

// ---- blocked form (panels of kCb columns): the same factor and inverse in
// about 5 n / kCb launches instead of 6 n.  Per panel K = [k0, k1):
//  k_bchol_panel  every CTA factors the diagonal block A_KK (kCb x kCb) in
//                 shared memory (the same arithmetic in every CTA, every
//                 pivot checked) and solves its rows below the panel,
//                 L_iK = A_iK L_KK^-T (CTA 0 writes L_KK);
//  k_bchol_trail  A_IJ -= L_IK L_JK^T on the lower tiles of the trailing
//                 matrix (32 x 32 tiles, the panel in shared memory).
// Then X = L^-1 by blocked forward substitution (k_btri_diag: X_KC =
// L_KK^-1 X_KC for the columns C < k1; k_btri_update: X_IC -= L_IK X_KC for
// the rows below) and A^-1 = X^T X over the lower tiles, mirrored
// (k_bgram).  FP64 throughout; the sums differ from the column-sweep form
// only in their order.
constexpr int kCb = 32;

// factor the kCb x kCb (or smaller, last panel) block in shared memory with
// one warp; returns false on a non-positive or non-finite pivot
__device__ bool bchol_diag(double (*D)[kCb + 1], int nb) {
  const int lane = threadIdx.x & 31;
  bool ok = true;
  for (int j = 0; j < nb; ++j) {
    const double d = D[j][j];
    if (!(d > 0.0) || !isfinite(d)) ok = false;
    const double ljj = sqrt(d);
    __syncwarp();
    if (lane == j) D[j][j] = ljj;
    if (lane > j && lane < nb) D[lane][j] = D[lane][j] / ljj;
    __syncwarp();
    if (lane > j && lane < nb)
      for (int m = j + 1; m <= lane; ++m) D[lane][m] = fma(-D[lane][j], D[m][j], D[lane][m]);
    __syncwarp();
  }
  return ok;
}

__global__ void __launch_bounds__(256) k_bchol_panel(int64_t n, int64_t k0, double *a, int *bad) {
  __shared__ double D[kCb][kCb + 1];
  if (*bad) return;
  const int nb = (int)(n - k0 < kCb ? n - k0 : kCb);
  const int64_t k1 = k0 + nb;
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int r = t / nb, c = t % nb;
    D[r][c] = c <= r ? a[(k0 + r) * n + k0 + c] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const bool ok = bchol_diag(D, nb);
    if (!ok && threadIdx.x == 0) atomicOr(bad, 1);
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
      const int r = t / nb, c = t % nb;
      if (c <= r) a[(k0 + r) * n + k0 + c] = D[r][c];
    }
  // rows below the panel: x_j = (a_j - sum_{m<j} x_m l_jm) / l_jj
  const int64_t i = k1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[kCb];
  double *row = a + i * n + k0;
#pragma unroll
  for (int j = 0; j < kCb; ++j) x[j] = j < nb ? row[j] : 0.0;
#pragma unroll
  for (int j = 0; j < kCb; ++j) {
    if (j >= nb) break;
    double s = x[j];
#pragma unroll
    for (int m = 0; m < j; ++m) s = fma(-x[m], D[j][m], s);
    x[j] = s / D[j][j];
  }
#pragma unroll
  for (int j = 0; j < kCb; ++j)
    if (j < nb) row[j] = x[j];
}

// lower tiles (I >= J) of the trailing matrix rows/columns >= k1
__global__ void __launch_bounds__(256) k_bchol_trail(int64_t n, int64_t k0, double *a,
                                                     const int *bad) {
  __shared__ double LI[32][kCb + 1], LJ[32][kCb + 1];
  if (*bad) return;
  const int nb = (int)(n - k0 < kCb ? n - k0 : kCb);
  const int64_t k1 = k0 + nb;
  // tile t -> (I, J) with J <= I, row-major over the lower triangle
  const int64_t t = blockIdx.x;
  int64_t I = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while (I * (I + 1) / 2 > t) --I;
  while ((I + 1) * (I + 2) / 2 <= t) ++I;
  const int64_t J = t - I * (I + 1) / 2;
  const int64_t i0 = k1 + I * 32, j0 = k1 + J * 32;
  for (int q = threadIdx.x; q < 32 * kCb; q += blockDim.x) {
    const int r = q / kCb, m = q % kCb;
    LI[r][m] = (i0 + r < n && m < nb) ? a[(i0 + r) * n + k0 + m] : 0.0;
    LJ[r][m] = (j0 + r < n && m < nb) ? a[(j0 + r) * n + k0 + m] : 0.0;
  }
  __syncthreads();
  const int ri = (threadIdx.x >> 4) * 2, cj = (threadIdx.x & 15) * 2;
  double s00 = 0.0, s01 = 0.0, s10 = 0.0, s11 = 0.0;
#pragma unroll
  for (int m = 0; m < kCb; ++m) {
    const double x0 = LI[ri][m], x1 = LI[ri + 1][m], y0 = LJ[cj][m], y1 = LJ[cj + 1][m];
    s00 = fma(x0, y0, s00);
    s01 = fma(x0, y1, s01);
    s10 = fma(x1, y0, s10);
    s11 = fma(x1, y1, s11);
  }
  const double sv[2][2] = {{s00, s01}, {s10, s11}};
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int64_t i = i0 + ri + u, j = j0 + cj + v;
      if (i < n && j <= i) a[i * n + j] -= sv[u][v];
    }
}

// X_KC = L_KK^-1 X_KC for the columns c < k1, one column per thread
__global__ void __launch_bounds__(256) k_btri_diag(int64_t n, int64_t k0, const double *l,
                                                   double *x) {
  __shared__ double D[kCb][kCb + 1];
  const int nb = (int)(n - k0 < kCb ? n - k0 : kCb);
  const int64_t k1 = k0 + nb;
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int r = t / nb, c = t % nb;
    D[r][c] = c <= r ? l[(k0 + r) * n + k0 + c] : 0.0;
  }
  __syncthreads();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k1) return;
  double y[kCb];
#pragma unroll
  for (int j = 0; j < kCb; ++j) y[j] = j < nb ? x[(k0 + j) * n + c] : 0.0;
#pragma unroll
  for (int j = 0; j < kCb; ++j) {
    if (j >= nb) break;
    double s = y[j];
#pragma unroll
    for (int m = 0; m < j; ++m) s = fma(-D[j][m], y[m], s);
    y[j] = s / D[j][j];
  }
#pragma unroll
  for (int j = 0; j < kCb; ++j)
    if (j < nb) x[(k0 + j) * n + c] = y[j];
}

// X_IC -= L_IK X_KC for the rows i >= k1 and the columns c < k1 (32 x 32
// tiles; blockIdx.x over the row tiles, blockIdx.y over the column tiles)
__global__ void __launch_bounds__(256) k_btri_update(int64_t n, int64_t k0, const double *l,
                                                     double *x) {
  __shared__ double LI[32][kCb + 1], XK[kCb][32 + 1];
  const int nb = (int)(n - k0 < kCb ? n - k0 : kCb);
  const int64_t k1 = k0 + nb;
  const int64_t i0 = k1 + (int64_t)blockIdx.x * 32, c0 = (int64_t)blockIdx.y * 32;
  for (int q = threadIdx.x; q < 32 * kCb; q += blockDim.x) {
    const int r = q / kCb, m = q % kCb;
    LI[r][m] = (i0 + r < n && m < nb) ? l[(i0 + r) * n + k0 + m] : 0.0;
    const int mm = q / 32, cc = q % 32;
    XK[mm][cc] = (mm < nb && c0 + cc < k1) ? x[(k0 + mm) * n + c0 + cc] : 0.0;
  }
  __syncthreads();
  const int ri = (threadIdx.x >> 4) * 2, cj = (threadIdx.x & 15) * 2;
  double s00 = 0.0, s01 = 0.0, s10 = 0.0, s11 = 0.0;
#pragma unroll
  for (int m = 0; m < kCb; ++m) {
    const double x0 = LI[ri][m], x1 = LI[ri + 1][m], y0 = XK[m][cj], y1 = XK[m][cj + 1];
    s00 = fma(x0, y0, s00);
    s01 = fma(x0, y1, s01);
    s10 = fma(x1, y0, s10);
    s11 = fma(x1, y1, s11);
  }
  const double sv[2][2] = {{s00, s01}, {s10, s11}};
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int64_t i = i0 + ri + u, c = c0 + cj + v;
      if (i < n && c < k1) x[i * n + c] -= sv[u][v];
    }
}

// inv_ij = sum_k X_ki X_kj (X lower triangular: k >= max(i, j)) on the lower
// tiles, written to both halves
__global__ void __launch_bounds__(256) k_bgram(int64_t n, const double *x, double *inv) {
  __shared__ double XI[32][32 + 1], XJ[32][32 + 1];
  const int64_t t = blockIdx.x;
  int64_t I = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while (I * (I + 1) / 2 > t) --I;
  while ((I + 1) * (I + 2) / 2 <= t) ++I;
  const int64_t J = t - I * (I + 1) / 2;
  const int64_t i0 = I * 32, j0 = J * 32;
  const int ri = (threadIdx.x >> 4) * 2, cj = (threadIdx.x & 15) * 2;
  double s00 = 0.0, s01 = 0.0, s10 = 0.0, s11 = 0.0;
  for (int64_t kb = i0; kb < n; kb += 32) {
    __syncthreads();
    for (int q = threadIdx.x; q < 32 * 32; q += blockDim.x) {
      const int m = q / 32, cc = q % 32;
      const bool in = kb + m < n;
      XI[m][cc] = (in && i0 + cc < n) ? x[(kb + m) * n + i0 + cc] : 0.0;
      XJ[m][cc] = (in && j0 + cc < n) ? x[(kb + m) * n + j0 + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int m = 0; m < 32; ++m) {
      const double x0 = XI[m][ri], x1 = XI[m][ri + 1], y0 = XJ[m][cj], y1 = XJ[m][cj + 1];
      s00 = fma(x0, y0, s00);
      s01 = fma(x0, y1, s01);
      s10 = fma(x1, y0, s10);
      s11 = fma(x1, y1, s11);
    }
  }
  const double sv[2][2] = {{s00, s01}, {s10, s11}};
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int64_t i = i0 + ri + u, j = j0 + cj + v;
      if (i < n && j < n && j <= i) {
        inv[i * n + j] = sv[u][v];
        inv[j * n + i] = sv[u][v];
      }
    }
}

// ===========================================================================
// Banded Cholesky for the standalone solver beyond the dense limit.
// lineal's CholeskySolver (cholesky/decomposition.hpp:52-107) factors row by
// row in the natural order (Cholesky-Banachiewicz, no reordering): row i of
// L fills every column from its first nonzero up to i, so the factor is the
// matrix's lower envelope -- a band of width bw = max_i (i - first column of
// row i).  Here the band is stored by rows, (bw + 1) values per row (column
// j of row i at j - i + bw), and factored with the dense form's 32-column
// panels restricted to the band window: k_band_panel factors the panel's
// diagonal block (in every CTA) and solves the rows below it that reach the
// panel; k_band_trail updates the window below and right of the panel.
// Entries outside the band are exact zeros of the factor and never stored.
// Each solve is a forward and a backward substitution by 32-row blocks in
// one CTA (k_band_fwd, k_band_bwd): a block's products with the band run
// over 32 warps, its triangle in one warp.  FP64 throughout; the sums run in
// another order than lineal's, so results agree to rounding.
// ===========================================================================
struct Band {
  int64_t n, bw, ld;
  double *b;
  __device__ __forceinline__ double get(int64_t i, int64_t j) const {
    return (i - j <= bw && j <= i) ? b[i * ld + (j - i + bw)] : 0.0;
  }
  __device__ __forceinline__ double *at(int64_t i, int64_t j) const {
    return b + i * ld + (j - i + bw);
  }
};

__global__ void k_band_width(int64_t n, const int64_t *rowptr, const int32_t *col,
                             unsigned long long *bw) {
  __shared__ unsigned long long part[8];
  unsigned long long m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (rowptr[i + 1] > rowptr[i]) {
      const int64_t j = col[rowptr[i]];
      if (j < i && (unsigned long long)(i - j) > m) m = (unsigned long long)(i - j);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long q = __shfl_xor_sync(0xffffffffu, m, o);
    m = q > m ? q : m;
  }
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = part[w] > m ? part[w] : m;
    atomicMax(bw, m);
  }
}

// the lower triangle of the CSR matrix into the band (zeros elsewhere)
__global__ void k_band_fill(Band B, const int64_t *rowptr, const int32_t *col, const double *v64,
                            const float *v32) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B.n;
       i += (int64_t)gridDim.x * blockDim.x)
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e) {
      const int64_t j = col[e];
      if (j <= i) *B.at(i, j) = v64 ? v64[e] : (double)v32[e];
    }
}

// panel [k0, k0 + nb): rows [k1, min(n, k1 + bw)) reach it
__global__ void __launch_bounds__(256) k_band_panel(Band B, int64_t k0, int *bad) {
  __shared__ double D[kCb][kCb + 1];
  if (*bad) return;
  const int64_t n = B.n;
  const int nb = (int)(n - k0 < kCb ? n - k0 : kCb);
  const int64_t k1 = k0 + nb, rend = k1 + B.bw < n ? k1 + B.bw : n;
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int r = t / nb, c = t % nb;
    D[r][c] = c <= r ? B.get(k0 + r, k0 + c) : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const bool ok = bchol_diag(D, nb);
    if (!ok && threadIdx.x == 0) atomicOr(bad, 1);
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
      const int r = t / nb, c = t % nb;
      if (c <= r && r - c <= B.bw) *B.at(k0 + r, k0 + c) = D[r][c];
    }
  const int64_t i = k1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rend) return;
  double x[kCb];
#pragma unroll
  for (int j = 0; j < kCb; ++j) x[j] = j < nb ? B.get(i, k0 + j) : 0.0;
#pragma unroll
  for (int j = 0; j < kCb; ++j) {
    if (j >= nb) break;
    double s = x[j];
#pragma unroll
    for (int m = 0; m < j; ++m) s = fma(-x[m], D[j][m], s);
    x[j] = s / D[j][j];
  }
#pragma unroll
  for (int j = 0; j < kCb; ++j)
    if (j < nb && i - (k0 + j) <= B.bw) *B.at(i, k0 + j) = x[j];
}

// the window [k1, rend)^2 (lower tiles): A_ij -= L_iK L_jK^T
__global__ void __launch_bounds__(256) k_band_trail(Band B, int64_t k0, const int *bad) {
  __shared__ double LI[32][kCb + 1], LJ[32][kCb + 1];
  if (*bad) return;
  const int64_t n = B.n;
  const int nb = (int)(n - k0 < kCb ? n - k0 : kCb);
  const int64_t k1 = k0 + nb, rend = k1 + B.bw < n ? k1 + B.bw : n;
  const int64_t t = blockIdx.x;
  int64_t I = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while (I * (I + 1) / 2 > t) --I;
  while ((I + 1) * (I + 2) / 2 <= t) ++I;
  const int64_t J = t - I * (I + 1) / 2;
  const int64_t i0 = k1 + I * 32, j0 = k1 + J * 32;
  for (int q = threadIdx.x; q < 32 * kCb; q += blockDim.x) {
    const int r = q / kCb, m = q % kCb;
    LI[r][m] = (i0 + r < rend && m < nb) ? B.get(i0 + r, k0 + m) : 0.0;
    LJ[r][m] = (j0 + r < rend && m < nb) ? B.get(j0 + r, k0 + m) : 0.0;
  }
  __syncthreads();
  const int ri = (threadIdx.x >> 4) * 2, cj = (threadIdx.x & 15) * 2;
  double s00 = 0.0, s01 = 0.0, s10 = 0.0, s11 = 0.0;
#pragma unroll
  for (int m = 0; m < kCb; ++m) {
    const double x0 = LI[ri][m], x1 = LI[ri + 1][m], y0 = LJ[cj][m], y1 = LJ[cj + 1][m];
    s00 = fma(x0, y0, s00);
    s01 = fma(x0, y1, s01);
    s10 = fma(x1, y0, s10);
    s11 = fma(x1, y1, s11);
  }
  const double sv[2][2] = {{s00, s01}, {s10, s11}};
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int64_t i = i0 + ri + u, j = j0 + cj + v;
      if (i < rend && j <= i) *B.at(i, j) -= sv[u][v];
    }
}

// L y = b by 32-row blocks, one CTA of 1024 threads: warp r sums row
// k0 + r's products with the earlier y, warp 0 then solves the block
__global__ void __launch_bounds__(1024) k_band_fwd(Band B, const double *b, double *y) {
  __shared__ double part[kCb];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int64_t k0 = 0; k0 < B.n; k0 += kCb) {
    const int nb = (int)(B.n - k0 < kCb ? B.n - k0 : kCb);
    if (w < nb) {
      const int64_t i = k0 + w, j0 = i - B.bw > 0 ? i - B.bw : 0;
      double s = 0.0;
      for (int64_t j = j0 + lane; j < k0; j += 32) s = fma(B.get(i, j), y[j], s);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) part[w] = s;
    }
    __syncthreads();
    if (w == 0) {
      double rhs = lane < nb ? b[k0 + lane] - part[lane] : 0.0, yv = 0.0;
      for (int m = 0; m < nb; ++m) {
        const double ym = __shfl_sync(0xffffffffu, rhs / B.get(k0 + m, k0 + m), m);
        if (lane == m) yv = ym;
        if (lane > m && lane < nb) rhs = fma(-B.get(k0 + lane, k0 + m), ym, rhs);
      }
      if (lane < nb) y[k0 + lane] = yv;
    }
    __syncthreads();
  }
}

// L^T x = y by 32-row blocks from the end: warp r sums column k0 + r's
// products with the later x, warp 0 solves the block's transposed triangle
__global__ void __launch_bounds__(1024) k_band_bwd(Band B, const double *y, double *x) {
  __shared__ double part[kCb];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nblk = (B.n + kCb - 1) / kCb;
  for (int64_t K = nblk - 1; K >= 0; --K) {
    const int64_t k0 = K * kCb;
    const int nb = (int)(B.n - k0 < kCb ? B.n - k0 : kCb);
    const int64_t k1 = k0 + nb;
    if (w < nb) {
      const int64_t j = k0 + w, iend = j + B.bw + 1 < B.n ? j + B.bw + 1 : B.n;
      double s = 0.0;
      for (int64_t i = k1 + lane; i < iend; i += 32) s = fma(B.get(i, j), x[i], s);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) part[w] = s;
    }
    __syncthreads();
    if (w == 0) {
      double rhs = lane < nb ? y[k0 + lane] - part[lane] : 0.0, xv = 0.0;
      for (int m = nb - 1; m >= 0; --m) {
        const double xm = __shfl_sync(0xffffffffu, rhs / B.get(k0 + m, k0 + m), m);
        if (lane == m) xv = xm;
        if (lane < m) rhs = fma(-B.get(k0 + m, k0 + lane), xm, rhs);
      }
      if (lane < nb) x[k0 + lane] = xv;
    }
    __syncthreads();
  }
}

// x = A^-1 b, one warp per row
template <typename XT>
__global__ void k_dense_apply(int64_t n, const double *ainv, const XT *b, XT *x) {
  pdl_trigger();
  pdl_wait();
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < n; i += nwarps) {
    double s = 0.0;
    const double *row = ainv + i * n;
    for (int64_t j = lane; j < n; j += 32) s = fma(row[j], (double)b[j], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[i] = (XT)s;
  }
}

// The explicit inverse of the coarsest matrix, applied as one dense product
// per V-cycle (a warp per row: the whole solve is one parallel launch, where
// two triangular solves would be a chain of n dependent steps).  Symmetric
// matrices: the dense FP64 Cholesky factor (CholeskySolver; every pivot
// positive) and the inverse formed from it.  Nonsymmetric: Gauss-Jordan
// elimination without pivoting, LuSolver's elimination order
// (lu/decomposition.hpp:31-122 does not pivot either), refusing pivots that
// are zero, non-finite or tiny against their row.
lgx_status dense_inverse(const Csr &a, cudaStream_t s, DBuf<double> &inv, int spd) {
  const int64_t n = a.n;
  LGX_CHECK(inv.alloc(n * n));
  DBuf<int> bad;
  LGX_CHECK(bad.alloc(1));
  LGX_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  if (n == 0) return LGX_OK;
  if (spd) {
    DBuf<double> l;
    LGX_CHECK(l.alloc(n * n));
    k_dense_from_csr<<<grid_for(n, 128), 128, 0, s>>>(n, a.rowptr.p, a.col.p,
                                                     a.storage == LGX_F64 ? a.v64.p : nullptr,
                                                     a.storage == LGX_F32 ? a.v32.p : nullptr,
                                                     l.p);
    LGX_LAUNCH_CHECK();
    // the blocked form (LGX_BLOCKED_CHOL=0: the column sweeps below)
    static const bool blocked = [] {
      const char *e = std::getenv("LGX_BLOCKED_CHOL");
      return !(e && e[0] == '0');
    }();
    if (blocked) {
      const int64_t npan = (n + kCb - 1) / kCb;
      for (int64_t K = 0; K < npan; ++K) {
        const int64_t k0 = K * kCb, k1 = std::min<int64_t>(k0 + kCb, n), below = n - k1;
        k_bchol_panel<<<(unsigned)std::max<int64_t>(1, (below + 255) / 256), 256, 0, s>>>(
          n, k0, l.p, bad.p);
        if (below > 0) {
          const int64_t T = (below + 31) / 32;
          k_bchol_trail<<<(unsigned)(T * (T + 1) / 2), 256, 0, s>>>(n, k0, l.p, bad.p);
        }
      }
      LGX_LAUNCH_CHECK();
      int h_bad = 0;
      LGX_CUDA(cudaMemcpyAsync(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      LGX_CUDA(cudaStreamSynchronize(s));
      if (h_bad) return fail(LGX_ERR_NOT_SPD, "matrix has a non-positive pivot");
      DBuf<double> xl;
      LGX_CHECK(xl.alloc(n * n));
      k_set_identity<<<(unsigned)std::min<int64_t>(grid_for(n * n, 256), 8192), 256, 0, s>>>(
        n, xl.p);
      for (int64_t K = 0; K < npan; ++K) {
        const int64_t k0 = K * kCb, k1 = std::min<int64_t>(k0 + kCb, n), below = n - k1;
        k_btri_diag<<<(unsigned)((k1 + 255) / 256), 256, 0, s>>>(n, k0, l.p, xl.p);
        if (below > 0)
          k_btri_update<<<dim3((unsigned)((below + 31) / 32), (unsigned)((k1 + 31) / 32)), 256, 0,
                          s>>>(n, k0, l.p, xl.p);
      }
      const int64_t T = (n + 31) / 32;
      k_bgram<<<(unsigned)(T * (T + 1) / 2), 256, 0, s>>>(n, xl.p, inv.p);
      LGX_LAUNCH_CHECK();
      LGX_CUDA(cudaStreamSynchronize(s));
      return LGX_OK;
    }
    for (int64_t k = 0; k < n; ++k) {
      k_chol_column<<<1, 256, 0, s>>>(n, k, l.p, bad.p);
      const int64_t m = n - k - 1;
      if (m > 0)
        k_chol_update<<<(unsigned)std::min<int64_t>(grid_for(m * m, 256), 4096), 256, 0, s>>>(
          n, k, l.p, bad.p);
    }
    LGX_LAUNCH_CHECK();
    int h_bad = 0;
    LGX_CUDA(cudaMemcpyAsync(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    LGX_CUDA(cudaStreamSynchronize(s));
    if (h_bad) return fail(LGX_ERR_NOT_SPD, "matrix has a non-positive pivot");
    // inv = I, then inv = L^-1 inv, then inv = L^-T inv
    k_set_identity<<<(unsigned)std::min<int64_t>(grid_for(n * n, 256), 8192), 256, 0, s>>>(
      n, inv.p);
    LGX_LAUNCH_CHECK();
    const unsigned gs = (unsigned)std::min<int64_t>(grid_for(n, 256), 64);
    for (int64_t k = 0; k < n; ++k) {
      k_tri_scale<<<gs, 256, 0, s>>>(n, k, l.p, inv.p);
      const int64_t rows = n - k - 1;
      if (rows > 0)
        k_tri_update<<<(unsigned)std::min<int64_t>(grid_for(rows * n, 256), 4096), 256, 0, s>>>(
          n, k, k + 1, n, 0, l.p, inv.p);
    }
    LGX_LAUNCH_CHECK();
    for (int64_t k = n - 1; k >= 0; --k) {
      k_tri_scale<<<gs, 256, 0, s>>>(n, k, l.p, inv.p);
      if (k > 0)
        k_tri_update<<<(unsigned)std::min<int64_t>(grid_for(k * n, 256), 4096), 256, 0, s>>>(
          n, k, 0, k, 1, l.p, inv.p);
    }
    LGX_LAUNCH_CHECK();
    LGX_CUDA(cudaStreamSynchronize(s));
    return LGX_OK;
  }
  DBuf<double> prow, pcol;
  LGX_CHECK(prow.alloc(n));
  LGX_CHECK(pcol.alloc(n));
  k_dense_from_csr<<<grid_for(n, 128), 128, 0, s>>>(n, a.rowptr.p, a.col.p,
                                                   a.storage == LGX_F64 ? a.v64.p : nullptr,
                                                   a.storage == LGX_F32 ? a.v32.p : nullptr,
                                                   inv.p);
  LGX_LAUNCH_CHECK();
  const unsigned g1 = (unsigned)std::min<int64_t>(grid_for(n, 256), 1024);
  const unsigned g2 = (unsigned)std::min<int64_t>(grid_for(n * n, 256), 4096);
  for (int64_t k = 0; k < n; ++k) {
    k_gj_pivot<<<g1, 256, 0, s>>>(n, k, inv.p, prow.p, pcol.p, bad.p);
    k_gj_update<<<g2, 256, 0, s>>>(n, k, inv.p, prow.p, pcol.p, bad.p);
  }
  LGX_LAUNCH_CHECK();
  int h_bad = 0;
  LGX_CUDA(cudaMemcpyAsync(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  if (h_bad)
    return fail(LGX_ERR_BREAKDOWN,
                "matrix has a zero, non-finite or tiny pivot (unpivoted elimination)");
  return LGX_OK;
}

// the coarsest level: CholeskySolver for symmetric hierarchies, LuSolver for
// nonsymmetric ones (test/aux/default.hpp:160-162)
lgx_status dense_inverse(const Csr &a, cudaStream_t s, DBuf<double> &inv) {
  const lgx_status st = dense_inverse(a, s, inv, a.symmetric ? 1 : 0);
  if (st == LGX_ERR_NOT_SPD || st == LGX_ERR_BREAKDOWN)
    return fail(st, "coarsest " + std::string(lgx_last_error()));
  return st;
}

// ===========================================================================
// Transfers in the colour-permuted spaces of two consecutive levels
// ===========================================================================
// agg_p[i'] = permuted coarse id of the aggregate of fine row perm_f[i']
__global__ void k_agg_permute(int64_t n, const int32_t *perm_f, const uint32_t *agg,
                              const int32_t *iperm_c, uint32_t *agg_p) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm_f ? perm_f[r] : r;
    const uint32_t a = agg[i];
    agg_p[r] = a < kIsolated ? (iperm_c ? (uint32_t)iperm_c[a] : a) : kIsolated;
  }
}

__global__ void k_rlist_len(int64_t nc, const int32_t *perm_c, const int64_t *list_ptr,
                            int64_t *len) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nc;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = perm_c ? perm_c[r] : r;
    len[r] = list_ptr[c + 1] - list_ptr[c];
  }
}

__global__ void k_rlist_fill(int64_t nc, const int32_t *perm_c, const int64_t *list_ptr,
                             const int32_t *list, const int32_t *iperm_f, const int64_t *rptr,
                             int32_t *rlist) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nc;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = perm_c ? perm_c[r] : r;
    int64_t o = rptr[r];
    for (int64_t k = list_ptr[c]; k < list_ptr[c + 1]; ++k, ++o)
      rlist[o] = iperm_f ? iperm_f[list[k]] : list[k];
  }
}

// coarse b[I'] = sum over the aggregate's fine rows (list order) of r
// (vector-shared.hpp:49-56)
template <typename XT>
__global__ void k_restrict(int64_t nc, const int64_t *rptr, const int32_t *rlist,
                           const XT *__restrict__ r, XT *__restrict__ bc) {
  pdl_trigger();
  pdl_wait();
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    XT s = XT(0);
    for (int64_t k = rptr[c]; k < rptr[c + 1]; ++k) s = s + r[rlist[k]];
    bc[c] = s;
  }
}

// x_f += inv_relax * refine(x_c) (vector-shared.hpp:121-134, solver.hpp:129-136)
template <typename XT>
__global__ void k_prolong(int64_t n, const uint32_t *__restrict__ agg_p, const XT *__restrict__ xc,
                          XT inv_relax, XT *__restrict__ x) {
  pdl_trigger();
  pdl_wait();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t a = agg_p[i];
    const XT ref = a < kIsolated ? xc[a] : XT(0);
    x[i] = x[i] + ref * inv_relax;
  }
}

template <typename T, typename U>
__global__ void k_convert(int64_t n, const T *src, U *dst) {
  pdl_trigger();
  pdl_wait();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (U)src[i];
}

}  // namespace lgx

// ===========================================================================
// Hierarchy
// ===========================================================================
namespace lgx {

int64_t amg_partitions(int64_t n, int64_t level, const lgx_amg_params &p) {
  double ps = (double)p.partition_size;
  for (int64_t l = 0; l < level; ++l) ps *= p.partition_growth;
  int64_t parts = ps >= 1.0 ? (int64_t)((double)n / ps) : n;
  const int64_t floor_parts = p.min_partitions < n / 1024 ? p.min_partitions : n / 1024;
  if (parts < floor_parts) parts = floor_parts;
  if (parts < 1) parts = 1;
  if (parts > p.max_partitions) parts = p.max_partitions;
  return parts;
}

// Setup phase timer (LGX_VERBOSE=1 prints the phases to stderr).
struct PhaseTimer {
  bool on = std::getenv("LGX_VERBOSE") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(cudaStream_t s, const char *what, int64_t level) {
    if (!on) return;
    cudaStreamSynchronize(s);
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[lgx setup] level %lld %-12s %9.2f ms\n", (long long)level, what,
                 std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};

// A given aggregate map (host arrays) checked and copied into `out` in place
// of strength + aggregation (FileAggregator, aggregation/independent.hpp:
// 279-298).  The checks make it what aggregation produces: every id below
// ncoarse or isolated, every aggregated vertex in exactly the list of its
// aggregate, no empty aggregate; the later kernels index with these ids.
static lgx_status check_map(const lgx_agg_map &m, int64_t n, const std::string &where) {
  if (m.n != n) return fail(LGX_ERR_INVALID, where + "fine size does not match the level");
  if (m.ncoarse < 1 && n > 0) return fail(LGX_ERR_INVALID, where + "no aggregates");
  if (m.ncoarse < 0 || m.ncoarse > (int64_t)kIsolated || (n > 0 && !m.agg) || !m.list_ptr)
    return fail(LGX_ERR_INVALID, where + "missing arrays or bad coarse size");
  const int64_t nc = m.ncoarse;
  if (m.list_ptr[0] != 0) return fail(LGX_ERR_INVALID, where + "list offsets must start at 0");
  int64_t aggregated = 0;
  for (int64_t v = 0; v < n; ++v) {
    if (m.agg[v] == kIsolated) continue;
    if ((int64_t)m.agg[v] >= nc) return fail(LGX_ERR_INVALID, where + "aggregate id out of range");
    ++aggregated;
  }
  if (m.list_ptr[nc] != aggregated)
    return fail(LGX_ERR_INVALID, where + "lists do not cover the aggregated vertices");
  if (aggregated > 0 && !m.list) return fail(LGX_ERR_INVALID, where + "missing lists");
  std::vector<uint8_t> seen((size_t)std::max<int64_t>(n, 1), 0);
  for (int64_t c = 0; c < nc; ++c) {
    if (m.list_ptr[c + 1] <= m.list_ptr[c])
      return fail(LGX_ERR_INVALID, where + "empty or decreasing aggregate list");
    for (int64_t k = m.list_ptr[c]; k < m.list_ptr[c + 1]; ++k) {
      const int32_t v = m.list[k];
      if (v < 0 || v >= n || seen[(size_t)v] || (int64_t)m.agg[v] != c)
        return fail(LGX_ERR_INVALID, where + "list entry out of range, repeated or misplaced");
      seen[(size_t)v] = 1;
    }
  }
  return LGX_OK;
}

static lgx_status upload_map(const lgx_agg_map &m, int64_t level, int64_t n, cudaStream_t s,
                             AggResult &out) {
  LGX_CHECK(check_map(m, n, "aggregate map of level " + std::to_string(level) + ": "));
  const int64_t nc = m.ncoarse, aggregated = m.list_ptr[nc];
  LGX_CHECK(out.agg.alloc(n));
  LGX_CHECK(out.list_ptr.alloc(nc + 1));
  LGX_CHECK(out.list.alloc(aggregated));
  if (n > 0)
    LGX_CUDA(cudaMemcpyAsync(out.agg.p, m.agg, sizeof(uint32_t) * (size_t)n,
                             cudaMemcpyHostToDevice, s));
  LGX_CUDA(cudaMemcpyAsync(out.list_ptr.p, m.list_ptr, sizeof(int64_t) * (size_t)(nc + 1),
                           cudaMemcpyHostToDevice, s));
  if (aggregated > 0)
    LGX_CUDA(cudaMemcpyAsync(out.list.p, m.list, sizeof(int32_t) * (size_t)aggregated,
                             cudaMemcpyHostToDevice, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  out.ncoarse = nc;
  for (auto &x : out.stats) x = 0;
  return LGX_OK;
}

// a level's smallest-last colouring: its pattern to the host,
// lgx_colour_smallest_last there, the colours back to the device
lgx_status colour_smallest_last(int64_t n, const int64_t *rowptr, const int32_t *col,
                                int32_t *colour, int32_t *ncolours, bool known_symmetric);

static lgx_status colouring_smallest_last(const Csr &a, cudaStream_t s, DBuf<int32_t> &colour,
                                          int32_t &ncolours) {
  const int64_t n = a.n;
  std::vector<int64_t> rowptr((size_t)n + 1);
  std::vector<int32_t> col((size_t)std::max<int64_t>(a.nnz, 1));
  std::vector<int32_t> h_colour((size_t)std::max<int64_t>(n, 1));
  LGX_CUDA(cudaMemcpyAsync(rowptr.data(), a.rowptr.p, sizeof(int64_t) * (size_t)(n + 1),
                           cudaMemcpyDeviceToHost, s));
  if (a.nnz > 0)
    LGX_CUDA(cudaMemcpyAsync(col.data(), a.col.p, sizeof(int32_t) * (size_t)a.nnz,
                             cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  LGX_CHECK(colour_smallest_last(n, rowptr.data(), col.data(), h_colour.data(), &ncolours,
                                 a.symmetric != 0));
  LGX_CHECK(colour.alloc(n));
  if (n > 0)
    LGX_CUDA(cudaMemcpyAsync(colour.p, h_colour.data(), sizeof(int32_t) * (size_t)n,
                             cudaMemcpyHostToDevice, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  return LGX_OK;
}

static lgx_status amg_build(const lgx_matrix *m, const lgx_amg_params &p,
                            const lgx_colouring *finest_colouring, const lgx_agg_map *maps,
                            int64_t nmaps, cudaStream_t s, lgx_amg &h) {
  PhaseTimer timer;
  h.p = p;
  h.f32 = p.cycle_f32 != 0;
  auto l0 = std::make_unique<lgx_amg_level>();
  // a stencil finest level: its assembled CSR serves the setup (strength,
  // aggregation, Galerkin product) and is released afterwards
  std::unique_ptr<lgx_matrix, lgx_status (*)(lgx_matrix *)> assembled(nullptr,
                                                                       lgx_matrix_destroy);
  if (m->kind != LGX_MATRIX_CSR) {
    if (p.cycle_f32)
      return fail(LGX_ERR_UNSUPPORTED, "a stencil finest level runs the FP64 cycle");
    lgx_matrix *tmp = nullptr;
    LGX_CHECK(lgx_stencil_to_csr(m, nullptr, s, &tmp));
    assembled.reset(tmp);
    if (tmp->n != m->n)
      return fail(LGX_ERR_UNSUPPORTED,
                  "stencil rows with a zero diagonal (ZeroToZero) have no assembled row");
    l0->a = &tmp->csr;
    l0->stencil = m;
    timer.mark(s, "assemble", 0);
  } else {
    l0->a = &m->csr;
  }
  h.lv.push_back(std::move(l0));
  bool aggressive = false;
  for (int64_t level = 0;; ++level) {
    lgx_amg_level &fine = *h.lv[level];
    const Csr &a = *fine.a;
    if (level < 32) {
      h.aggressive[level] = aggressive;
      h.given[level] = maps != nullptr;
    }
    if (maps) {
      if (level >= nmaps)
        return fail(LGX_ERR_INVALID, "no aggregate map for level " + std::to_string(level));
      LGX_CHECK(upload_map(maps[level], level, a.n, s, fine.agg));
      timer.mark(s, "given map", level);
    } else {
      DBuf<uint8_t> dep, inf, iso;
      LGX_CHECK(dep.alloc(a.nnz));
      LGX_CHECK(inf.alloc(a.nnz));
      LGX_CHECK(iso.alloc(a.n));
      LGX_CHECK(strength(a, aggressive ? p.aggressive_threshold : p.strong_threshold, dep.p,
                         inf.p, iso.p, s));
      timer.mark(s, "strength", level);
      LGX_CHECK(aggregate(a, dep.p, inf.p, iso.p, p.min_aggregate_size, p.max_aggregate_size,
                          amg_partitions(a.n, level, p), aggressive, s, fine.agg));
      timer.mark(s, "aggregate", level);
    }
    if (level < 32)
      for (int k = 0; k < 5; ++k) h.stats[level][k] = fine.agg.stats[k];
    if (fine.agg.ncoarse == 0 && a.n > 0)
      return fail(LGX_ERR_INVALID, "aggregation produced no aggregates (all rows isolated)");
    auto coarse = std::make_unique<lgx_amg_level>();
    LGX_CHECK(galerkin(a, fine.agg, p.coarse_f32, s, coarse->own));
    timer.mark(s, "galerkin", level);
    coarse->a = &coarse->own;
    const int64_t fsize = a.n, csize = coarse->own.n;
    h.lv.push_back(std::move(coarse));
    // level_action (hierarchy/wright.hpp:120-143)
    bool stop = false;
    if (csize < p.min_coarsen_size) {
      stop = true;
      h.stop_reason = LGX_STOP_TOO_SMALL;
    } else if (level + 1 >= p.max_level_num) {
      stop = true;
      h.stop_reason = LGX_STOP_TOO_MANY_LEVELS;
    } else if (p.min_coarsen_factor * (double)csize > (double)fsize) {
      if (aggressive) {
        stop = true;
        h.stop_reason = LGX_STOP_TOO_SMALL_RATE;
      } else {
        aggressive = true;
      }
    }
    if (!stop && level + 2 >= 32) {
      stop = true;
      h.stop_reason = LGX_STOP_LEVEL_CAP;
    }
    if (stop) break;
  }
  const int64_t L = (int64_t)h.lv.size();
  // smoother colourings (all but the coarsest level)
  for (int64_t l = 0; l + 1 < L; ++l) {
    lgx_amg_level &lv = *h.lv[l];
    if (lv.stencil) {
      // matrix-free red-black sweeps in natural order: the permutation of
      // the transfers is the identity
      lgx_colouring *rb = nullptr;
      LGX_CHECK(lgx_colouring_create_red_black(lv.stencil, s, &rb));
      lv.col.reset(rb);
      const int64_t n = lv.a->n;
      LGX_CHECK(rb->perm.alloc(n));
      LGX_CHECK(rb->iperm.alloc(n));
      if (n) {
        k_iota<<<std::min<int64_t>(grid_for(n, 256), 16384), 256, 0, s>>>(n, rb->perm.p);
        LGX_LAUNCH_CHECK();
        k_iota<<<std::min<int64_t>(grid_for(n, 256), 16384), 256, 0, s>>>(n, rb->iperm.p);
        LGX_LAUNCH_CHECK();
      }
      timer.mark(s, "colouring", l);
      continue;
    }
    lv.col = std::make_unique<lgx_colouring>();
    if (l == 0 && finest_colouring) {
      LGX_CHECK(colouring_build(*lv.a, finest_colouring->colour.p, finest_colouring->ncolours, s,
                                *lv.col));
    } else {
      int32_t nc = 0;
      if (l > 0 && p.coarse_smallest_last)
        LGX_CHECK(colouring_smallest_last(*lv.a, s, lv.col->colour, nc));
      else
        LGX_CHECK(colouring_jp(*lv.a, p.colour_seed + (uint64_t)l, s, lv.col->colour, nc));
      LGX_CHECK(colouring_build(*lv.a, lv.col->colour.p, nc, s, *lv.col));
    }
    if (h.f32) LGX_CHECK(colouring_make_f32(*lv.col, s));
    if (h.f32 && p.cycle_bf16) LGX_CHECK(colouring_make_bf16(*lv.col, s));
    if (l == 0 && p.grid27 && m->grid_points) {
      bool attached = false;
      LGX_CHECK(grid27_attach(*lv.col, m->grid_dims, m->grid_points, s, &attached));
    }
    timer.mark(s, "colouring", l);
  }
  // transfers in permuted spaces
  for (int64_t l = 0; l + 1 < L; ++l) {
    lgx_amg_level &f = *h.lv[l];
    lgx_amg_level &c = *h.lv[l + 1];
    const int32_t *perm_c = c.col ? c.col->perm.p : nullptr;
    const int32_t *iperm_c = c.col ? c.col->iperm.p : nullptr;
    const int64_t nf = f.a->n, nc = c.a->n;
    LGX_CHECK(f.agg_p.alloc(nf));
    k_agg_permute<<<std::min<int64_t>(grid_for(nf, 256), 16384), 256, 0, s>>>(
      nf, f.col->perm.p, f.agg.agg.p, iperm_c, f.agg_p.p);
    LGX_LAUNCH_CHECK();
    DBuf<int64_t> len;
    LGX_CHECK(len.alloc(nc));
    LGX_CHECK(f.rptr.alloc(nc + 1));
    if (nc) {
      k_rlist_len<<<std::min<int64_t>(grid_for(nc, 256), 16384), 256, 0, s>>>(
        nc, perm_c, f.agg.list_ptr.p, len.p);
      LGX_LAUNCH_CHECK();
    }
    LGX_CHECK(inclusive_offsets(nc, len.p, f.rptr.p, s));
    const int64_t total = f.agg.list.n;
    LGX_CHECK(f.rlist.alloc(total));
    if (nc) {
      k_rlist_fill<<<std::min<int64_t>(grid_for(nc, 256), 16384), 256, 0, s>>>(
        nc, perm_c, f.agg.list_ptr.p, f.agg.list.p, f.col->iperm.p, f.rptr.p, f.rlist.p);
      LGX_LAUNCH_CHECK();
    }
    LGX_CUDA(cudaStreamSynchronize(s));
  }
  // cycle vectors
  for (int64_t l = 0; l < L; ++l) {
    lgx_amg_level &lv = *h.lv[l];
    const int64_t n = lv.a->n;
    if (h.f32) {
      LGX_CHECK(lv.b32.alloc(n));
      LGX_CHECK(lv.x32.alloc(n));
      LGX_CHECK(lv.r32.alloc(n));
    } else {
      LGX_CHECK(lv.b64.alloc(n));
      LGX_CHECK(lv.x64.alloc(n));
      LGX_CHECK(lv.r64.alloc(n));
    }
  }
  timer.mark(s, "transfers", -1);
  LGX_CHECK(dense_inverse(*h.lv[L - 1]->a, s, h.inv));
  timer.mark(s, "coarse_inv", L - 1);
  if (assembled && L > 1) {
    // keep the sizes of the assembled finest matrix, release its arrays
    lgx_amg_level &l0 = *h.lv[0];
    l0.own.n = assembled->csr.n;
    l0.own.nnz = assembled->csr.nnz;
    l0.own.symmetric = assembled->csr.symmetric;
    l0.a = &l0.own;
    LGX_CUDA(cudaStreamSynchronize(s));
    assembled.reset();
  } else if (assembled) {
    // a one-level hierarchy keeps the assembled matrix as its (coarsest) level
    lgx_amg_level &l0 = *h.lv[0];
    l0.own = std::move(assembled->csr);
    l0.a = &l0.own;
    l0.stencil = nullptr;
  }
  return LGX_OK;
}

// Smoother sweep / residual on one level with the level's value storage:
// double cycles read the stored values (double or float), float cycles read
// float values (the stored floats or the float copy of a double level).
template <typename XT>
static lgx_status level_sor(lgx_amg_level &lv, const lgx_amg &h, int forward, const XT *b, XT *x,
                            cudaStream_t s, int from_zero = 0, XT *r_last = nullptr,
                            int64_t *res_from = nullptr) {
  if (res_from) *res_from = lv.a->n;
  const lgx_colouring &c = *lv.col;
  const double relax = h.p.smoother_relax;
  const int ultra = h.p.smoother_ultra;
  if (lv.stencil) {
    if constexpr (sizeof(XT) == 8)
      return stencil_sor_sweep(lv.stencil, relax, forward, ultra, from_zero ? nullptr : x, x, b,
                               s);
    else
      return fail(LGX_ERR_UNSUPPORTED, "a stencil finest level runs the FP64 cycle");
  }
  if constexpr (sizeof(XT) == 8) {
    if (c.pcsr.storage == LGX_F64)
      return mc_sor_sweep<double, double>(c, c.pcsr.v64.p, relax, forward, ultra, b, x, s,
                                          from_zero, nullptr, r_last, res_from);
    return mc_sor_sweep<float, double>(c, c.pcsr.v32.p, relax, forward, ultra, b, x, s,
                                       from_zero, nullptr, r_last, res_from);
  } else {
    if (h.p.cycle_bf16)
      return mc_sor_sweep<bf16, float>(c, c.pv16.p, relax, forward, ultra, b, x, s, from_zero,
                                       c.pscale.p);
    const float *v = c.pcsr.storage == LGX_F32 ? c.pcsr.v32.p : c.pv32.p;
    return mc_sor_sweep<float, float>(c, v, relax, forward, ultra, b, x, s, from_zero, nullptr,
                                      r_last, res_from);
  }
}

// The residual of rows [0, rend) of a level whose sweep left the residuals
// of its last colour (rows rend on) already; the whole residual when rend
// is the level's size.
template <typename XT>
static lgx_status level_residual_part(lgx_amg_level &lv, const lgx_amg &h, const XT *b,
                                      const XT *x, XT *r, int64_t rend, cudaStream_t s);

template <typename XT>
static lgx_status level_residual(lgx_amg_level &lv, const lgx_amg &h, const XT *b, const XT *x,
                                 XT *r, cudaStream_t s) {
  const lgx_colouring &c = *lv.col;
  if (lv.stencil) {
    if constexpr (sizeof(XT) == 8)
      return matrix_residual(lv.stencil, b, x, r, nullptr, nullptr, nullptr, s);
    else
      return fail(LGX_ERR_UNSUPPORTED, "a stencil finest level runs the FP64 cycle");
  }
  if constexpr (sizeof(XT) == 8) {
    if (c.pcsr.storage == LGX_F64)
      return csr_residual<double, double>(c.pcsr, c.pcsr.v64.p, b, x, r, nullptr, nullptr,
                                          nullptr, s);
    return csr_residual<float, double>(c.pcsr, c.pcsr.v32.p, b, x, r, nullptr, nullptr, nullptr,
                                       s);
  } else {
    if (h.p.cycle_bf16)
      return csr_residual<bf16, float>(c.pcsr, c.pv16.p, b, x, r, nullptr, nullptr, nullptr, s,
                                       c.pscale.p);
    const float *v = c.pcsr.storage == LGX_F32 ? c.pcsr.v32.p : c.pv32.p;
    return csr_residual<float, float>(c.pcsr, v, b, x, r, nullptr, nullptr, nullptr, s);
  }
}

template <typename XT>
static lgx_status level_residual_part(lgx_amg_level &lv, const lgx_amg &h, const XT *b,
                                      const XT *x, XT *r, int64_t rend, cudaStream_t s) {
  if (rend >= lv.a->n) return level_residual<XT>(lv, h, b, x, r, s);
  const lgx_colouring &c = *lv.col;
  bool done = false;
  if constexpr (sizeof(XT) == 8) {
    if (c.pcsr.storage == LGX_F64)
      LGX_CHECK((grid_residual_rows<double, double>(c.pcsr, c.pcsr.v64.p, b, x, r, 0, rend, s,
                                                    &done)));
    else
      LGX_CHECK((grid_residual_rows<float, double>(c.pcsr, c.pcsr.v32.p, b, x, r, 0, rend, s,
                                                   &done)));
  } else {
    const float *v = c.pcsr.storage == LGX_F32 ? c.pcsr.v32.p : c.pv32.p;
    LGX_CHECK((grid_residual_rows<float, float>(c.pcsr, v, b, x, r, 0, rend, s, &done)));
  }
  // the sweep wrote residuals only through the grid rows this residual uses
  if (!done) return fail(LGX_ERR_INVALID, "partial residual without grid rows");
  return LGX_OK;
}

template <typename XT>
static XT *level_vec(lgx_amg_level &lv, int which) {
  if constexpr (sizeof(XT) == 8) {
    return which == 0 ? (XT *)lv.b64.p : which == 1 ? (XT *)lv.x64.p : (XT *)lv.r64.p;
  } else {
    return which == 0 ? (XT *)lv.b32.p : which == 1 ? (XT *)lv.x32.p : (XT *)lv.r32.p;
  }
}

// the residuals of a forward sweep's last colour from its own kernel
// (LGX_FUSED_RESIDUAL=0: a separate residual pass over every row)
static bool fused_residual_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("LGX_FUSED_RESIDUAL");
    return !(e && e[0] == '0');
  }();
  return on;
}

// V-cycle in permuted space (multigrid/solver.hpp:56-176, REGULAR cycle with
// one iteration): forward SOR from zero, residual restricted by aggregate
// sums, dense coarsest solve, correction injected with 1/relax, backward SOR
// in place.  b0/x0 are the finest-level vectors (permuted order).
template <typename XT>
static lgx_status vcycle_impl(lgx_amg &h, const XT *b0, XT *x0, cudaStream_t s) {
  const int64_t L = (int64_t)h.lv.size();
  for (int64_t l = 0; l + 1 < L; ++l) {
    lgx_amg_level &lv = *h.lv[l];
    const XT *b = l == 0 ? b0 : level_vec<XT>(lv, 0);
    XT *x = l == 0 ? x0 : level_vec<XT>(lv, 1);
    const int64_t n = lv.a->n;
    if (n == 0) continue;
    // forward sweep from x = 0; its last colour, on float 7-point grid rows,
    // also leaves its rows' residuals, so the residual pass covers the rows
    // before it
    XT *r = level_vec<XT>(lv, 2);
    int64_t res_from = n;
    LGX_CHECK(level_sor<XT>(lv, h, 1, b, x, s, 1, fused_residual_enabled() ? r : nullptr,
                            &res_from));
    LGX_CHECK(level_residual_part<XT>(lv, h, b, x, r, res_from, s));
    lgx_amg_level &cv = *h.lv[l + 1];
    const int64_t nc = cv.a->n;
    if (nc) {
      LGX_CUDA(launch_pdl(sizeof(XT) == 4 || nc <= pdl_fp64_rows(), k_restrict<XT>,
                          dim3(std::min<int64_t>(grid_for(nc, 128), 65535)),
                          dim3(128), 0, s, nc, (const int64_t *)lv.rptr.p,
                          (const int32_t *)lv.rlist.p, (const XT *)level_vec<XT>(lv, 2),
                          level_vec<XT>(cv, 0)));
      count_launch();
    }
  }
  {
    lgx_amg_level &last = *h.lv[L - 1];
    const int64_t nc = last.a->n;
    if (nc) {
      XT *bl = L == 1 ? const_cast<XT *>(b0) : level_vec<XT>(last, 0);
      XT *xl = L == 1 ? x0 : level_vec<XT>(last, 1);
      LGX_CUDA(launch_pdl(sizeof(XT) == 4 || nc <= pdl_fp64_rows(), k_dense_apply<XT>,
                          dim3((unsigned)std::min<int64_t>(grid_for(nc * 32, 256), 4096)),
                          dim3(256), 0, s, nc, (const double *)h.inv.p, (const XT *)bl, xl));
      count_launch();
    }
  }
  const XT inv_relax = (XT)(1.0 / h.p.relax);
  for (int64_t l = L - 2; l >= 0; --l) {
    lgx_amg_level &lv = *h.lv[l];
    const XT *b = l == 0 ? b0 : level_vec<XT>(lv, 0);
    XT *x = l == 0 ? x0 : level_vec<XT>(lv, 1);
    const int64_t n = lv.a->n;
    if (n == 0) continue;
    LGX_CUDA(launch_pdl(sizeof(XT) == 4 || n <= pdl_fp64_rows(), k_prolong<XT>,
                        dim3(std::min<int64_t>(grid_for(n, 256), 65535)),
                        dim3(256), 0, s, n, (const uint32_t *)lv.agg_p.p,
                        (const XT *)level_vec<XT>(*h.lv[l + 1], 1), inv_relax, x));
    count_launch();
    LGX_CHECK(level_sor<XT>(lv, h, 0, b, x, s));
  }
  return LGX_OK;
}

const Csr &amg_finest_permuted(const lgx_amg &h) { return h.lv[0]->col->pcsr; }
lgx_colouring *amg_finest_colouring(lgx_amg &h) { return h.lv[0]->col.get(); }

// Applies the preconditioner in the finest level's permuted space with
// double vectors (the outer Krylov vectors).
lgx_status amg_apply_permuted(lgx_amg &h, const double *b, double *x, cudaStream_t s) {
  lgx_amg_level &l0 = *h.lv[0];
  const int64_t n = l0.a->n;
  if (!h.f32) return vcycle_impl<double>(h, b, x, s);
  LGX_CUDA(launch_pdl(true, k_convert<double, float>,
                      dim3(std::min<int64_t>(grid_for(n, 256), 16384)),
                      dim3(256), 0, s, n, b, l0.b32.p));
  count_launch();
  LGX_CHECK(vcycle_impl<float>(h, l0.b32.p, l0.x32.p, s));
  LGX_CUDA(launch_pdl(true, k_convert<float, double>,
                      dim3(std::min<int64_t>(grid_for(n, 256), 16384)),
                      dim3(256), 0, s, n, (const float *)l0.x32.p, x));
  count_launch();
  return LGX_OK;
}

// The float V-cycle on float vectors of the finest level's permuted space
// (the inner solves of the refinement driver); needs a cycle_f32 hierarchy.
bool amg_cycle_f32(const lgx_amg &h) { return h.f32; }
lgx_status amg_apply_permuted_f32(lgx_amg &h, const float *b, float *x, cudaStream_t s) {
  if (!h.f32) return fail(LGX_ERR_UNSUPPORTED, "float V-cycle needs a cycle_f32 hierarchy");
  return vcycle_impl<float>(h, b, x, s);
}
// float values of the finest permuted matrix (the cycle's own copy)
const float *amg_finest_values_f32(const lgx_amg &h) {
  const lgx_colouring &c = *h.lv[0]->col;
  return c.pcsr.storage == LGX_F32 ? c.pcsr.v32.p : c.pv32.p;
}

}  // namespace lgx

using namespace lgx;

extern "C" {

void lgx_amg_default_params(lgx_amg_params *p) {
  if (!p) return;
  p->min_aggregate_size = 6;
  p->max_aggregate_size = 9;
  p->partition_size = 4096;
  p->partition_growth = 4.0;
  p->min_partitions = 8;
  p->max_partitions = 1 << 30;
  p->strong_threshold = 1.0 / 3.0;
  p->aggressive_threshold = 1.0 / 3.0;
  p->max_level_num = 16;
  p->min_coarsen_size = 2000;
  p->min_coarsen_factor = 1.2;
  p->coarse_f32 = 0;
  p->cycle_f32 = 0;
  p->relax = 1.0;
  p->smoother_relax = 1.0;
  p->smoother_ultra = 0;
  p->colour_seed = 0x5eed;
  p->cycle_bf16 = 0;
  p->grid27 = 1;
  p->coarse_smallest_last = 0;
}

static lgx_status amg_setup(const lgx_matrix *a, const lgx_amg_params *p,
                            const lgx_colouring *finest_colouring, const lgx_agg_map *maps,
                            int64_t nmaps, lgx_stream stream, lgx_amg **out) {
  if (!a || !p || !out) return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind != LGX_MATRIX_CSR && finest_colouring && !finest_colouring->stencil_rb)
    return fail(LGX_ERR_INVALID, "a stencil finest level takes its red-black colouring");
  if (finest_colouring && finest_colouring->n != a->n)
    return fail(LGX_ERR_INVALID, "finest colouring does not match the matrix");
  if (p->max_aggregate_size > 64 || p->min_aggregate_size < 1 ||
      p->min_aggregate_size > p->max_aggregate_size)
    return fail(LGX_ERR_INVALID, "aggregate sizes must satisfy 1 <= min <= max <= 64");
  if (!(p->relax != 0.0)) return fail(LGX_ERR_INVALID, "relax must be non-zero");
  if (!(p->partition_growth >= 1.0))
    return fail(LGX_ERR_INVALID, "partition_growth must be at least 1");
  auto *h = new lgx_amg();
  lgx_status st = amg_build(a, *p, finest_colouring, maps, nmaps, stream, *h);
  if (st != LGX_OK) {
    delete h;
    return st;
  }
  *out = h;
  return LGX_OK;
}

lgx_status lgx_amg_setup(const lgx_matrix *a, const lgx_amg_params *p,
                         const lgx_colouring *finest_colouring, lgx_stream stream,
                         lgx_amg **out) {
  return amg_setup(a, p, finest_colouring, nullptr, 0, stream, out);
}

lgx_status lgx_agg_map_check(const lgx_agg_map *m, int64_t n) {
  if (!m) return fail(LGX_ERR_INVALID, "null aggregate map");
  return check_map(*m, n, "aggregate map: ");
}

lgx_status lgx_amg_setup_given(const lgx_matrix *a, const lgx_amg_params *p,
                               const lgx_colouring *finest_colouring, const lgx_agg_map *maps,
                               int64_t nmaps, lgx_stream stream, lgx_amg **out) {
  if (!maps || nmaps < 1) return fail(LGX_ERR_INVALID, "no aggregate maps given");
  return amg_setup(a, p, finest_colouring, maps, nmaps, stream, out);
}

lgx_status lgx_amg_destroy(lgx_amg *h) {
  delete h;
  return LGX_OK;
}

lgx_status lgx_amg_info(const lgx_amg *h, int64_t *nlevels, int64_t *rows, int64_t *nnz,
                        int64_t max_levels) {
  if (!h) return fail(LGX_ERR_INVALID, "null hierarchy");
  const int64_t L = (int64_t)h->lv.size();
  if (nlevels) *nlevels = L;
  for (int64_t l = 0; l < L && l < max_levels; ++l) {
    if (rows) rows[l] = h->lv[l]->a->n;
    if (nnz) nnz[l] = h->lv[l]->a->nnz;
  }
  return LGX_OK;
}

lgx_status lgx_amg_level_download(const lgx_amg *h, int64_t level, int64_t *h_rowptr,
                                  int32_t *h_col, double *h_val, uint32_t *h_agg,
                                  lgx_stream stream) {
  if (!h || level < 0 || level >= (int64_t)h->lv.size())
    return fail(LGX_ERR_INVALID, "bad level");
  const lgx_amg_level &lv = *h->lv[level];
  if (lv.stencil)
    return fail(LGX_ERR_UNSUPPORTED, "the finest level is a matrix-free stencil (no stored CSR)");
  const Csr &c = *lv.a;
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
      k_convert<float, double><<<std::min<int64_t>(grid_for(c.nnz, 256), 16384), 256, 0,
                                 stream>>>(c.nnz, c.v32.p, tmp.p);
      LGX_LAUNCH_CHECK();
      LGX_CUDA(cudaMemcpyAsync(h_val, tmp.p, sizeof(double) * c.nnz, cudaMemcpyDeviceToHost,
                               stream));
      LGX_CUDA(cudaStreamSynchronize(stream));
    }
  }
  if (h_agg) {
    if (level + 1 >= (int64_t)h->lv.size())
      return fail(LGX_ERR_INVALID, "the coarsest level has no aggregate map");
    LGX_CUDA(cudaMemcpyAsync(h_agg, lv.agg.agg.p, sizeof(uint32_t) * c.n, cudaMemcpyDeviceToHost,
                             stream));
  }
  LGX_CUDA(cudaStreamSynchronize(stream));
  return LGX_OK;
}

lgx_status lgx_amg_setup_log(const lgx_amg *h, lgx_amg_level_log *levels, int64_t max_levels,
                             int64_t *nlevels, int32_t *stop_reason) {
  if (!h || (levels && max_levels < 0)) return fail(LGX_ERR_INVALID, "bad argument");
  const int64_t L = (int64_t)h->lv.size();
  if (nlevels) *nlevels = L;
  if (stop_reason) *stop_reason = h->stop_reason;
  for (int64_t l = 0; levels && l < std::min(L, max_levels); ++l) {
    const Csr &c = *h->lv[l]->a;
    lgx_amg_level_log &o = levels[l];
    o = lgx_amg_level_log{};
    o.rows = c.n;
    o.columns = c.n;
    o.nnz = c.nnz;
    if (l + 1 < L && l < 32) {
      o.aggregate_num = h->stats[l][0];
      o.multi_vertex_aggregate_num = h->stats[l][1];
      o.single_vertex_aggregate_num = h->stats[l][2];
      o.merged_aggregate_num = h->stats[l][3];
      o.isolated_aggregate_num = h->stats[l][4];
      o.aggressive = h->aggressive[l];
      o.given_map = h->given[l];
    }
  }
  return LGX_OK;
}

lgx_status lgx_amg_level_lists(const lgx_amg *h, int64_t level, int64_t *h_list_ptr,
                               int32_t *h_list, int64_t *list_len, lgx_stream stream) {
  if (!h || level < 0 || level + 1 >= (int64_t)h->lv.size())
    return fail(LGX_ERR_INVALID, "bad level (the coarsest level has no aggregate lists)");
  const AggResult &g = h->lv[level]->agg;
  const int64_t nc = g.ncoarse;
  if (g.list_ptr.n < nc + 1) return fail(LGX_ERR_INVALID, "hierarchy holds no aggregate lists for this level");
  int64_t total = 0;
  LGX_CUDA(cudaMemcpyAsync(&total, g.list_ptr.p + nc, sizeof(int64_t), cudaMemcpyDeviceToHost,
                           stream));
  if (h_list_ptr)
    LGX_CUDA(cudaMemcpyAsync(h_list_ptr, g.list_ptr.p, sizeof(int64_t) * (size_t)(nc + 1),
                             cudaMemcpyDeviceToHost, stream));
  LGX_CUDA(cudaStreamSynchronize(stream));
  if (total < 0 || total > g.list.n) return fail(LGX_ERR_INVALID, "aggregate lists inconsistent");
  if (list_len) *list_len = total;
  if (h_list && total > 0) {
    LGX_CUDA(cudaMemcpyAsync(h_list, g.list.p, sizeof(int32_t) * (size_t)total,
                             cudaMemcpyDeviceToHost, stream));
    LGX_CUDA(cudaStreamSynchronize(stream));
  }
  return LGX_OK;
}

// Standalone dense direct solver: the coarsest-level solve on its own
// (CholeskySolver / LuSolver, direct/cholesky/solver.hpp:22-67,
// direct/lu/solver.hpp:21-66): the explicit inverse once, then one dense
// product per solve.
struct lgx_direct {
  int64_t n = 0;
  lgx::DBuf<double> inv;
  // banded Cholesky beyond the dense limit: bw >= 0, the band and a work
  // vector for the forward substitution
  int64_t bw = -1, ld = 0;
  lgx::DBuf<double> band, y;
};

namespace lgx {
// the band may take at most this many values (16 GiB)
constexpr int64_t kBandMaxEntries = (int64_t)1 << 31;

static lgx_status band_create(const Csr &a, cudaStream_t s, lgx_direct &d) {
  const int64_t n = a.n;
  DBuf<unsigned long long> bwd;
  LGX_CHECK(bwd.alloc(1));
  LGX_CUDA(cudaMemsetAsync(bwd.p, 0, sizeof(unsigned long long), s));
  k_band_width<<<(unsigned)std::min<int64_t>(grid_for(n, 256), 4096), 256, 0, s>>>(
    n, a.rowptr.p, a.col.p, bwd.p);
  LGX_LAUNCH_CHECK();
  unsigned long long hbw = 0;
  LGX_CUDA(cudaMemcpyAsync(&hbw, bwd.p, sizeof(hbw), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  const int64_t bw = (int64_t)hbw, ld = bw + 1;
  if (ld > kBandMaxEntries / n)
    return fail(LGX_ERR_INVALID, "the banded Cholesky takes at most 2^31 band values (n = " +
                                     std::to_string(n) + ", bandwidth " + std::to_string(bw) +
                                     ")");
  d.bw = bw;
  d.ld = ld;
  LGX_CHECK(d.band.alloc(n * ld));
  LGX_CHECK(d.y.alloc(n));
  LGX_CUDA(cudaMemsetAsync(d.band.p, 0, sizeof(double) * n * ld, s));
  const Band B{n, bw, ld, d.band.p};
  k_band_fill<<<(unsigned)std::min<int64_t>(grid_for(n, 256), 16384), 256, 0, s>>>(
    B, a.rowptr.p, a.col.p, a.storage == LGX_F64 ? a.v64.p : nullptr,
    a.storage == LGX_F32 ? a.v32.p : nullptr);
  LGX_LAUNCH_CHECK();
  DBuf<int> bad;
  LGX_CHECK(bad.alloc(1));
  LGX_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  for (int64_t k0 = 0; k0 < n; k0 += kCb) {
    const int64_t k1 = std::min<int64_t>(k0 + kCb, n), rend = std::min<int64_t>(k1 + bw, n);
    k_band_panel<<<(unsigned)std::max<int64_t>(1, (rend - k1 + 255) / 256), 256, 0, s>>>(
      B, k0, bad.p);
    if (rend > k1) {
      const int64_t T = (rend - k1 + 31) / 32;
      k_band_trail<<<(unsigned)(T * (T + 1) / 2), 256, 0, s>>>(B, k0, bad.p);
    }
  }
  LGX_LAUNCH_CHECK();
  int h_bad = 0;
  LGX_CUDA(cudaMemcpyAsync(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  if (h_bad) return fail(LGX_ERR_NOT_SPD, "matrix has a non-positive pivot");
  return LGX_OK;
}
}  // namespace lgx

lgx_status lgx_direct_create(const lgx_matrix *a, int kind, lgx_stream stream,
                             lgx_direct **out) {
  if (!a || !out) return fail(LGX_ERR_INVALID, "null argument");
  if (kind != LGX_DIRECT_CHOLESKY && kind != LGX_DIRECT_LU)
    return fail(LGX_ERR_INVALID, "kind must be LGX_DIRECT_CHOLESKY or LGX_DIRECT_LU");
  if (a->kind != LGX_MATRIX_CSR)
    return fail(LGX_ERR_UNSUPPORTED, "the direct solver needs a CSR matrix");
  auto d = std::make_unique<lgx_direct>();
  d->n = a->csr.n;
  if (a->csr.n > LGX_DIRECT_MAX_ROWS) {
    // beyond the dense limit: the banded Cholesky (lineal's factor is the
    // envelope of the natural order); the unpivoted LU stays dense
    if (kind != LGX_DIRECT_CHOLESKY)
      return fail(LGX_ERR_INVALID, "the dense LU solver takes at most " +
                                       std::to_string(LGX_DIRECT_MAX_ROWS) + " rows");
    LGX_CHECK(band_create(a->csr, (cudaStream_t)stream, *d));
    *out = d.release();
    return LGX_OK;
  }
  LGX_CHECK(dense_inverse(a->csr, (cudaStream_t)stream, d->inv, kind == LGX_DIRECT_CHOLESKY));
  *out = d.release();
  return LGX_OK;
}

lgx_status lgx_direct_solve(const lgx_direct *d, const double *d_b, double *d_x,
                            lgx_stream stream) {
  if (!d) return fail(LGX_ERR_INVALID, "null solver");
  if (d->n == 0) return LGX_OK;
  if (!d_b || !d_x) return fail(LGX_ERR_INVALID, "null vector");
  if (d_b == d_x) return fail(LGX_ERR_INVALID, "b and x must not be the same vector");
  const cudaStream_t s = (cudaStream_t)stream;
  if (d->bw >= 0) {
    const Band B{d->n, d->bw, d->ld, const_cast<double *>(d->band.p)};
    double *y = const_cast<double *>(d->y.p);
    k_band_fwd<<<1, 1024, 0, s>>>(B, d_b, y);
    k_band_bwd<<<1, 1024, 0, s>>>(B, y, d_x);
    LGX_LAUNCH_CHECK();
    count_launch();
    count_launch();
    return LGX_OK;
  }
  LGX_CUDA(launch_pdl(false, k_dense_apply<double>,
                      dim3((unsigned)std::min<int64_t>(grid_for(d->n * 32, 256), 4096)), dim3(256),
                      0, s, d->n, (const double *)d->inv.p, d_b, d_x));
  count_launch();
  return LGX_OK;
}

lgx_status lgx_direct_destroy(lgx_direct *d) {
  delete d;
  return LGX_OK;
}

lgx_status lgx_amg_vcycle(lgx_amg *h, const double *d_b, double *d_x, lgx_stream stream) {
  if (!h || !d_b || !d_x) return fail(LGX_ERR_INVALID, "null argument");
  lgx_amg_level &l0 = *h->lv[0];
  const int64_t n = l0.a->n;
  if (!h->nat_b.p) {
    LGX_CHECK(h->nat_b.alloc(n));
    LGX_CHECK(h->nat_x.alloc(n));
  }
  const int32_t *perm = h->lv.size() > 1 ? l0.col->perm.p : nullptr;
  if (perm) {
    LGX_CHECK(gather<double, double>(n, perm, d_b, h->nat_b.p, stream));
    LGX_CHECK(amg_apply_permuted(*h, h->nat_b.p, h->nat_x.p, stream));
    return scatter<double, double>(n, perm, h->nat_x.p, d_x, stream);
  }
  return amg_apply_permuted(*h, d_b, d_x, stream);
}

int lgx_amg_grid27(const lgx_amg *h) {
  return h && !h->lv.empty() && h->lv[0]->col && h->lv[0]->col->pcsr.grid ? 1 : 0;
}

lgx_status lgx_amg_strength(const lgx_matrix *a, double theta, uint8_t *d_depends,
                            uint8_t *d_influences, uint8_t *d_isolated, lgx_stream stream) {
  if (!a || !d_depends || !d_influences || !d_isolated)
    return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind != LGX_MATRIX_CSR) return fail(LGX_ERR_UNSUPPORTED, "strength needs a CSR matrix");
  return strength(a->csr, theta, d_depends, d_influences, d_isolated, stream);
}

lgx_status lgx_amg_aggregate(const lgx_matrix *a, const uint8_t *d_depends,
                             const uint8_t *d_influences, const uint8_t *d_isolated,
                             int32_t min_size, int32_t max_size, int64_t nparts, int aggressive,
                             uint32_t *d_agg, int64_t *ncoarse, lgx_stream stream) {
  if (!a || !d_depends || !d_influences || !d_isolated || !d_agg)
    return fail(LGX_ERR_INVALID, "null argument");
  if (a->kind != LGX_MATRIX_CSR)
    return fail(LGX_ERR_UNSUPPORTED, "aggregation needs a CSR matrix");
  if (max_size > 64 || min_size < 1 || min_size > max_size)
    return fail(LGX_ERR_INVALID, "aggregate sizes must satisfy 1 <= min <= max <= 64");
  AggResult r;
  LGX_CHECK(aggregate(a->csr, d_depends, d_influences, d_isolated, min_size, max_size, nparts,
                      aggressive, stream, r, d_agg));
  if (ncoarse) *ncoarse = r.ncoarse;
  return LGX_OK;
}

}  // extern "C"
