// Finest level of a grid matrix without column indices.
//
// Two patterns, each with the colouring whose colour classes are contiguous
// grid sub-lattices:
//  * 27 points, parity colouring (even edges): row r of the colour-permuted
//    matrix is the cell (i, j, k) with
//      c = r / B,  q = r % B,  (i, j, k) = 2 (q / (h1 h2), q / h2 % h1, q % h2)
//                                          + (c >> 2, (c >> 1) & 1, c & 1),
//    B = n / 8, h = n / 2, and the neighbour at offset (dz, dy, dx) sits at
//      r' = c' B + ((i' >> 1) h1 + (j' >> 1)) h2 + (k' >> 1),
//      c' = 4 (i' & 1) + 2 (j' & 1) + (k' & 1),
//    i.e. at r + delta[c][e] for a table of 8 x 27 deltas;
//  * 7 points, red-black colouring c = (i + j + k) & 1 (even n2): B = n / 2,
//    line L = q / h2 = i n1 + j, k = 2 (q % h2) + s with s = (c + i + j) & 1,
//    and the neighbours (other colour) at q -+ n1 h2 (axis 0), q -+ h2
//    (axis 1), q - 1 + s and q + s (axis 2), plus (1 - c) B.
// The kernels compute those indices instead of reading column indices
// (4 bytes per entry less: a third of the FP64 bytes, half of the float
// bytes, two thirds of the bfloat16 bytes), and consecutive rows of a colour
// -- consecutive k -- gather consecutive entries of every neighbour colour,
// so the x reads of a warp are contiguous.  The values are stored per
// offset (v[e S + r], S the padded plane stride); each row sums its entries
// in offset order, which is the CSR row order, with the arithmetic of the
// CSR row operations (SpmvOp, ResidualOp, SorOp), so every result is
// bit-identical to the CSR path.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>

#include "lgx_internal.cuh"
#include "lgx_rows.cuh"

namespace lgx {

// kernel view; pts = 27 or 7; delta[c][e] = r' - r for a row of colour c
// and its in-grid neighbour at offset e (27 points: the same for every row
// of a colour)
struct G27 {
  int pts, n0, n1, n2, h1, h2;
  int64_t n, block, stride, n1h2;
  int32_t delta[8][27];
};

static G27 view(const Grid27 &g) {
  G27 v{g.points, g.n0, g.n1, g.n2, g.n1 / 2, g.n2 / 2, g.n, g.block, g.stride,
        (int64_t)g.n1 * (g.n2 / 2), {}};
  if (g.points != 27) return v;
  for (int c = 0; c < 8; ++c) {
    const int pi = c >> 2, pj = (c >> 1) & 1, pk = c & 1;
    for (int e = 0; e < 27; ++e) {
      const int dz = e / 9 - 1, dy = (e / 3) % 3 - 1, dx = e % 3 - 1;
      const int c2 = ((pi + dz) & 1) * 4 + ((pj + dy) & 1) * 2 + ((pk + dx) & 1);
      // floor((p + d) / 2) for p + d in [-1, 2]
      const int fz = (pi + dz + 2) / 2 - 1, fy = (pj + dy + 2) / 2 - 1, fx = (pk + dx + 2) / 2 - 1;
      v.delta[c][e] = (int32_t)((int64_t)(c2 - c) * g.block +
                                ((int64_t)fz * v.h1 + fy) * v.h2 + fx);
    }
  }
  return v;
}

// offsets of entry e in CSR row order: 27 points lexicographic (dz, dy, dx);
// 7 points (-1,0,0) (0,-1,0) (0,0,-1) (0,0,0) (0,0,1) (0,1,0) (1,0,0)
template <int PTS>
__host__ __device__ constexpr int g_dz(int e) {
  return PTS == 27 ? e / 9 - 1 : (e == 0 ? -1 : e == 6 ? 1 : 0);
}
template <int PTS>
__host__ __device__ constexpr int g_dy(int e) {
  return PTS == 27 ? (e / 3) % 3 - 1 : (e == 1 ? -1 : e == 5 ? 1 : 0);
}
template <int PTS>
__host__ __device__ constexpr int g_dx(int e) {
  return PTS == 27 ? e % 3 - 1 : (e == 2 ? -1 : e == 4 ? 1 : 0);
}
template <int PTS>
__host__ __device__ constexpr int g_diag() {
  return PTS == 27 ? 13 : 3;
}

// a row's cell and what its neighbour indices need
struct GCell {
  int i, j, k, c, s;
  int64_t q;
};

template <int PTS>
__device__ __forceinline__ GCell g_cell(const G27 &g, int64_t r) {
  GCell x;
  const unsigned ur = (unsigned)r, blk = (unsigned)g.block;
  const unsigned c = ur / blk, q = ur - c * blk;
  x.c = (int)c;
  x.q = q;
  if constexpr (PTS == 27) {
    const unsigned hh = (unsigned)g.h1 * (unsigned)g.h2;
    const unsigned a = q / hh, rem = q - a * hh;
    const unsigned bq = rem / (unsigned)g.h2, d = rem - bq * (unsigned)g.h2;
    x.i = 2 * (int)a + (int)(c >> 2);
    x.j = 2 * (int)bq + (int)((c >> 1) & 1);
    x.k = 2 * (int)d + (int)(c & 1);
    x.s = 0;
  } else {
    const unsigned L = q / (unsigned)g.h2, d = q - L * (unsigned)g.h2;
    x.i = (int)(L / (unsigned)g.n1);
    x.j = (int)(L - (unsigned)x.i * (unsigned)g.n1);
    x.s = (int)((c + (unsigned)x.i + (unsigned)x.j) & 1u);
    x.k = 2 * (int)d + x.s;
  }
  return x;
}

// permuted index of the in-grid neighbour at offset e
template <int PTS>
__device__ __forceinline__ int64_t g_nb(const G27 &g, const GCell &x, int64_t r, int e) {
  if constexpr (PTS == 27) {
    return r + g.delta[x.c][e];
  } else {
    const int64_t base = (int64_t)(1 - x.c) * g.block + x.q;
    switch (e) {
      case 0: return base - g.n1h2;
      case 1: return base - g.h2;
      case 2: return base - 1 + x.s;
      case 4: return base + x.s;
      case 5: return base + g.h2;
      case 6: return base + g.n1h2;
      default: return r;
    }
  }
}

// in-grid tests of a row's neighbours: bit 0/1 lower/upper neighbour exists
// along axis 0, bits 2/3 axis 1, bits 4/5 axis 2
__device__ __forceinline__ unsigned g27_sides(const G27 &g, int i, int j, int k) {
  return (unsigned)(i > 0) | (unsigned)(i + 1 < g.n0) << 1 | (unsigned)(j > 0) << 2 |
         (unsigned)(j + 1 < g.n1) << 3 | (unsigned)(k > 0) << 4 | (unsigned)(k + 1 < g.n2) << 5;
}

template <int PTS>
__device__ __forceinline__ bool g_in(unsigned sides, int e) {
  const int dz = g_dz<PTS>(e), dy = g_dy<PTS>(e), dx = g_dx<PTS>(e);
  unsigned need = 0;
  if (dz < 0) need |= 1u;
  if (dz > 0) need |= 2u;
  if (dy < 0) need |= 4u;
  if (dy > 0) need |= 8u;
  if (dx < 0) need |= 16u;
  if (dx > 0) need |= 32u;
  return (sides & need) == need;
}

// the permuted index of an in-grid cell from its coordinates (the build's
// independent check of g_nb)
template <int PTS>
__device__ __forceinline__ int64_t g_row_of(const G27 &g, int i, int j, int k) {
  if constexpr (PTS == 27) {
    const int64_t c = (i & 1) * 4 + (j & 1) * 2 + (k & 1);
    return c * g.block + ((int64_t)(i >> 1) * g.h1 + (j >> 1)) * g.h2 + (k >> 1);
  } else {
    const int64_t c = (i + j + k) & 1;
    return c * g.block + ((int64_t)i * g.n1 + j) * g.h2 + (k >> 1);
  }
}

// ---- build: CSR rows -> per-offset values, checking the structure --------
// bad |= 1: a row is not the cell the colour order puts there; 2: a row's
// entries are not exactly its in-grid neighbours in offset order; 4: the
// kernels' neighbour index disagrees with the coordinates
template <typename VT, int PTS>
__global__ void k_g27_fill(G27 g, const int64_t *__restrict__ rowptr,
                           const int32_t *__restrict__ col, const VT *__restrict__ val,
                           const int32_t *__restrict__ perm, VT *__restrict__ out, int *bad) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < g.n;
       r += (int64_t)gridDim.x * blockDim.x) {
    const GCell x = g_cell<PTS>(g, r);
    if (perm && perm[r] != ((int64_t)x.i * g.n1 + x.j) * g.n2 + x.k) atomicOr(bad, 1);
    if (g_row_of<PTS>(g, x.i, x.j, x.k) != r) atomicOr(bad, 1);
    int64_t p = rowptr[r];
    const int64_t pe = rowptr[r + 1];
    for (int e = 0; e < PTS; ++e) {
      VT v = static_cast<VT>(0.0f);
      const int i2 = x.i + g_dz<PTS>(e), j2 = x.j + g_dy<PTS>(e), k2 = x.k + g_dx<PTS>(e);
      if ((unsigned)i2 < (unsigned)g.n0 && (unsigned)j2 < (unsigned)g.n1 &&
          (unsigned)k2 < (unsigned)g.n2) {
        const int64_t want = g_row_of<PTS>(g, i2, j2, k2);
        if (g_nb<PTS>(g, x, r, e) != want) atomicOr(bad, 4);
        if (p < pe && (int64_t)col[p] == want) {
          v = val[p];
          ++p;
        } else {
          atomicOr(bad, 2);
        }
      }
      out[(int64_t)e * g.stride + r] = v;
    }
    if (p != pe) atomicOr(bad, 2);
  }
}

// ---- row operations ---------------------------------------------------------
// MODE 0: y = A x; 1: r = b - A x (bf16: A x scaled by the row factor);
// 2: SOR row in place (the arithmetic of SorOp, lgx_smoother.cu); 4: the
// SOR row of MODE 2, then the row's residual b - A x with its new x written
// to y (the last colour of a forward sweep: every neighbour already holds
// its final value, and the residual is MODE 1's sum in the same order)
struct G27Sor {
  double relax, m1;
  int ultra, relax_one, from_zero;
  int64_t visit_end;
  const double *rdiag;
  // sweep from zero: bit e set when the neighbour at offset e lies in a
  // colour the sweep has not visited yet (it reads as 0 and is not loaded);
  // the same for every row of a colour launch (g27_unvisited)
  uint32_t fz_mask = 0;
};

// The offsets whose neighbours lie in colours after colour c: the parity
// colouring c = 4 (i & 1) + 2 (j & 1) + (k & 1) gives the neighbour at
// (dz, dy, dx) the colour c ^ (4 [dz != 0] + 2 [dy != 0] + [dx != 0]); the
// red-black colouring gives every neighbour the other colour.  Colours
// occupy consecutive row blocks, so "a later colour" is "a row at or past
// the launch's first row", the test a forward sweep from zero makes.
template <int PTS>
static uint32_t g27_unvisited(int c) {
  uint32_t m = 0;
  for (int e = 0; e < PTS; ++e) {
    if (e == g_diag<PTS>()) continue;
    const int nc = PTS == 27 ? c ^ (4 * (g_dz<PTS>(e) != 0) + 2 * (g_dy<PTS>(e) != 0) +
                                    (g_dx<PTS>(e) != 0))
                             : 1 - c;
    if (nc > c) m |= 1u << e;
  }
  return m;
}

// Loads through the non-coherent path as volatile asm, which the compiler
// does not sink into the branches that use them: every load of a round is
// issued unconditionally.  Every address read is valid (values exist for all
// 27 offsets; a neighbour outside the grid reads the row itself), and no
// launch writes what it reads this way (a sweep writes one colour and reads
// the others).
__device__ __forceinline__ double g27_ld(const double *p) {
  double v;
  asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float g27_ld(const float *p) {
  float v;
  asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ bf16 g27_ld(const bf16 *p) {
  unsigned short v;
  asm volatile("ld.global.nc.u16 %0, [%1];" : "=h"(v) : "l"(p));
  return __ushort_as_bfloat16(v);
}

// entries whose loads are issued together before their FMAs: rounds of
// three (nine rounds for 27 points, three for 7).  Measured at 256^3 (AMG-PCG, FP64 / float cycle): rounds of 27
// (float) 346 ms mixed; of 9: FP64 456, mixed 296 ms; of 3: FP64 432, mixed
// 274 ms; single loads: FP64 452, mixed 297 ms -- short rounds keep the
// registers low and more warps resident, which hides the gathers better
// than deeper rounds in fewer warps.
constexpr int kG27Batch = 3;

template <int MODE>
constexpr bool g_sor_mode() {
  return MODE == 2 || MODE == 4;
}

// One row's state through its entries, in the arithmetic of SpmvOp
// (MODE 0), ResidualOp (MODE 1) and SorOp (MODE 2 and 4, lgx_smoother.cu).
template <typename VT, typename XT, int MODE, int PTS>
struct G27Row {
  static constexpr int kDiag = g_diag<PTS>();
  XT acc = XT(0), diag = XT(0), xi = XT(0);  // sum | SOR accum (bf16: t), diagonal (bf16: v_ii)
  XT xnew = XT(0);                           // SOR: the row's new x
  __device__ __forceinline__ void init(int64_t r, const XT *b, const XT *x, const G27Sor &so) {
    if constexpr (g_sor_mode<MODE>()) {
      xi = so.from_zero ? XT(0) : x[r];
      if constexpr (!kIsBf16<VT>) acc = b[r];
    }
  }
  // entry e with value a and neighbour value xv (in: inside the grid)
  __device__ __forceinline__ void step(int e, bool in, XT a, XT xv, const G27Sor &so) {
    if (!in) return;
    if constexpr (!g_sor_mode<MODE>()) {
      acc = fma(a, xv, acc);
    } else if constexpr (kIsBf16<VT>) {
      if (e == kDiag) diag = a;
      else acc = fma(a, xv, acc);
    } else {
      if (e == kDiag) {
        diag = a;
        if (so.ultra) acc = fma(-a, xi, acc);
      } else {
        acc = fma(-a, xv, acc);
      }
    }
  }
  __device__ __forceinline__ void finish(int64_t r, const XT *b, XT *x, XT *y, const float *scale,
                                         const G27Sor &so) {
    if constexpr (MODE == 0) {
      y[r] = acc;
    } else if constexpr (MODE == 1) {
      XT sum = acc;
      if constexpr (kIsBf16<VT>) sum = sum * scale[r];
      y[r] = b[r] - sum;
    } else {
      const XT relax = (XT)so.relax, m1 = (XT)so.m1;
      if constexpr (kIsBf16<VT>) {
        const XT si = scale[r];
        const XT dg = si * diag;
        XT accum = fma(-si, acc, b[r]);
        if (so.ultra) {
          accum = fma(-dg, xi, accum);
          xnew = xi + relax * accum / fabs(dg);
        } else {
          xnew = fma(relax, accum / dg, m1 * xi);
        }
        x[r] = xnew;
      } else {
        if (so.ultra) {
          xnew = xi + relax * acc / fabs(diag);
          x[r] = xnew;
          return;
        }
        XT quot;
        if constexpr (sizeof(XT) == 8) {
          const double yr = so.rdiag ? so.rdiag[r] : 0.0;
          quot = (nonzero_bits(yr) && exponent_within_400(acc)) ? div_by_recip(acc, diag, yr)
                                                                : acc / diag;
          if (so.relax_one && nonzero_bits(quot) && exponent_field(xi) != 0x7ff) {
            xnew = quot;  // fma(1, q, 0 * x_i) == q for nonzero q and finite x_i
            x[r] = xnew;
            return;
          }
        } else {
          quot = acc / diag;
        }
        xnew = fma(relax, quot, m1 * xi);
        x[r] = xnew;
      }
    }
  }
};

// x of neighbour c for entry e of a row (0 for unvisited colours in a
// forward sweep from zero; the diagonal's x is not read here)
template <typename XT, int MODE, int PTS>
__device__ __forceinline__ XT g27_x(const XT *x, int64_t c, int e, const G27Sor &so) {
  if (g_sor_mode<MODE>() && e == g_diag<PTS>()) return XT(0);
  // the load stays unconditional (a round's loads go out together)
  const XT xl = g27_ld(x + c);
  return (g_sor_mode<MODE>() && ((so.fz_mask >> e) & 1u)) ? XT(0) : xl;
}

// one row per thread
template <typename VT, typename XT, int MODE, int PTS>
__global__ void __launch_bounds__(256)
  k_g27_rows(G27 g, int64_t rb, int64_t re, const VT *__restrict__ v, const XT *__restrict__ b,
             XT *x, XT *__restrict__ y, const float *__restrict__ scale, G27Sor so) {
  pdl_trigger();
  pdl_wait();
  const int64_t r = rb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= re) return;
  const GCell cell = g_cell<PTS>(g, r);
  const unsigned sides = g27_sides(g, cell.i, cell.j, cell.k);
  constexpr int B = kG27Batch;
  G27Row<VT, XT, MODE, PTS> row;
  row.init(r, b, x, so);
  // the loads of a round do not branch -- a neighbour outside the grid reads
  // x of the row itself, which step() then skips -- so they go out together
#pragma unroll
  for (int e0 = 0; e0 < PTS; e0 += B) {
    XT xv[B], av[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const int e = e0 + u;
      if (e >= PTS) break;
      av[u] = cvt<XT>(g27_ld(v + (int64_t)e * g.stride + r));
      xv[u] = g27_x<XT, MODE, PTS>(x, g_in<PTS>(sides, e) ? g_nb<PTS>(g, cell, r, e) : r, e, so);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const int e = e0 + u;
      if (e >= PTS) break;
      row.step(e, g_in<PTS>(sides, e), av[u], xv[u], so);
    }
  }
  row.finish(r, b, x, y, scale, so);
  if constexpr (MODE == 4) {
    // the residual with the new x: the values and neighbours again (L1),
    // the row's own x from the register
    XT sum = XT(0);
#pragma unroll
    for (int e0 = 0; e0 < PTS; e0 += B) {
      XT xv[B], av[B];
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int e = e0 + u;
        if (e >= PTS) break;
        av[u] = cvt<XT>(g27_ld(v + (int64_t)e * g.stride + r));
        xv[u] = (e == g_diag<PTS>() || !g_in<PTS>(sides, e))
                  ? row.xnew
                  : g27_ld(x + g_nb<PTS>(g, cell, r, e));
      }
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int e = e0 + u;
        if (e >= PTS) break;
        if (g_in<PTS>(sides, e)) sum = fma(av[u], xv[u], sum);
      }
    }
    y[r] = b[r] - sum;
  }
}

// four consecutive rows of a colour per thread (float vectors): the value
// planes load as one 16-byte (float) or 8-byte (bfloat16) vector per entry.
// The host uses it when rows come in aligned fours inside one line of the
// grid (h2 and the colour block size multiples of 4), so the four cells
// differ only in k (by 2 each).
template <typename VT, int R>
__device__ __forceinline__ void g27_ldv(const VT *p, float (&out)[R]);
template <>
__device__ __forceinline__ void g27_ldv<float, 4>(const float *p, float (&out)[4]) {
  asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(out[0]), "=f"(out[1]), "=f"(out[2]), "=f"(out[3])
               : "l"(p));
}
template <>
__device__ __forceinline__ void g27_ldv<bf16, 4>(const bf16 *p, float (&out)[4]) {
  unsigned short h[4];
  asm volatile("ld.global.nc.v4.u16 {%0, %1, %2, %3}, [%4];"
               : "=h"(h[0]), "=h"(h[1]), "=h"(h[2]), "=h"(h[3])
               : "l"(p));
#pragma unroll
  for (int q = 0; q < 4; ++q) out[q] = __bfloat162float(__ushort_as_bfloat16(h[q]));
}

template <typename VT, int MODE, int PTS>
__global__ void __launch_bounds__(256)
  k_g27_rows4(G27 g, int64_t rb, int64_t re, const VT *__restrict__ v,
              const float *__restrict__ b, float *x, float *__restrict__ y,
              const float *__restrict__ scale, G27Sor so) {
  constexpr int R = 4;
  pdl_trigger();
  pdl_wait();
  const int64_t r0 = rb + (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * R;
  if (r0 >= re) return;
  // the four cells share i, j and colour; k grows by 2 and q by 1
  GCell cell[R];
  cell[0] = g_cell<PTS>(g, r0);
  unsigned sides[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    cell[q] = cell[0];
    cell[q].k += 2 * q;
    cell[q].q += q;
    sides[q] = g27_sides(g, cell[q].i, cell[q].j, cell[q].k);
  }
  G27Row<VT, float, MODE, PTS> row[R];
#pragma unroll
  for (int q = 0; q < R; ++q) row[q].init(r0 + q, b, x, so);
  constexpr int B = kG27Batch;
#pragma unroll
  for (int e0 = 0; e0 < PTS; e0 += B) {
    float av[B][R], xv[B][R];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const int e = e0 + u;
      if (e >= PTS) break;
      g27_ldv<VT, R>(v + (int64_t)e * g.stride + r0, av[u]);
#pragma unroll
      for (int q = 0; q < R; ++q)
        xv[u][q] = g27_x<float, MODE, PTS>(
          x, g_in<PTS>(sides[q], e) ? g_nb<PTS>(g, cell[q], r0 + q, e) : r0 + q, e, so);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const int e = e0 + u;
      if (e >= PTS) break;
#pragma unroll
      for (int q = 0; q < R; ++q) row[q].step(e, g_in<PTS>(sides[q], e), av[u][q], xv[u][q], so);
    }
  }
#pragma unroll
  for (int q = 0; q < R; ++q) row[q].finish(r0 + q, b, x, y, scale, so);
}

// ---- grid rows with the values staged by the tensor engine ---------------
// Float or FP64 values and vectors on the 27- and 7-point grids: each CTA of
// RT rows has its rows' value-plane segments (PTS x RT values, one 2-D box of
// the value array viewed as [PTS][stride]) brought into shared memory by one
// cp.async.bulk.tensor copy, issued before the kernel waits for its
// predecessor (the values are constant); every thread then issues all its x
// gathers at once (x is written by other colours' launches and read through
// the non-coherent path), waits for the copy (bounded) and runs G27Row's
// arithmetic on the staged values, so results equal k_g27_rows bit for bit.
// The row-per-thread kernel keeps three value loads per round in flight and
// reaches 0.62 of HBM on a 27-point float sweep.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            uint64_t *bar) {
  asm volatile(
    "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
    " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
    "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
    : "memory");
}

// FZ: a forward sweep from zero (x of the colours from visit_end on reads
// as 0), a template argument so that other launches carry no per-entry test.
// Rows whose neighbours all lie inside the grid (all but the boundary
// layers) skip the per-entry inside tests.  T = float: 256 rows per CTA
// (T = double would take 128: the 27 gathered x of a row take 54
// registers); every row's sum in offset order as in k_g27_rows.
template <typename T>
constexpr int g_rows_per_cta() {
  return sizeof(T) == 8 ? 128 : 256;
}
template <typename T, int PTS>
constexpr int g_ctas_per_sm() {
  return sizeof(T) == 8 ? (PTS == 27 ? 5 : 8) : (PTS == 27 ? 4 : 6);
}

template <typename T, int MODE, bool FZ, int PTS>
__global__ void __launch_bounds__(g_rows_per_cta<T>(), g_ctas_per_sm<T, PTS>())
  k_g27_vtma(const __grid_constant__ CUtensorMap vmap, G27 g, int64_t rb, int64_t re,
             const T *__restrict__ b, T *x, T *__restrict__ y, G27Sor so, int *err) {
  constexpr int RT = g_rows_per_cta<T>();
  __shared__ __align__(128) T sv[PTS * RT];
  __shared__ uint64_t bar;
  const int64_t t0 = rb + (int64_t)blockIdx.x * RT;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, PTS * RT * (unsigned)sizeof(T));
    tma_load_2d(sv, &vmap, (int)t0, 0, &bar);
  }
  pdl_trigger();
  pdl_wait();
  const int64_t r = t0 + threadIdx.x;
  const bool active = r < re;
  constexpr int kDiag = g_diag<PTS>();
  G27Row<T, T, MODE, PTS> row;
  T xv[PTS];
  unsigned sides = 0;
  if (active) {
    const GCell cell = g_cell<PTS>(g, r);
    sides = g27_sides(g, cell.i, cell.j, cell.k);
    row.init(r, b, x, so);
    if (sides == 0x3Fu) {
#pragma unroll
      for (int e = 0; e < PTS; ++e) {
        if ((g_sor_mode<MODE>() && e == kDiag) || (FZ && ((so.fz_mask >> e) & 1u))) {
          xv[e] = T(0);
          continue;
        }
        xv[e] = g27_ld(x + g_nb<PTS>(g, cell, r, e));
      }
    } else {
#pragma unroll
      for (int e = 0; e < PTS; ++e) {
        if ((g_sor_mode<MODE>() && e == kDiag) || (FZ && ((so.fz_mask >> e) & 1u))) {
          xv[e] = T(0);
          continue;
        }
        xv[e] = g27_ld(x + (g_in<PTS>(sides, e) ? g_nb<PTS>(g, cell, r, e) : r));
      }
    }
  }
  if (!mbar_wait_bounded(&bar, 0)) {
    // the copy did not complete in time: report, wait once more (bounded)
    // for it and leave
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      (void)mbar_wait_bounded(&bar, 0);
    }
    return;
  }
  if (!active) return;
  const T *svt = sv + threadIdx.x;
  if (sides == 0x3Fu) {
#pragma unroll
    for (int e = 0; e < PTS; ++e) row.step(e, true, svt[e * RT], xv[e], so);
  } else {
#pragma unroll
    for (int e = 0; e < PTS; ++e) row.step(e, g_in<PTS>(sides, e), svt[e * RT], xv[e], so);
  }
  row.finish(r, b, x, y, nullptr, so);
  if constexpr (MODE == 4) {
    // the residual with the new x (staged values, gathered neighbours)
    T sum = T(0);
#pragma unroll
    for (int e = 0; e < PTS; ++e)
      if (sides == 0x3Fu || g_in<PTS>(sides, e))
        sum = fma(svt[e * RT], e == kDiag ? row.xnew : xv[e], sum);
    y[r] = b[r] - sum;
  }
}

// the tensor-staged kernels serve float rows with 16-byte-aligned row starts
// (LGX_G27_TMA=0 switches it off)
static bool g27_tma_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("LGX_G27_TMA");
    return !(e && e[0] == '0');
  }();
  return on;
}

using G27EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                 const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                 const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static G27EncodeFn g27_encode() {
  static const G27EncodeFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (G27EncodeFn) nullptr;
    }
    return (G27EncodeFn)p;
  }();
  return fn;
}

// the values viewed as [points][stride], boxes of points x rows-per-CTA
// (cached on the grid, keyed by the value array)
template <typename T>
static const CUtensorMap *g27_value_map(const Grid27 &gr, const T *v) {
  unsigned char *store = sizeof(T) == 8 ? gr.vmap64 : gr.vmap32;
  const void *&key = sizeof(T) == 8 ? gr.vmap64_key : gr.vmap32_key;
  static_assert(sizeof(CUtensorMap) <= sizeof(gr.vmap32), "tensor map storage");
  if (key == v) return reinterpret_cast<const CUtensorMap *>(store);
  const G27EncodeFn encode = g27_encode();
  if (!encode) return nullptr;
  CUtensorMap *map = reinterpret_cast<CUtensorMap *>(store);
  const cuuint64_t gdim[2] = {(cuuint64_t)gr.stride, (cuuint64_t)gr.points};
  const cuuint64_t gstride[1] = {(cuuint64_t)gr.stride * sizeof(T)};
  const cuuint32_t box[2] = {(cuuint32_t)g_rows_per_cta<T>(), (cuuint32_t)gr.points};
  const cuuint32_t estride[2] = {1, 1};
  if (encode(map, sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
             2, const_cast<T *>(v), gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return nullptr;
  key = v;
  return map;
}

template <typename T, int MODE, int PTS>
static bool g27_tma_launch(const Grid27 &gr, const T *v, int64_t rb, int64_t re, const T *b, T *x,
                           T *y, const G27Sor &so, bool pdl, cudaStream_t s, lgx_status *st) {
  if (!g27_tma_enabled() || gr.points != PTS || rb % (16 / (int64_t)sizeof(T)) ||
      ((uintptr_t)v & 15u) || (gr.stride * (int64_t)sizeof(T)) % 16 ||
      gr.stride > (int64_t)INT32_MAX)
    return false;
  const CUtensorMap *map = g27_value_map<T>(gr, v);
  if (!map) return false;
  constexpr int RT = g_rows_per_cta<T>();
  const int64_t ctas = (re - rb + RT - 1) / RT;
  auto kern = k_g27_vtma<T, MODE, false, PTS>;
  if constexpr (g_sor_mode<MODE>())
    if (so.from_zero) kern = k_g27_vtma<T, MODE, true, PTS>;
  const cudaError_t e = launch_pdl(pdl, kern, dim3((unsigned)ctas), dim3(RT), 0, s, *map,
                                   view(gr), rb, re, b, x, y, so, device_error_flag());
  *st = e == cudaSuccess ? LGX_OK : cuda_fail(e, "k_g27_vtma");
  count_launch();
  return true;
}

// four-row kernels for bfloat16 values (LGX_G27_ROWS4=0 switches them off)
static bool g27_rows4_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("LGX_G27_ROWS4");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <typename VT>
static const VT *grid_values(const Grid27 &g, const VT *src) {
  if constexpr (sizeof(VT) == 8) return src == g.src64 ? (const VT *)g.v64.p : nullptr;
  else if constexpr (kIsBf16<VT>) return src == g.src16 ? (const VT *)g.v16.p : nullptr;
  else return src == g.src32 ? (const VT *)g.v32.p : nullptr;
}

template <typename VT, typename XT, int MODE, int PTS>
static lgx_status launch_g27_pts(const Grid27 &gr, const VT *v, int64_t rb, int64_t re,
                                 const XT *b, XT *x, XT *y, const float *scale,
                                 const G27Sor &so, cudaStream_t s) {
  const int64_t rows = re - rb;
  const bool pdl = sizeof(XT) == 4 || rows <= pdl_fp64_rows();
  if constexpr (kIsBf16<VT>) {
    // bfloat16 values: four rows per thread (8-byte value loads) when every
    // thread's four rows are whole, in one colour block and in one grid line.
    // Measured at 256^3 (27 points): bf16 cycle 296 -> 273 ms; float values
    // lose with it (272 -> 281 ms: their rows run one per thread)
    if (g27_rows4_enabled() && (gr.n2 / 2) % 4 == 0 && gr.block % 4 == 0 && rb % 4 == 0 &&
        re % 4 == 0) {
      LGX_CUDA(launch_pdl(pdl, k_g27_rows4<VT, MODE, PTS>,
                          dim3((unsigned)((rows / 4 + 255) / 256)), dim3(256), 0, s, view(gr),
                          rb, re, v, b, x, y, scale, so));
      count_launch();
      return LGX_OK;
    }
  }
  // float rows take the value-staged kernel; FP64 rows stay on k_g27_rows:
  // they are FP64-pipe bound, and staging their 216 bytes of values per row
  // leaves too few warps per SM to cover the FMA chains (measured at 256^3:
  // FP64 SOR sweep 1.198 -> 1.328 ms, FP64 AMG-PCG 420 -> 480 ms)
  if constexpr (std::is_same_v<VT, float> && std::is_same_v<XT, float>) {
    lgx_status st = LGX_OK;
    if (g27_tma_launch<VT, MODE, PTS>(gr, v, rb, re, b, x, y, so, pdl, s, &st)) return st;
  }
  LGX_CUDA(launch_pdl(pdl, k_g27_rows<VT, XT, MODE, PTS>, dim3((unsigned)((rows + 255) / 256)),
                      dim3(256), 0, s, view(gr), rb, re, v, b, x, y, scale, so));
  count_launch();
  return LGX_OK;
}

template <typename VT, typename XT, int MODE>
static lgx_status launch_g27(const Grid27 &gr, const VT *v, int64_t rb, int64_t re, const XT *b,
                             XT *x, XT *y, const float *scale, const G27Sor &so,
                             cudaStream_t s) {
  if (re <= rb) return LGX_OK;
  if constexpr (MODE == 4) {
    // the sweep with residuals serves the 7-point grid only (grid_sweep_residual)
    if (gr.points != 7) return fail(LGX_ERR_UNSUPPORTED, "sweep with residual: 27-point grid");
    return launch_g27_pts<VT, XT, MODE, 7>(gr, v, rb, re, b, x, y, scale, so, s);
  } else {
    if (gr.points == 7)
      return launch_g27_pts<VT, XT, MODE, 7>(gr, v, rb, re, b, x, y, scale, so, s);
    return launch_g27_pts<VT, XT, MODE, 27>(gr, v, rb, re, b, x, y, scale, so, s);
  }
}

template <typename VT, typename XT>
lgx_status grid_spmv(const Csr &a, const VT *val, const XT *x, XT *y, cudaStream_t s,
                     bool *done) {
  *done = false;
  if (!a.grid) return LGX_OK;
  const VT *v = grid_values(*a.grid, val);
  if (!v) return LGX_OK;
  LGX_CHECK((launch_g27<VT, XT, 0>(*a.grid, v, 0, a.n, nullptr, const_cast<XT *>(x), y, nullptr,
                                   G27Sor{}, s)));
  *done = true;
  return LGX_OK;
}

template <typename VT, typename XT>
lgx_status grid_residual(const Csr &a, const VT *val, const XT *b, const XT *x, XT *r,
                         const float *scale, cudaStream_t s, bool *done) {
  *done = false;
  if (!a.grid) return LGX_OK;
  const VT *v = grid_values(*a.grid, val);
  if (!v) return LGX_OK;
  LGX_CHECK((launch_g27<VT, XT, 1>(*a.grid, v, 0, a.n, b, const_cast<XT *>(x), r, scale,
                                   G27Sor{}, s)));
  *done = true;
  return LGX_OK;
}

template <typename VT, typename XT>
lgx_status grid_sor_rows(const Csr &a, const VT *val, int64_t rb, int64_t re, const XT *b, XT *x,
                         double relax, int ultra, const double *rdiag, int relax_one,
                         int from_zero, int64_t visit_end, const float *scale, cudaStream_t s,
                         bool *done, XT *r_out) {
  *done = false;
  if (!a.grid) return LGX_OK;
  const VT *v = grid_values(*a.grid, val);
  if (!v) return LGX_OK;
  G27Sor so{relax, 1.0 - relax, ultra, relax_one, from_zero, visit_end, rdiag};
  // the float SOR of SorOp forms XT(1) - XT(relax): the same in XT
  so.m1 = (double)((XT)1 - (XT)relax);
  // a forward sweep from zero visits the colours in order: the rows before
  // rb (= visit_end, a colour's first row) are visited, the others read 0
  if (from_zero) {
    const Grid27 &gr = *a.grid;
    if (rb != visit_end || rb % gr.block || re - rb > gr.block)
      return fail(LGX_ERR_INVALID, "grid sweep from zero: rows are not one colour's block");
    const int c = (int)(rb / gr.block);
    so.fz_mask = gr.points == 27 ? g27_unvisited<27>(c) : g27_unvisited<7>(c);
  }
  if constexpr (!kIsBf16<VT> && sizeof(XT) == 4) {
    if (r_out) {
      LGX_CHECK((launch_g27<VT, XT, 4>(*a.grid, v, rb, re, b, x, r_out, scale, so, s)));
      *done = true;
      return LGX_OK;
    }
  }
  if (r_out) return fail(LGX_ERR_UNSUPPORTED, "sweep with residual: FP64 or bfloat16 rows");
  LGX_CHECK((launch_g27<VT, XT, 2>(*a.grid, v, rb, re, b, x, nullptr, scale, so, s)));
  *done = true;
  return LGX_OK;
}

// A red-black sweep's second colour leaves half the residual for free: its
// rows hold every value the residual needs.  Float rows only: measured at
// 256^3 (7-point, sigma = 3, to 1e-10) the float-vector CG went 318.7 ->
// 308.6 ms, while the FP64 solve went 531.6 -> 562.7 ms (the FP64 row with
// its residual holds 48 instead of 40 registers on an FP64-pipe-bound
// launch).  On the 27-point grid the last of eight colours would save an
// eighth of the residual pass at the price of a longer row, so it keeps the
// pass.
bool grid_sweep_residual(const Csr &a) { return a.grid && a.grid->points == 7; }

template <typename VT, typename XT>
lgx_status grid_residual_rows(const Csr &a, const VT *val, const XT *b, const XT *x, XT *r,
                              int64_t rb, int64_t re, cudaStream_t s, bool *done) {
  *done = false;
  if (!a.grid) return LGX_OK;
  const VT *v = grid_values(*a.grid, val);
  if (!v) return LGX_OK;
  LGX_CHECK((launch_g27<VT, XT, 1>(*a.grid, v, rb, re, b, const_cast<XT *>(x), r, nullptr,
                                   G27Sor{}, s)));
  *done = true;
  return LGX_OK;
}

template lgx_status grid_spmv<double, double>(const Csr &, const double *, const double *,
                                              double *, cudaStream_t, bool *);
template lgx_status grid_spmv<float, double>(const Csr &, const float *, const double *, double *,
                                             cudaStream_t, bool *);
template lgx_status grid_spmv<float, float>(const Csr &, const float *, const float *, float *,
                                            cudaStream_t, bool *);
template lgx_status grid_residual<double, double>(const Csr &, const double *, const double *,
                                                  const double *, double *, const float *,
                                                  cudaStream_t, bool *);
template lgx_status grid_residual<float, double>(const Csr &, const float *, const double *,
                                                 const double *, double *, const float *,
                                                 cudaStream_t, bool *);
template lgx_status grid_residual<float, float>(const Csr &, const float *, const float *,
                                                const float *, float *, const float *,
                                                cudaStream_t, bool *);
template lgx_status grid_residual<bf16, float>(const Csr &, const bf16 *, const float *,
                                               const float *, float *, const float *,
                                               cudaStream_t, bool *);
template lgx_status grid_sor_rows<double, double>(const Csr &, const double *, int64_t, int64_t,
                                                  const double *, double *, double, int,
                                                  const double *, int, int, int64_t,
                                                  const float *, cudaStream_t, bool *, double *);
template lgx_status grid_sor_rows<float, double>(const Csr &, const float *, int64_t, int64_t,
                                                 const double *, double *, double, int,
                                                 const double *, int, int, int64_t,
                                                 const float *, cudaStream_t, bool *, double *);
template lgx_status grid_sor_rows<float, float>(const Csr &, const float *, int64_t, int64_t,
                                                const float *, float *, double, int,
                                                const double *, int, int, int64_t, const float *,
                                                cudaStream_t, bool *, float *);
template lgx_status grid_sor_rows<bf16, float>(const Csr &, const bf16 *, int64_t, int64_t,
                                               const float *, float *, double, int,
                                               const double *, int, int, int64_t, const float *,
                                               cudaStream_t, bool *, float *);
template lgx_status grid_residual_rows<double, double>(const Csr &, const double *,
                                                       const double *, const double *, double *,
                                                       int64_t, int64_t, cudaStream_t, bool *);
template lgx_status grid_residual_rows<float, double>(const Csr &, const float *, const double *,
                                                      const double *, double *, int64_t, int64_t,
                                                      cudaStream_t, bool *);
template lgx_status grid_residual_rows<float, float>(const Csr &, const float *, const float *,
                                                     const float *, float *, int64_t, int64_t,
                                                     cudaStream_t, bool *);

// ---- attach -------------------------------------------------------------------
template <typename VT>
static lgx_status fill_one(const G27 &g, const Csr &p, const VT *src, const int32_t *perm,
                           DBuf<VT> &out, int *bad, cudaStream_t s) {
  LGX_CHECK(out.alloc(g.pts * g.stride));
  const unsigned grid = (unsigned)std::min<int64_t>(grid_for(g.n, 256), 16384);
  if (g.pts == 27)
    k_g27_fill<VT, 27><<<grid, 256, 0, s>>>(g, p.rowptr.p, p.col.p, src, perm, out.p, bad);
  else
    k_g27_fill<VT, 7><<<grid, 256, 0, s>>>(g, p.rowptr.p, p.col.p, src, perm, out.p, bad);
  LGX_LAUNCH_CHECK();
  count_launch();
  return LGX_OK;
}

lgx_status grid27_attach(lgx_colouring &c, const int64_t dims[3], int points, cudaStream_t s,
                         bool *attached) {
  *attached = false;
  const int64_t n = dims[0] * dims[1] * dims[2];
  const int ncol = points == 27 ? 8 : 2;
  if (points != 27 && points != 7) return LGX_OK;
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 2 || dims[2] % 2 || dims[0] > (1 << 30) ||
      dims[1] > (1 << 30) || dims[2] > (1 << 30) ||
      n + 64 > (int64_t)INT32_MAX)  // 32-bit row arithmetic in the kernels
    return LGX_OK;
  if (points == 27 && (dims[0] % 2 || dims[1] % 2)) return LGX_OK;
  if (c.n != n || c.ncolours != ncol || c.pcsr.n != n) return LGX_OK;
  for (int q = 0; q <= ncol; ++q)
    if (c.offsets[q] != q * (n / ncol)) return LGX_OK;
  auto gr = std::make_shared<Grid27>();
  gr->points = points;
  gr->n0 = (int)dims[0];
  gr->n1 = (int)dims[1];
  gr->n2 = (int)dims[2];
  gr->n = n;
  gr->block = n / ncol;
  gr->stride = ((n + 31) / 32) * 32;
  if ((gr->stride / 32) % 2 == 0) gr->stride += 32;
  const G27 g = view(*gr);
  DBuf<int> bad;
  LGX_CHECK(bad.alloc(1));
  LGX_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  const Csr &p = c.pcsr;
  if (p.storage == LGX_F64) {
    LGX_CHECK(fill_one<double>(g, p, p.v64.p, c.perm.p, gr->v64, bad.p, s));
    gr->src64 = p.v64.p;
  } else {
    LGX_CHECK(fill_one<float>(g, p, p.v32.p, c.perm.p, gr->v32, bad.p, s));
    gr->src32 = p.v32.p;
  }
  if (c.pv32.p) {
    LGX_CHECK(fill_one<float>(g, p, c.pv32.p, nullptr, gr->v32, bad.p, s));
    gr->src32 = c.pv32.p;
  }
  if (c.pv16.p) {
    LGX_CHECK(fill_one<bf16>(g, p, c.pv16.p, nullptr, gr->v16, bad.p, s));
    gr->src16 = c.pv16.p;
  }
  int h_bad = 0;
  LGX_CUDA(cudaMemcpyAsync(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  if (h_bad) return LGX_OK;  // not this structure: the CSR path stays
  c.pcsr.grid = gr;
  *attached = true;
  return LGX_OK;
}

}  // namespace lgx
