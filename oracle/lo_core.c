/*
 * Oracle core: partitions, geometry, valuators, stencil rows, CSR assembly,
 * generators, CSR kernels, reductions and colouring.
 * TEST INFRASTRUCTURE ONLY (see lineal_oracle.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "lineal_oracle.h"

#ifdef _OPENMP
#include <omp.h>
#endif

void lo_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int lo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void lo_csr_free(lo_csr *a) {
  free(a->rowptr);
  free(a->col);
  free(a->val);
  a->rowptr = NULL;
  a->col = NULL;
  a->val = NULL;
}

int64_t lo_csr_nnz(const lo_csr *a) { return a->rowptr[a->n]; }

int lo_csr_alloc(lo_csr *a, int64_t n, int64_t nnz) {
  a->n = n;
  a->ncols = n;
  a->rowptr = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  a->col = (int32_t *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int32_t));
  a->val = (double *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(double));
  a->symmetric = 0;
  a->is_f32 = 0;
  return (a->rowptr && a->col && a->val) ? 0 : -1;
}

int64_t lo_part_begin(int64_t n, int64_t p, int64_t k) {
  const int64_t base = n / p, rem = n % p;
  return k * base + (k < rem ? k : rem);
}

/* box-equidistant.hpp:67-79: q_d = prod_{e != d} h_e / h_d with h = L / N */
void lo_axis_quotients(const int64_t dims[3], const double lengths[3], double q[3]) {
  double h[3];
  for (int d = 0; d < 3; ++d) h[d] = lengths[d] / (double)dims[d];
  for (int d = 0; d < 3; ++d) {
    double area = 1.0;
    for (int e = 0; e < 3; ++e)
      if (e != d) area = area * h[e];
    q[d] = area / h[d];
  }
}

/* math/harmonic-mean.hpp:13-25: 2ab/(a+b) if ab != 0 else 0 */
double lo_harmonic_mean(double a, double b) {
  const double p = a * b;
  return p != 0.0 ? (p + p) / (a + b) : 0.0;
}

/* test/aux/materials.hpp:217-233: (sum of coordinates except the flow axis)
 * modulo the material count; index -> position is row-major, last axis
 * fastest (python-reference/defs/defs.py:63-70). */
void lo_material_diagonal_lines(const int64_t dims[3], int64_t max_material_num, uint8_t *mat) {
  const int64_t n = dims[0] * dims[1] * dims[2];
  for (int64_t i = 0; i < n; ++i) {
    const int64_t z = i % dims[2], y = (i / dims[2]) % dims[1];
    mat[i] = (uint8_t)((y + z) % max_material_num);
  }
}

/* python-reference/defs/materials.py:22-38 (flow axis 0) */
void lo_material_flow_cylinder_gap(const int64_t dims[3], double radius, uint8_t *mat) {
  const int64_t n = dims[0] * dims[1] * dims[2];
  const int64_t mid = dims[0] / 2;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t z = i % dims[2], y = (i / dims[2]) % dims[1], x = i / (dims[1] * dims[2]);
    const double fy = (double)y / (double)dims[1] - 0.5, fz = (double)z / (double)dims[2] - 0.5;
    const double v = fy * fy + fz * fz;
    mat[i] = (v <= radius && x != mid) ? 3 : 0;
  }
}

/* lookup-wright.hpp:73-85 */
void lo_lookup_tables(const double coeffs[4], const double q[3], double conn[48]) {
  for (int d = 0; d < 3; ++d)
    for (int f = 0; f < 16; ++f)
      conn[d * 16 + f] = lo_harmonic_mean(coeffs[f / 4], coeffs[f % 4]) * q[d];
}

double lo_diffusion_factor(const lo_stencil *s, int a, int b) {
  if (!s->henry) return lo_harmonic_mean(s->coeffs[a], s->coeffs[b]);
  const double fa = (s->gaseous_mask >> a) & 1 ? s->henry_constant : 1.0;
  const double fb = (s->gaseous_mask >> b) & 1 ? s->henry_constant : 1.0;
  return lo_harmonic_mean(s->coeffs[a] * fb, s->coeffs[b] * fa);
}

void lo_stencil_init(lo_stencil *s) {
  if (s->k) return;
  lo_lookup_tables(s->coeffs, s->q, s->conn);
  if (s->henry)
    for (int d = 0; d < 3; ++d)
      for (int f = 0; f < 16; ++f) s->conn[d * 16 + f] = lo_diffusion_factor(s, f / 4, f % 4) * s->q[d];
}

static inline double st_cell_value(const lo_stencil *s, int64_t i) {
  return s->k ? s->k[i] : s->coeffs[s->mat[i]];
}
/* connection_value (lookup: table gather; value: hm(k_from, k_to) * q_d;
 * values: the same with the conductivities of axis d) */
static inline double st_conn(const lo_stencil *s, int d, int64_t from, int64_t to) {
  if (s->k) {
    const double *kd = d == 1 && s->k1 ? s->k1 : d == 2 && s->k2 ? s->k2 : s->k;
    return lo_harmonic_mean(kd[from], kd[to]) * s->q[d];
  }
  return s->conn[d * 16 + s->mat[from] * 4 + s->mat[to]];
}

typedef struct {
  int64_t cols[7];
  double vals[7];
  int cnt;     /* off-diagonal entries in visiting order, then the diagonal */
  double diag;
} st_row;

/* algorithm.hpp:93-227 (valued, unordered): diagonal starts at
 * diagonal_base (0), border summands of the flow axis (start, end), then the
 * "before" neighbours of dims 0,1,2 and the "after" neighbours of dims 2,1,0
 * each adding their connection value; finally valuator.diagonal(). */
static void st_make_row(const lo_stencil *s, int64_t idx, st_row *row) {
  const int64_t n1 = s->dims[1], n2 = s->dims[2];
  const int64_t stride[3] = {n1 * n2, n2, 1};
  const int64_t pos[3] = {idx / (n1 * n2), (idx / n2) % n1, idx % n2};
  const double cv = st_cell_value(s, idx);
  double diag = 0.0;
  if (pos[0] == 0) diag += (2.0 * s->q[0]) * cv;
  if (pos[0] + 1 == s->dims[0]) diag += (2.0 * s->q[0]) * cv;
  row->cnt = 0;
  for (int d = 0; d < 3; ++d) {
    if (pos[d] > 0) {
      const int64_t j = idx - stride[d];
      const double c = st_conn(s, d, idx, j);
      row->cols[row->cnt] = j;
      row->vals[row->cnt] = -c;
      ++row->cnt;
      diag += c;
    }
  }
  for (int d = 2; d >= 0; --d) {
    if (pos[d] + 1 < s->dims[d]) {
      const int64_t j = idx + stride[d];
      const double c = st_conn(s, d, idx, j);
      row->cols[row->cnt] = j;
      row->vals[row->cnt] = -c;
      ++row->cnt;
      diag += c;
    }
  }
  if (s->zero_to_one && diag == 0.0) diag = 1.0;
  row->diag = diag;
}

void lo_stencil_spmv(const lo_stencil *s, const double *x, double *y) {
  const int64_t n = s->dims[0] * s->dims[1] * s->dims[2];
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    st_row row;
    st_make_row(s, i, &row);
    double sum = 0.0;
    for (int e = 0; e < row.cnt; ++e) sum = fma(row.vals[e], x[row.cols[e]], sum);
    y[i] = fma(row.diag, x[i], sum);
  }
}

void lo_stencil_diagonal(const lo_stencil *s, double *d) {
  const int64_t n = s->dims[0] * s->dims[1] * s->dims[2];
  for (int64_t i = 0; i < n; ++i) {
    st_row row;
    st_make_row(s, i, &row);
    d[i] = row.diag;
  }
}

/* stencil/vector/shared.hpp:181-205: border_rhs_summand = 2 q_0 c * u_D */
void lo_stencil_rhs(const lo_stencil *s, double *b) {
  const int64_t n1 = s->dims[1], n2 = s->dims[2];
  const int64_t n = s->dims[0] * n1 * n2;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t p0 = i / (n1 * n2);
    const double cv = st_cell_value(s, i);
    double sum = 0.0;
    if (p0 == 0) sum += ((2.0 * s->q[0]) * cv) * s->sol_start;
    if (p0 + 1 == s->dims[0]) sum += ((2.0 * s->q[0]) * cv) * s->sol_end;
    b[i] = sum;
  }
}

/* EffDiffCalc (component-wise/sink/effective-diffusion.hpp:226-320) on the
 * two middle planes of the flow axis (cells of plane mid = n0 / 2 and their
 * neighbours in plane mid + 1):
 *   area_part = sum(filled(c1) + filled(c2)) / (n1 n2) / 2      (AreaPartSink)
 *   flux      = sum hm(c1, c2) (x(c2) - x(c1))                   (EffDiffSink)
 *   eff       = flux q0 / (area_part L1 L2) L0 / (u_end - u_start)
 * with hm the harmonic mean of the two cells' coefficients (the lookup or
 * value valuator's diffusion_coeff), filled(c) = 0 for materials flagged in
 * none_mask (lookup valuator; every cell is filled for the value valuator)
 * and, with a compress map, only pairs whose cells both have a row.  Sums
 * run in cell order. */
double lo_effective_diffusion(const lo_stencil *s, const double lengths[3], uint8_t none_mask,
                              const double *sol, const int64_t *compress_map,
                              double *area_part) {
  const int64_t n1 = s->dims[1], n2 = s->dims[2], other = n1 * n2;
  const int64_t mid = s->dims[0] / 2;
  int64_t filled = 0;
  double flux = 0.0;
  for (int64_t c = 0; c < other; ++c) {
    const int64_t i1 = mid * other + c, i2 = i1 + other;
    if (s->mat) {
      filled += !((none_mask >> s->mat[i1]) & 1u);
      filled += !((none_mask >> s->mat[i2]) & 1u);
    } else {
      filled += 2;
    }
    const double hm = s->mat ? lo_diffusion_factor(s, s->mat[i1], s->mat[i2])
                             : lo_harmonic_mean(st_cell_value(s, i1), st_cell_value(s, i2));
    if (compress_map) {
      const int64_t k1 = compress_map[i1], k2 = compress_map[i2];
      if (k1 >= 0 && k2 >= 0) flux += hm * (sol[k2] - sol[k1]);
    } else {
      flux += hm * (sol[i2] - sol[i1]);
    }
  }
  const double ap = (double)filled / (double)other * 0.5;
  if (area_part) *area_part = ap;
  double out = flux;
  out *= s->q[0];
  out /= ap * (lengths[1] * lengths[2]);
  out *= lengths[0];
  return out / (s->sol_end - s->sol_start);
}

/* csr/create-from.hpp:82-232: rows of the stencil matrix with zero
 * off-diagonals dropped and sorted columns; with ZeroToZero valuators rows
 * whose diagonal is 0 are removed (compress map). */
int lo_stencil_to_csr(const lo_stencil *s, lo_csr *out, int64_t *compress_map) {
  const int64_t n = s->dims[0] * s->dims[1] * s->dims[2];
  int64_t *cmap = (int64_t *)malloc((size_t)n * sizeof(int64_t));
  int64_t rows = 0, nnz = 0;
  for (int64_t i = 0; i < n; ++i) {
    st_row row;
    st_make_row(s, i, &row);
    if (!s->zero_to_one && row.diag == 0.0) {
      cmap[i] = -1;
      continue;
    }
    cmap[i] = rows++;
    nnz += 1;
    for (int e = 0; e < row.cnt; ++e) nnz += row.vals[e] != 0.0;
  }
  if (lo_csr_alloc(out, rows, nnz)) {
    free(cmap);
    return -1;
  }
  int64_t pos = 0, r = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (cmap[i] < 0) continue;
    st_row row;
    st_make_row(s, i, &row);
    out->rowptr[r] = pos;
    /* sorted insertion: before entries are ascending, then diagonal, then after ascending */
    int64_t cols[7];
    double vals[7];
    int cnt = 0;
    for (int e = 0; e < row.cnt; ++e) {
      if (row.vals[e] == 0.0) continue;
      cols[cnt] = cmap[row.cols[e]];
      vals[cnt] = row.vals[e];
      ++cnt;
    }
    cols[cnt] = r;
    vals[cnt] = row.diag;
    ++cnt;
    for (int a = 1; a < cnt; ++a) { /* insertion sort, tiny */
      int64_t c = cols[a];
      double v = vals[a];
      int b = a - 1;
      while (b >= 0 && cols[b] > c) {
        cols[b + 1] = cols[b];
        vals[b + 1] = vals[b];
        --b;
      }
      cols[b + 1] = c;
      vals[b + 1] = v;
    }
    for (int e = 0; e < cnt; ++e) {
      out->col[pos] = (int32_t)cols[e];
      out->val[pos] = vals[e];
      ++pos;
    }
    ++r;
  }
  out->rowptr[rows] = pos;
  out->symmetric = 1;
  if (compress_map) memcpy(compress_map, cmap, (size_t)n * sizeof(int64_t));
  free(cmap);
  return 0;
}

/* Generic structured assembly used by the 27-point and 7-point generators.
 * Rows are independent: a parallel count pass, offsets, a parallel fill. */
static int64_t structured_row_len(const int64_t dims[3], int npts, int64_t i) {
  const int64_t n0 = dims[0], n1 = dims[1], n2 = dims[2];
  const int64_t p[3] = {i / (n1 * n2), (i / n2) % n1, i % n2};
  int64_t c = 1;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b)
      for (int cc = -1; cc <= 1; ++cc) {
        const int m = abs(a) + abs(b) + abs(cc);
        if (m == 0 || (npts == 7 && m != 1)) continue;
        if (p[0] + a < 0 || p[0] + a >= n0 || p[1] + b < 0 || p[1] + b >= n1 ||
            p[2] + cc < 0 || p[2] + cc >= n2)
          continue;
        ++c;
      }
  return c;
}

static int gen_structured(const int64_t dims[3], const double *k, int npts, lo_csr *out) {
  const int64_t n0 = dims[0], n1 = dims[1], n2 = dims[2];
  const int64_t n = n0 * n1 * n2;
  int64_t *len = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
  if (!len) return -1;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) len[i] = structured_row_len(dims, npts, i);
  int64_t nnz = 0;
  for (int64_t i = 0; i < n; ++i) nnz += len[i];
  if (lo_csr_alloc(out, n, nnz)) {
    free(len);
    return -1;
  }
  int64_t pos = 0;
  for (int64_t i = 0; i < n; ++i) {
    out->rowptr[i] = pos;
    pos += len[i];
  }
  out->rowptr[n] = pos;
  free(len);
  static const double w[4] = {0.0, 1.0, 0.5, 0.25};
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const int64_t p[3] = {i / (n1 * n2), (i / n2) % n1, i % n2};
    int64_t pos_i = out->rowptr[i];
    const double ki = k[i];
    double diag = 0.0;
    if (p[0] == 0) diag = diag + 2.0 * ki;
    if (p[0] + 1 == n0) diag = diag + 2.0 * ki;
    int64_t dpos = -1;
    /* offsets in ascending column order: a (axis 0) outermost */
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b)
        for (int cc = -1; cc <= 1; ++cc) {
          const int m = abs(a) + abs(b) + abs(cc);
          if (npts == 7 && m > 1) continue;
          if (p[0] + a < 0 || p[0] + a >= n0 || p[1] + b < 0 || p[1] + b >= n1 ||
              p[2] + cc < 0 || p[2] + cc >= n2)
            continue;
          const int64_t j = i + a * n1 * n2 + b * n2 + cc;
          out->col[pos_i] = (int32_t)j;
          if (m == 0) {
            dpos = pos_i;
            out->val[pos_i] = 0.0;
          } else {
            const double c = lo_harmonic_mean(ki, k[j]) * w[m];
            out->val[pos_i] = -c;
            diag = diag + c;
          }
          ++pos_i;
        }
    if (diag == 0.0) diag = 1.0;
    out->val[dpos] = diag;
  }
  out->symmetric = 1;
  return 0;
}

int lo_gen_27pt(const int64_t dims[3], const double *k, lo_csr *out) {
  return gen_structured(dims, k, 27, out);
}
int lo_gen_7pt(const int64_t dims[3], const double *k, lo_csr *out) {
  return gen_structured(dims, k, 7, out);
}

/* First-order upwind convection-diffusion, D = 1, unit spacing:
 * a_ij = -(1 + max(-v_d*s, 0)) for the neighbour at side s (+1/-1) of axis d,
 * a_ii = sum of |a_ij| over all six directions (missing neighbours act as
 * zero Dirichlet values, so they still count). */
int lo_gen_convdiff(const int64_t dims[3], const double v[3], lo_csr *out) {
  const int64_t n0 = dims[0], n1 = dims[1], n2 = dims[2];
  const int64_t n = n0 * n1 * n2;
  const int64_t stride[3] = {n1 * n2, n2, 1};
  int64_t nnz = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t p[3] = {i / (n1 * n2), (i / n2) % n1, i % n2};
    nnz += 1;
    for (int d = 0; d < 3; ++d) nnz += (p[d] > 0) + (p[d] + 1 < dims[d]);
  }
  if (lo_csr_alloc(out, n, nnz)) return -1;
  int64_t pos = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t p[3] = {i / (n1 * n2), (i / n2) % n1, i % n2};
    out->rowptr[i] = pos;
    double off[6];
    for (int d = 0; d < 3; ++d) {
      const double up_minus = v[d] > 0.0 ? v[d] : 0.0;  /* inflow from the - side */
      const double up_plus = v[d] < 0.0 ? -v[d] : 0.0;  /* inflow from the + side */
      off[2 * d] = 1.0 + up_minus;
      off[2 * d + 1] = 1.0 + up_plus;
    }
    double diag = 0.0;
    for (int e = 0; e < 6; ++e) diag = diag + off[e];
    /* ascending columns: -d0, -d1, -d2, diag, +d2, +d1, +d0 */
    for (int d = 0; d < 3; ++d)
      if (p[d] > 0) {
        out->col[pos] = (int32_t)(i - stride[d]);
        out->val[pos++] = -off[2 * d];
      }
    out->col[pos] = (int32_t)i;
    out->val[pos++] = diag;
    for (int d = 2; d >= 0; --d)
      if (p[d] + 1 < dims[d]) {
        out->col[pos] = (int32_t)(i + stride[d]);
        out->val[pos++] = -off[2 * d + 1];
      }
  }
  out->rowptr[n] = pos;
  out->symmetric = 0;
  return 0;
}

/* matrix-vector-product.hpp:71-82 */
void lo_csr_spmv(const lo_csr *a, const double *x, double *y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < a->n; ++i) {
    double sum = 0.0;
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) sum = fma(a->val[e], x[a->col[e]], sum);
    y[i] = sum;
  }
}

void lo_csr_residual(const lo_csr *a, const double *b, const double *x, double *r) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < a->n; ++i) {
    double sum = 0.0;
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) sum = fma(a->val[e], x[a->col[e]], sum);
    r[i] = b[i] - sum;
  }
}

/* accumulator.hpp:28-48 sums per-thread partials (merged through
 * atomic_ref, in arrival order).  Here the partials belong to LO_DOT_BLOCKS
 * fixed contiguous blocks, each summed in index order and merged in block
 * order, so the result is the same for every thread count. */
double lo_dot(int64_t n, const double *a, const double *b) {
  double part[LO_DOT_BLOCKS];
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < LO_DOT_BLOCKS; ++k) {
    const int64_t lo = lo_part_begin(n, LO_DOT_BLOCKS, k), hi = lo_part_begin(n, LO_DOT_BLOCKS, k + 1);
    double s = 0.0;
    for (int64_t i = lo; i < hi; ++i) s += a[i] * b[i];
    part[k] = s;
  }
  double s = 0.0;
  for (int64_t k = 0; k < LO_DOT_BLOCKS; ++k) s += part[k];
  return s;
}
double lo_norm2sq(int64_t n, const double *a) { return lo_dot(n, a, a); }
double lo_max_norm(int64_t n, const double *a) {
  double m = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double v = fabs(a[i]);
    if (v > m) m = v;
  }
  return m;
}

/* splitmix64 finaliser: priority of vertex i for the colouring */
static uint64_t lo_hash(uint64_t seed, uint64_t i) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + i + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Jones-Plassmann: in each round every uncoloured vertex whose (priority,
 * index) exceeds that of all uncoloured neighbours takes the smallest colour
 * not used by an already coloured neighbour (colours of the current round
 * are not visible within the round, so the result is order independent). */
int32_t lo_colour_jp(const lo_csr *a, uint64_t seed, int32_t *colour) {
  const int64_t n = a->n;
  uint64_t *prio = (uint64_t *)malloc((size_t)n * sizeof(uint64_t));
  int32_t *next = (int32_t *)malloc((size_t)n * sizeof(int32_t));
  for (int64_t i = 0; i < n; ++i) {
    prio[i] = lo_hash(seed, (uint64_t)i);
    colour[i] = -1;
  }
  int64_t left = n;
  int32_t ncol = 0;
  while (left > 0) {
    /* a round reads colour[] only and writes next[i] of its own vertex */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      next[i] = -1;
      if (colour[i] >= 0) continue;
      int is_max = 1;
      uint64_t used = 0; /* colours < 64 as a bitmask, larger ones by scan */
      for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) {
        const int64_t j = a->col[e];
        if (j == i) continue;
        if (colour[j] < 0) {
          if (prio[j] > prio[i] || (prio[j] == prio[i] && j > i)) {
            is_max = 0;
            break;
          }
        } else if (colour[j] < 64) {
          used |= 1ull << colour[j];
        }
      }
      if (!is_max) continue;
      int32_t c = 0;
      for (;;) {
        int taken = 0;
        if (c < 64) {
          taken = (int)((used >> c) & 1ull);
        } else {
          for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e)
            if (a->col[e] != i && colour[a->col[e]] == c) taken = 1;
        }
        if (!taken) break;
        ++c;
      }
      next[i] = c;
    }
    int64_t done = 0;
    int32_t top = ncol;
#pragma omp parallel for schedule(static) reduction(+ : done) reduction(max : top)
    for (int64_t i = 0; i < n; ++i)
      if (next[i] >= 0) {
        colour[i] = next[i];
        ++done;
        if (next[i] + 1 > top) top = next[i] + 1;
      }
    left -= done;
    ncol = top;
  }
  free(prio);
  free(next);
  return ncol;
}

/* Smallest-last greedy colouring, restated from its specification (the
 * library's lgx_colour_smallest_last): buckets by remaining off-diagonal
 * degree, each a list whose head is the most recent insertion (initial
 * insertion in index order); repeatedly remove the head of the lowest
 * non-empty bucket and move its remaining neighbours (CSR order) to the
 * head of the bucket below; colour in reverse removal order with the
 * smallest colour no coloured neighbour has. */
static int32_t colour_smallest_last_rows(const lo_csr *a, int32_t *colour);

static int cmp_i32(const void *x, const void *y) {
  const int32_t a = *(const int32_t *)x, b = *(const int32_t *)y;
  return (a > b) - (a < b);
}

/* The adjacency the colouring uses: a's rows when the off-diagonal pattern
 * is structurally symmetric (returns 0), else in *out the pattern of A + A^T
 * with sorted rows and no diagonal (returns 1; the caller frees it). */
static int sl_symmetrised(const lo_csr *a, lo_csr *out) {
  const int64_t n = a->n;
  int64_t *tp = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i)
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e)
      if (a->col[e] != i) ++tp[a->col[e] + 1];
  for (int64_t i = 0; i < n; ++i) tp[i + 1] += tp[i];
  int32_t *tc = (int32_t *)malloc((size_t)(tp[n] + 1) * sizeof(int32_t));
  int64_t *fill = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) fill[i] = tp[i];
  for (int64_t i = 0; i < n; ++i)
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e)
      if (a->col[e] != i) tc[fill[a->col[e]]++] = (int32_t)i;
  int64_t maxrow = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t len = a->rowptr[i + 1] - a->rowptr[i] + tp[i + 1] - tp[i];
    if (len > maxrow) maxrow = len;
  }
  int32_t *row = (int32_t *)malloc((size_t)(maxrow + 1) * sizeof(int32_t));
  int symmetric = 1;
  for (int64_t i = 0; i < n && symmetric; ++i) {
    int64_t m = 0;
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e)
      if (a->col[e] != i) row[m++] = a->col[e];
    qsort(row, (size_t)m, sizeof(int32_t), cmp_i32);
    if (m != tp[i + 1] - tp[i]) symmetric = 0;
    for (int64_t k = 0; k < m && symmetric; ++k)
      if (row[k] != tc[tp[i] + k]) symmetric = 0;
  }
  if (!symmetric) {
    int64_t total = 0;
    int64_t *rp = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
    int32_t *cc = (int32_t *)malloc((size_t)(a->rowptr[n] + tp[n] + 1) * sizeof(int32_t));
    rp[0] = 0;
    for (int64_t i = 0; i < n; ++i) {
      int64_t m = 0;
      for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e)
        if (a->col[e] != i) row[m++] = a->col[e];
      for (int64_t k = tp[i]; k < tp[i + 1]; ++k) row[m++] = tc[k];
      qsort(row, (size_t)m, sizeof(int32_t), cmp_i32);
      for (int64_t k = 0; k < m; ++k)
        if (k == 0 || row[k] != row[k - 1]) cc[total++] = row[k];
      rp[i + 1] = total;
    }
    memset(out, 0, sizeof(*out));
    out->n = n;
    out->ncols = n;
    out->rowptr = rp;
    out->col = cc;
  }
  free(tp);
  free(tc);
  free(fill);
  free(row);
  return !symmetric;
}

int32_t lo_colour_smallest_last(const lo_csr *a_in, int32_t *colour) {
  lo_csr sym;
  const int own = a_in->n > 0 && sl_symmetrised(a_in, &sym);
  const lo_csr *a = own ? &sym : a_in;
  const int32_t nc = colour_smallest_last_rows(a, colour);
  if (own) {
    free(sym.rowptr);
    free(sym.col);
  }
  return nc;
}

static int32_t colour_smallest_last_rows(const lo_csr *a, int32_t *colour) {
  const int64_t n = a->n;
  if (n <= 0) return 0;
  int64_t *d = (int64_t *)malloc((size_t)n * sizeof(int64_t));
  int64_t *nx = (int64_t *)malloc((size_t)n * sizeof(int64_t));
  int64_t *pv = (int64_t *)malloc((size_t)n * sizeof(int64_t));
  unsigned char *gone = (unsigned char *)calloc((size_t)n, 1);
  int64_t *order = (int64_t *)malloc((size_t)n * sizeof(int64_t));
  int64_t dmax = 0;
  for (int64_t i = 0; i < n; ++i) {
    d[i] = 0;
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) d[i] += a->col[e] != i;
    if (d[i] > dmax) dmax = d[i];
  }
  int64_t *top = (int64_t *)malloc((size_t)(dmax + 1) * sizeof(int64_t));
  for (int64_t b = 0; b <= dmax; ++b) top[b] = -1;
  for (int64_t i = 0; i < n; ++i) {  /* insert at the head of bucket d[i] */
    pv[i] = -1;
    nx[i] = top[d[i]];
    if (nx[i] >= 0) pv[nx[i]] = i;
    top[d[i]] = i;
  }
  int64_t b = 0;
  for (int64_t k = 0; k < n; ++k) {
    while (top[b] < 0) ++b;
    const int64_t v = top[b];
    top[b] = nx[v];
    if (nx[v] >= 0) pv[nx[v]] = -1;
    gone[v] = 1;
    order[k] = v;
    for (int64_t e = a->rowptr[v]; e < a->rowptr[v + 1]; ++e) {
      const int64_t u = a->col[e];
      if (u == v || gone[u]) continue;
      /* out of bucket d[u] ... */
      if (pv[u] >= 0) nx[pv[u]] = nx[u]; else top[d[u]] = nx[u];
      if (nx[u] >= 0) pv[nx[u]] = pv[u];
      /* ... into the head of bucket d[u] - 1 */
      d[u] -= 1;
      pv[u] = -1;
      nx[u] = top[d[u]];
      if (nx[u] >= 0) pv[nx[u]] = u;
      top[d[u]] = u;
    }
    if (b > 0) b -= 1;
  }
  int64_t *seen = (int64_t *)malloc((size_t)(dmax + 2) * sizeof(int64_t));
  for (int64_t c = 0; c <= dmax + 1; ++c) seen[c] = -1;
  for (int64_t i = 0; i < n; ++i) colour[i] = -1;
  int32_t nc = 0;
  for (int64_t k = n - 1; k >= 0; --k) {
    const int64_t v = order[k];
    for (int64_t e = a->rowptr[v]; e < a->rowptr[v + 1]; ++e)
      if (a->col[e] != v && colour[a->col[e]] >= 0) seen[colour[a->col[e]]] = v;
    int32_t c = 0;
    while (seen[c] == v) ++c;
    colour[v] = c;
    if (c + 1 > nc) nc = c + 1;
  }
  free(d);
  free(nx);
  free(pv);
  free(gone);
  free(order);
  free(top);
  free(seen);
  return nc;
}

void lo_colour_order(int64_t n, const int32_t *colour, int32_t ncolours, int32_t *order) {
  int64_t pos = 0;
  for (int32_t c = 0; c < ncolours; ++c)
    for (int64_t i = 0; i < n; ++i)
      if (colour[i] == c) order[pos++] = (int32_t)i;
}
