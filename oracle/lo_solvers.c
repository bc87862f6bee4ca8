/*
 * Oracle smoothers, Krylov solvers and the coarse Cholesky solver.
 * TEST INFRASTRUCTURE ONLY (see lineal_oracle.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "lineal_oracle.h"

/* jacobi/sweep.hpp:66-87 */
void lo_jacobi_sweep(const lo_csr *a, double relax, const double *x_in, double *x_out,
                     const double *b) {
  const double m1 = 1.0 - relax;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < a->n; ++i) {
    double accum = b[i], diag = 0.0;
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) {
      const int64_t j = a->col[e];
      if (j == i) {
        diag = a->val[e];
      } else {
        accum = fma(-a->val[e], x_in ? x_in[j] : 0.0, accum);
      }
    }
    const double quot = accum / diag;
    x_out[i] = fma(relax, quot, m1 * (x_in ? x_in[i] : 0.0));
  }
}

/* One row of gauss-seidel-variant/sweep.hpp:134-200.  use_new(j) tells
 * whether x_out[j] (already updated in this sweep) is read instead of x_in[j];
 * in_range(j) is the thread-range test used by the ultra variant. */
static inline void sor_row(const lo_csr *a, int64_t i, double relax, double m1, const double *x_in,
                           double *x_out, const double *b, int ultra, int64_t pb, int64_t pe,
                           const int32_t *rank, int forward) {
  double accum = b[i], diag = 0.0, div = 0.0;
  const double xi = x_in ? x_in[i] : 0.0;
  for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) {
    const int64_t j = a->col[e];
    const double aij = a->val[e];
    if (j == i) {
      diag = aij;
      if (ultra) accum = fma(-aij, xi, accum);
      continue;
    }
    int contains, use_new;
    if (rank) {
      contains = 1;
      use_new = forward ? (rank[j] < rank[i]) : (rank[j] > rank[i]);
    } else {
      contains = (j >= pb && j < pe);
      use_new = contains && (forward ? (j < i) : (j > i));
    }
    if (ultra && !contains) div += fabs(aij);
    const double xj = use_new ? x_out[j] : (x_in ? x_in[j] : 0.0);
    accum = fma(-aij, xj, accum);
  }
  if (ultra) {
    x_out[i] = xi + relax * accum / (fabs(diag) + 0.5 * div);
  } else {
    const double quot = accum / diag;
    x_out[i] = fma(relax, quot, m1 * xi);
  }
}

void lo_sor_sweep(const lo_csr *a, double relax, const double *x_in, double *x_out,
                  const double *b, int forward, int ultra, int64_t nparts) {
  const double m1 = 1.0 - relax;
  if (nparts < 1) nparts = 1;
  if (nparts > a->n && a->n > 0) nparts = a->n;
#pragma omp parallel for schedule(static, 1)
  for (int64_t p = 0; p < nparts; ++p) {
    const int64_t pb = lo_part_begin(a->n, nparts, p), pe = lo_part_begin(a->n, nparts, p + 1);
    if (forward) {
      for (int64_t i = pb; i < pe; ++i) sor_row(a, i, relax, m1, x_in, x_out, b, ultra, pb, pe, NULL, 1);
    } else {
      for (int64_t i = pe - 1; i >= pb; --i)
        sor_row(a, i, relax, m1, x_in, x_out, b, ultra, pb, pe, NULL, 0);
    }
  }
}

void lo_sor_sweep_ordered(const lo_csr *a, double relax, const double *x_in, double *x_out,
                          const double *b, int forward, int ultra, const int32_t *order) {
  const double m1 = 1.0 - relax;
  const int64_t n = a->n;
  int32_t *rank = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
  for (int64_t k = 0; k < n; ++k) rank[order[k]] = (int32_t)k;
  if (forward) {
    for (int64_t k = 0; k < n; ++k)
      sor_row(a, order[k], relax, m1, x_in, x_out, b, ultra, 0, n, rank, 1);
  } else {
    for (int64_t k = n - 1; k >= 0; --k)
      sor_row(a, order[k], relax, m1, x_in, x_out, b, ultra, 0, n, rank, 0);
  }
  free(rank);
}

void lo_sor_sweep_coloured(const lo_csr *a, double relax, const double *x_in, double *x_out,
                           const double *b, int forward, int ultra, const int32_t *order,
                           const int32_t *colour, const int64_t *colour_ptr, int32_t ncolours) {
  const double m1 = 1.0 - relax;
  for (int32_t cc = 0; cc < ncolours; ++cc) {
    const int32_t c = forward ? cc : ncolours - 1 - cc;
#pragma omp parallel for schedule(static)
    for (int64_t k = colour_ptr[c]; k < colour_ptr[c + 1]; ++k) {
      /* rank order = colour order for a proper colouring: colour[] stands in
       * for the rank of sor_row */
      sor_row(a, order[k], relax, m1, x_in, x_out, b, ultra, 0, a->n, colour, forward);
    }
  }
}

int lo_colouring_is_proper(const lo_csr *a, const int32_t *colour) {
  int proper = 1;
#pragma omp parallel for schedule(static) reduction(&& : proper)
  for (int64_t i = 0; i < a->n; ++i)
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e)
      if (a->col[e] != i && colour[a->col[e]] == colour[i]) proper = 0;
  return proper;
}

/* The float smoother of the precision form: the row of sor_row in float
 * arithmetic (fmaf, float division) on the matrix values rounded to float,
 * rows visited in `order` (rank-based new/old choice, so ultra adds no
 * off-range term). */
void lo_sor_sweep_ordered_f32(const lo_csr *a, float relax, const float *x_in, float *x_out,
                              const float *b, int forward, int ultra, const int32_t *order) {
  const float m1 = 1.0f - relax;
  const int64_t n = a->n;
  int32_t *rank = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
  for (int64_t k = 0; k < n; ++k) rank[order[k]] = (int32_t)k;
  for (int64_t kk = 0; kk < n; ++kk) {
    const int64_t i = order[forward ? kk : n - 1 - kk];
    float accum = b[i], diag = 0.0f;
    const float xi = x_in ? x_in[i] : 0.0f;
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) {
      const int64_t j = a->col[e];
      const float aij = (float)a->val[e];
      if (j == i) {
        diag = aij;
        if (ultra) accum = fmaf(-aij, xi, accum);
        continue;
      }
      const int use_new = forward ? (rank[j] < rank[i]) : (rank[j] > rank[i]);
      const float xj = use_new ? x_out[j] : (x_in ? x_in[j] : 0.0f);
      accum = fmaf(-aij, xj, accum);
    }
    if (ultra) {
      x_out[i] = xi + relax * accum / fabsf(diag);
    } else {
      const float quot = accum / diag;
      x_out[i] = fmaf(relax, quot, m1 * xi);
    }
  }
  free(rank);
}

/* ---- Cholesky (cholesky/decomposition.hpp:52-107) -------------------- */
int lo_cholesky_factor(const lo_csr *a, double *l) {
  const int64_t n = a->n;
  memset(l, 0, (size_t)(n * n) * sizeof(double));
  /* lower_builder rows; a dense row plus a "stored" flag reproduces the
   * sparse builder because entries equal to zero are never inserted. */
  for (int64_t i = 0; i < n; ++i) {
    double *li = l + i * n;
    double diag = 0.0;
    /* lambda(j, base): value = (base - dot(row_j, row_i so far)) / L_jj */
#define LO_CHOL_LAMBDA(J, BASE)                                              \
  do {                                                                       \
    const int64_t jj = (J);                                                  \
    const double *lj = l + jj * n;                                           \
    double dp = 0.0;                                                         \
    for (int64_t kk = 0; kk < jj; ++kk)                                      \
      if (li[kk] != 0.0 && lj[kk] != 0.0) dp += li[kk] * lj[kk];             \
    const double value = ((BASE) - dp) / lj[jj];                             \
    if (value != 0.0) {                                                      \
      diag -= value * value;                                                 \
      li[jj] = value;                                                        \
    }                                                                        \
  } while (0)
    int64_t next_start = 0;
    int is_first = 1;
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) {
      const int64_t j = a->col[e];
      if (j < i) {
        if (is_first) {
          is_first = 0;
        } else {
          for (int64_t k = next_start; k < j; ++k) LO_CHOL_LAMBDA(k, 0.0);
        }
        LO_CHOL_LAMBDA(j, a->val[e]);
        next_start = j + 1;
      } else if (j == i) {
        diag += a->val[e];
      }
    }
    for (int64_t j = next_start; j < i; ++j) LO_CHOL_LAMBDA(j, 0.0);
#undef LO_CHOL_LAMBDA
    if (!(diag >= 0.0)) return -1;
    li[i] = sqrt(diag);
  }
  return 0;
}

/* substitution.hpp:27-55 (forward) and 91-115 (column-oriented backward
 * substitution with the transpose) */
void lo_cholesky_solve(int64_t n, const double *l, const double *b, double *x) {
  double *aux = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
  for (int64_t i = 0; i < n; ++i) {
    double sum = b[i];
    const double *li = l + i * n;
    for (int64_t j = 0; j < i; ++j)
      if (li[j] != 0.0) sum -= li[j] * aux[j];
    aux[i] = sum / li[i];
  }
  for (int64_t i = 0; i < n; ++i) x[i] = aux[i];
  for (int64_t j = n - 1; j >= 0; --j) {
    const double *lj = l + j * n;
    const double sj = x[j] / lj[j];
    x[j] = sj;
    for (int64_t i = 0; i < j; ++i)
      if (lj[i] != 0.0) x[i] = x[i] - lj[i] * sj;
  }
  free(aux);
}

/* lu/decomposition.hpp:31-122 (row-wise LU without pivoting), dense storage:
 * row i starts from A's row; each lower entry j < i, in increasing j (fill-in
 * included), becomes l_ij = w_j / u_jj and subtracts l_ij times U's row j
 * past its diagonal; then u_ii = w_i and u_ik = w_k for k > i (unit lower
 * diagonal).  lu holds L below and U on and above the diagonal.  Returns 0,
 * or -1 for a zero pivot. */
int lo_lu_factor(const lo_csr *a, double *lu) {
  const int64_t n = a->n;
  memset(lu, 0, (size_t)(n * n) * sizeof(double));
  for (int64_t i = 0; i < n; ++i) {
    double *w = lu + i * n;
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) w[a->col[e]] = a->val[e];
    for (int64_t j = 0; j < i; ++j) {
      if (w[j] == 0.0) continue;
      const double *uj = lu + j * n;
      const double l = w[j] / uj[j];
      w[j] = l;
      for (int64_t k = j + 1; k < n; ++k)
        if (uj[k] != 0.0) w[k] -= l * uj[k];
    }
    if (w[i] == 0.0) return -1;
  }
  return 0;
}

/* lu/solver.hpp:37-60: forward substitution with the unit lower factor,
 * backward substitution with the upper factor */
void lo_lu_solve(int64_t n, const double *lu, const double *b, double *x) {
  for (int64_t i = 0; i < n; ++i) {
    double sum = b[i];
    const double *li = lu + i * n;
    for (int64_t j = 0; j < i; ++j)
      if (li[j] != 0.0) sum -= li[j] * x[j];
    x[i] = sum;
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    double sum = x[i];
    const double *ui = lu + i * n;
    for (int64_t k = i + 1; k < n; ++k)
      if (ui[k] != 0.0) sum -= ui[k] * x[k];
    x[i] = sum / ui[i];
  }
}

/* ---- preconditioner application: z = M^-1 r from a zero start -------- */
static void precon_apply(const lo_csr *a, const lo_precon *m, const double *r, double *z,
                         double *aux) {
  switch (m ? m->kind : LO_PRECON_NONE) {
    case LO_PRECON_JACOBI: lo_jacobi_sweep(a, m->relax, NULL, z, r); break;
    case LO_PRECON_SSOR:
      /* SsorBroom (gauss-seidel-variant/solver.hpp:44-89): forward into aux, backward into z */
      lo_sor_sweep(a, m->relax, NULL, aux, r, 1, m->ultra, m->nparts);
      lo_sor_sweep(a, m->relax, aux, z, r, 0, m->ultra, m->nparts);
      break;
    case LO_PRECON_AMG: lo_amg_vcycle(m->amg, r, z); break;
    default: memcpy(z, r, (size_t)a->n * sizeof(double)); break;
  }
}

/* conjugate-gradients/solver.hpp:50-115 */
int64_t lo_pcg(const lo_csr *a, const double *b, double *x, const lo_precon *m, double rtol,
               int64_t maxit, int64_t rere_period, double *history) {
  const int64_t n = a->n;
  const int has_precon = m && m->kind != LO_PRECON_NONE;
  double *r = (double *)malloc((size_t)n * sizeof(double));
  double *q = (double *)malloc((size_t)n * sizeof(double));
  double *p = (double *)malloc((size_t)n * sizeof(double));
  double *aux = (double *)malloc((size_t)n * sizeof(double));
  double res2, rho;
  lo_csr_residual(a, b, x, r);
  res2 = lo_norm2sq(n, r);
  if (has_precon) {
    precon_apply(a, m, r, p, aux);
    rho = lo_dot(n, p, r);
  } else {
    memcpy(p, r, (size_t)n * sizeof(double));
    rho = res2;
  }
  const double r0 = sqrt(res2);
  if (history) history[0] = r0;
  int64_t it = 0;
  while (it < maxit && sqrt(res2) > rtol * r0 && rho != 0.0) {
    lo_csr_spmv(a, p, q);
    const double alpha = rho / lo_dot(n, p, q);
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) x[i] = x[i] + p[i] * alpha;
    if (rere_period > 0 && it > 0 && it % rere_period == 0) {
      lo_csr_residual(a, b, x, r);
    } else {
      #pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) r[i] = r[i] - q[i] * alpha;
    }
    res2 = lo_norm2sq(n, r);
    const double old_rho = rho;
    if (has_precon) {
      precon_apply(a, m, r, q, aux);
      rho = lo_dot(n, r, q);
      const double beta = rho / old_rho;
      #pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) p[i] = q[i] + p[i] * beta;
    } else {
      rho = res2;
      const double beta = rho / old_rho;
      #pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) p[i] = r[i] + p[i] * beta;
    }
    ++it;
    if (history) history[it] = sqrt(res2);
  }
  free(r);
  free(q);
  free(p);
  free(aux);
  return it;
}

/* bicgstab/solver.hpp:51-151 */
int64_t lo_pbicgstab(const lo_csr *a, const double *b, double *x, const lo_precon *m,
                     double rtol, int64_t maxit, int64_t rere_period, double *history) {
  const int64_t n = a->n;
  const int has_precon = m && m->kind != LO_PRECON_NONE;
  double *r = (double *)malloc((size_t)n * sizeof(double));
  double *r0v = (double *)malloc((size_t)n * sizeof(double));
  double *p = (double *)malloc((size_t)n * sizeof(double));
  double *v = (double *)malloc((size_t)n * sizeof(double));
  double *t = (double *)malloc((size_t)n * sizeof(double));
  double *px = (double *)malloc((size_t)n * sizeof(double));
  double *aux = (double *)malloc((size_t)n * sizeof(double));
  lo_csr_residual(a, b, x, r);
  memcpy(r0v, r, (size_t)n * sizeof(double));
  memcpy(p, r, (size_t)n * sizeof(double));
  double res2 = lo_norm2sq(n, r), rho = res2, alpha = 0.0, omega = 0.0;
  const double rn0 = sqrt(res2);
  if (history) history[0] = rn0;
  int64_t it = 0;
  while (it < maxit && sqrt(res2) > rtol * rn0 && rho != 0.0) {
    const double *y = p;
    if (has_precon) {
      precon_apply(a, m, p, px, aux);
      y = px;
    }
    lo_csr_spmv(a, y, v);
    alpha = rho / lo_dot(n, r0v, v);
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) x[i] = x[i] + y[i] * alpha;
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) r[i] = r[i] - v[i] * alpha;
    res2 = lo_norm2sq(n, r);
    const double *z = r;
    if (has_precon) {
      precon_apply(a, m, r, px, aux);
      z = px;
    }
    lo_csr_spmv(a, z, t);
    const double on = lo_dot(n, t, r), od = lo_norm2sq(n, t);
    omega = on / od;
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) x[i] = x[i] + z[i] * omega;
    const double old_rho = rho;
    if (rere_period > 0 && it > 0 && it % rere_period == 0) {
      lo_csr_residual(a, b, x, r);
    } else {
      #pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) r[i] = r[i] - t[i] * omega;
    }
    rho = lo_dot(n, r, r0v);
    res2 = lo_norm2sq(n, r);
    const double beta = (rho / old_rho) * (alpha / omega);
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) p[i] = r[i] + (p[i] - v[i] * omega) * beta;
    ++it;
    if (history) history[it] = sqrt(res2);
  }
  free(r);
  free(r0v);
  free(p);
  free(v);
  free(t);
  free(px);
  free(aux);
  return it;
}
