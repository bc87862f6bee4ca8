/*
 * Oracle aggregation AMG: strength of connection, greedy aggregation per
 * partition, aggregate-map merge, Galerkin product, hierarchy and V-cycle.
 * TEST INFRASTRUCTURE ONLY (see lineal_oracle.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "lineal_oracle.h"

void lo_amg_default_params(lo_amg_params *p) {
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
  p->relax = 1.0;
  p->smoother_relax = 1.0;
  p->smoother_ultra = 0;
  p->smoother_parts = 0;
  p->colour_seed = 0x5eed;
  p->coarse_smallest_last = 0;
}

static int64_t find_col(const lo_csr *a, int64_t row, int64_t col) {
  int64_t lo = a->rowptr[row], hi = a->rowptr[row + 1];
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (a->col[mid] < col) lo = mid + 1; else hi = mid;
  }
  return (lo < a->rowptr[row + 1] && a->col[lo] == col) ? lo : -1;
}

static int64_t diag_pos(const lo_csr *a, int64_t row) { return find_col(a, row, row); }

/* dependency/criterion.hpp:35-78, graph weights via NegativeOffdiagonalTransform
 * (weight-transform.hpp:28-38): w_ij = -a_ij, vertex weight a_jj.
 * strength = max(w_ij,0) * w_ji' / a_jj with w_ji' = max(w_ij,0) for
 * value-symmetric matrices, else max(w_ji,0) (0 if absent); strong iff
 * strength > theta * max_strength of the row.  For float matrices the
 * arithmetic is float (GraphWeight = matrix value type). */
void lo_amg_strength(const lo_csr *a, double theta, uint8_t *depends, uint8_t *influences,
                     uint8_t *isolated) {
  const int64_t n = a->n;
  const int64_t nnz = lo_csr_nnz(a);
  memset(depends, 0, (size_t)nnz);
  memset(influences, 0, (size_t)nnz);
  double *strength = (double *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(double));
  double *diag = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) diag[i] = a->val[diag_pos(a, i)];
  /* row i writes depends of its own entries and influences of the entry
   * (j, i) of each neighbour row j: no two rows write the same byte */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    if (a->is_f32) {
      float maxs = 0.0f;
      for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) {
        const int64_t j = a->col[e];
        if (j == i) continue;
        const float w = -(float)a->val[e];
        const float nn = w > 0.0f ? w : 0.0f;
        float opp;
        if (a->symmetric) {
          opp = nn;
        } else {
          const int64_t r = find_col(a, j, i);
          const float wr = r >= 0 ? -(float)a->val[r] : 0.0f;
          opp = r >= 0 ? (wr > 0.0f ? wr : 0.0f) : 0.0f;
        }
        const float s = nn * opp / (float)diag[j];
        strength[e] = s;
        if (s > maxs) maxs = s;
      }
      const float lb = (float)theta * maxs;
      int any = 0;
      for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) {
        const int64_t j = a->col[e];
        if (j == i) continue;
        const int cond = (float)strength[e] > lb;
        any |= cond;
        depends[e] = (uint8_t)cond;
        const int64_t r = find_col(a, j, i);
        if (r >= 0) influences[r] = (uint8_t)cond;
      }
      isolated[i] = (uint8_t)!any;
    } else {
      double maxs = 0.0;
      for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) {
        const int64_t j = a->col[e];
        if (j == i) continue;
        const double w = -a->val[e];
        const double nn = w > 0.0 ? w : 0.0;
        double opp;
        if (a->symmetric) {
          opp = nn;
        } else {
          const int64_t r = find_col(a, j, i);
          const double wr = r >= 0 ? -a->val[r] : 0.0;
          opp = r >= 0 ? (wr > 0.0 ? wr : 0.0) : 0.0;
        }
        const double s = nn * opp / diag[j];
        strength[e] = s;
        if (s > maxs) maxs = s;
      }
      const double lb = theta * maxs;
      int any = 0;
      for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) {
        const int64_t j = a->col[e];
        if (j == i) continue;
        const int cond = strength[e] > lb;
        any |= cond;
        depends[e] = (uint8_t)cond;
        const int64_t r = find_col(a, j, i);
        if (r >= 0) influences[r] = (uint8_t)cond;
      }
      isolated[i] = (uint8_t)!any;
    }
  }
  free(strength);
  free(diag);
}

/* ---- greedy aggregation (aggregation/base.hpp:28-711) ----------------- */
typedef struct {
  const lo_csr *a;
  const uint8_t *dep, *inf, *iso;
  int64_t pb, pe;             /* partition [pb, pe) */
  uint32_t *agg;              /* global map, local aggregate ids during aggregation */
  int32_t min_size, max_size;
  /* coarse -> fine lists: block k holds up to max_size vertices */
  int32_t *blocks;
  int32_t *block_len;
  int64_t counter;            /* AggregateGenerator::aggregate_counter_ */
  /* front: sorted set + markers (AggregateFront, base.hpp:28-74) */
  int32_t *front;
  int64_t front_len;
  uint8_t *front_mark;
  /* connected aggregates (AggregateHelpers::connected) */
  int64_t *conn;
  int64_t conn_len, conn_cap;
  int32_t *cand;
  int64_t cand_len;
  int64_t stats[5];
} agg_state;

static int front_contains(const agg_state *s, int64_t v) { return s->front_mark[v - s->pb]; }
static void front_insert(agg_state *s, int64_t v) {
  int64_t lo = 0, hi = s->front_len;
  while (lo < hi) {
    const int64_t mid = (lo + hi) / 2;
    if (s->front[mid] < v) lo = mid + 1; else hi = mid;
  }
  if (lo < s->front_len && s->front[lo] == v) return;
  memmove(s->front + lo + 1, s->front + lo, (size_t)(s->front_len - lo) * sizeof(int32_t));
  s->front[lo] = (int32_t)v;
  ++s->front_len;
  s->front_mark[v - s->pb] = 1;
}
static void front_erase(agg_state *s, int64_t v) {
  int64_t lo = 0, hi = s->front_len;
  while (lo < hi) {
    const int64_t mid = (lo + hi) / 2;
    if (s->front[mid] < v) lo = mid + 1; else hi = mid;
  }
  if (lo < s->front_len && s->front[lo] == v) {
    memmove(s->front + lo, s->front + lo + 1, (size_t)(s->front_len - lo - 1) * sizeof(int32_t));
    --s->front_len;
  }
  s->front_mark[v - s->pb] = 0;
}
static void helpers_clear(agg_state *s) {
  for (int64_t k = 0; k < s->front_len; ++k) s->front_mark[s->front[k] - s->pb] = 0;
  s->front_len = 0;
  s->conn_len = 0;
}
static int is_connected(const agg_state *s, uint32_t ag) {
  for (int64_t k = 0; k < s->conn_len; ++k)
    if (s->conn[k] == (int64_t)ag) return 1;
  return 0;
}
static inline int in_range(const agg_state *s, int64_t v) { return v >= s->pb && v < s->pe; }

/* AggregateManager::add_help (base.hpp:263-287) */
static void add_help(agg_state *s, int64_t v, uint32_t agg, int64_t *vertex_num) {
  ++*vertex_num;
  s->agg[v] = agg;
  s->blocks[(int64_t)agg * s->max_size + s->block_len[agg]++] = (int32_t)v;
  const lo_csr *a = s->a;
  for (int64_t e = a->rowptr[v]; e < a->rowptr[v + 1]; ++e) {
    const int64_t t = a->col[e];
    if (t == v || !in_range(s, t)) continue;
    const uint32_t ta = s->agg[t];
    if (ta < LO_ISOLATED) {
      if (!is_connected(s, ta)) {
        if (s->conn_len == s->conn_cap) {
          s->conn_cap *= 2;
          s->conn = (int64_t *)realloc(s->conn, (size_t)s->conn_cap * sizeof(int64_t));
        }
        s->conn[s->conn_len++] = ta;
      }
    }
    if (ta == LO_UNAGGREGATED && !front_contains(s, t)) front_insert(s, t);
  }
}

static void add_candidates(agg_state *s, uint32_t agg, int64_t *vertex_num) {
  for (int64_t k = 0; k < s->cand_len; ++k) {
    front_erase(s, s->cand[k]);
    add_help(s, s->cand[k], agg, vertex_num);
  }
}

/* grow_aggregate (base.hpp:532-585) */
static void grow(agg_state *s, uint32_t agg, int64_t *size) {
  const lo_csr *a = s->a;
  while (*size < s->min_size) {
    int64_t m0 = 0, m2 = 0;
    double m1 = 0.0;
    int has_cons2 = 0;
    s->cand_len = 0;
    for (int64_t f = 0; f < s->front_len; ++f) {
      const int64_t vtx = s->front[f];
      if (s->iso[vtx]) continue;
      int64_t con = 0, nbs = 0, cons2 = 0, cons1 = 0;
      for (int64_t e = a->rowptr[vtx]; e < a->rowptr[vtx + 1]; ++e) {
        const int64_t t = a->col[e];
        if (t == vtx || !in_range(s, t)) continue;
        const uint32_t ha = s->agg[t];
        const int dep = s->dep[e], inf = s->inf[e];
        con += (ha < LO_ISOLATED) && is_connected(s, ha);
        nbs += front_contains(s, t);
        cons2 += (ha == agg) && (inf && dep);
        cons1 += (ha == agg) && (!inf && dep);
      }
      const int64_t adj = (a->rowptr[vtx + 1] - a->rowptr[vtx]) - 1; /* full off-diagonal count */
      const double cond = (double)con / (double)adj;
      if (cons2 > 0 && !has_cons2) {
        has_cons2 = 1;
        m0 = cons2;
        m1 = cond;
        m2 = nbs;
        s->cand_len = 0;
        s->cand[s->cand_len++] = (int32_t)vtx;
      } else {
        const int64_t t0 = has_cons2 ? cons2 : cons1;
        if (t0 > 0) {
          /* lexicographic <=> on (Size, double, Size) */
          int cmp;
          if (t0 != m0) cmp = t0 > m0 ? 1 : -1;
          else if (cond != m1) cmp = cond > m1 ? 1 : (cond < m1 ? -1 : 2 /* unordered */);
          else if (nbs != m2) cmp = nbs > m2 ? 1 : -1;
          else cmp = 0;
          if (cmp == 1) {
            m0 = t0;
            m1 = cond;
            m2 = nbs;
            s->cand_len = 0;
            s->cand[s->cand_len++] = (int32_t)vtx;
          } else if (cmp == 0) {
            s->cand[s->cand_len++] = (int32_t)vtx;
          }
        }
      }
    }
    if (s->cand_len == 0) break;
    const int64_t room = s->max_size - *size;
    if (s->cand_len > room) s->cand_len = room;
    add_candidates(s, agg, size);
  }
}

/* round_aggregate (base.hpp:601-636) */
static void round_agg(agg_state *s, uint32_t agg, int64_t *size) {
  const lo_csr *a = s->a;
  while (*size < s->max_size) {
    s->cand_len = 0;
    for (int64_t f = 0; f < s->front_len; ++f) {
      const int64_t vtx = s->front[f];
      if (s->iso[vtx]) continue;
      int64_t cons = 0, unagg = 0, inagg = 0;
      for (int64_t e = a->rowptr[vtx]; e < a->rowptr[vtx + 1]; ++e) {
        const int64_t t = a->col[e];
        if (t == vtx || !in_range(s, t)) continue;
        const uint32_t ha = s->agg[t];
        cons += (ha == agg) && s->dep[e];
        unagg += ha == LO_UNAGGREGATED;
        inagg += ha == agg;
      }
      if (cons == 0 || unagg >= inagg) continue;
      s->cand[s->cand_len++] = (int32_t)vtx;
      break;
    }
    if (s->cand_len == 0) break;
    const int64_t room = s->max_size - *size;
    if (s->cand_len > room) s->cand_len = room;
    add_candidates(s, agg, size);
  }
}

/* handle_vertex (base.hpp:638-677) */
static void handle_vertex(agg_state *s, int64_t seed, int aggressive) {
  if (s->agg[seed] != LO_UNAGGREGATED) return;
  if (s->iso[seed]) {
    s->agg[seed] = LO_ISOLATED;
    ++s->stats[4];
    return;
  }
  const uint32_t agg = (uint32_t)s->counter;
  int64_t size = 0;
  add_help(s, seed, agg, &size);
  grow(s, agg, &size);
  round_agg(s, agg, &size);
  if (size == 1 && s->max_size > 1) {
    /* find_merge_aggregate (base.hpp:487-503): first strong in-range edge whose
     * head lies in an aggregate with room */
    const lo_csr *a = s->a;
    uint32_t target = LO_UNAGGREGATED;
    for (int64_t e = a->rowptr[seed]; e < a->rowptr[seed + 1]; ++e) {
      const int64_t t = a->col[e];
      if (t == seed || !in_range(s, t)) continue;
      if (!(s->dep[e] || s->inf[e])) continue;
      const uint32_t ta = s->agg[t];
      if (ta < LO_ISOLATED && s->block_len[ta] < s->max_size) {
        target = ta;
        break;
      }
    }
    if (target != LO_UNAGGREGATED) {
      /* move_to (multithread.hpp:210-230) */
      s->block_len[agg] = 0;
      s->agg[seed] = target;
      s->blocks[(int64_t)target * s->max_size + s->block_len[target]++] = (int32_t)seed;
      ++s->stats[3];
      helpers_clear(s);
      return;
    }
    if (aggressive) {
      s->block_len[agg] = 0;
      s->agg[seed] = LO_ISOLATED;
      ++s->stats[4];
      helpers_clear(s);
      return;
    }
    ++s->stats[2];
  } else {
    ++s->stats[1];
  }
  ++s->counter; /* finalize -> next_index */
  helpers_clear(s);
}

int64_t lo_amg_aggregate(const lo_csr *a, const uint8_t *depends, const uint8_t *influences,
                         const uint8_t *isolated, int32_t min_size, int32_t max_size,
                         int64_t nparts, int aggressive, uint32_t *agg, int64_t **list_ptr_out,
                         int32_t **list_out, int64_t stats[5]) {
  const int64_t n = a->n;
  if (nparts < 1) nparts = 1;
  if (nparts > n && n > 0) nparts = n;
  for (int64_t i = 0; i < n; ++i) agg[i] = LO_UNAGGREGATED;
  int64_t *pcount = (int64_t *)calloc((size_t)nparts + 1, sizeof(int64_t));
  int32_t **pblocks = (int32_t **)calloc((size_t)nparts, sizeof(int32_t *));
  int32_t **plens = (int32_t **)calloc((size_t)nparts, sizeof(int32_t *));
  int64_t st[5] = {0, 0, 0, 0, 0};
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : st[:5])
  for (int64_t p = 0; p < nparts; ++p) {
    agg_state s;
    memset(&s, 0, sizeof(s));
    s.a = a;
    s.dep = depends;
    s.inf = influences;
    s.iso = isolated;
    s.pb = lo_part_begin(n, nparts, p);
    s.pe = lo_part_begin(n, nparts, p + 1);
    s.agg = agg;
    s.min_size = min_size;
    s.max_size = max_size;
    const int64_t psize = s.pe - s.pb;
    s.blocks = (int32_t *)malloc((size_t)(psize * max_size + 1) * sizeof(int32_t));
    s.block_len = (int32_t *)calloc((size_t)psize + 1, sizeof(int32_t));
    s.front = (int32_t *)malloc((size_t)(psize + 1) * sizeof(int32_t));
    s.front_mark = (uint8_t *)calloc((size_t)psize + 1, 1);
    s.conn_cap = 64;
    s.conn = (int64_t *)malloc((size_t)s.conn_cap * sizeof(int64_t));
    s.cand = (int32_t *)malloc((size_t)(psize + 1) * sizeof(int32_t));
    for (int64_t v = s.pb; v < s.pe; ++v) handle_vertex(&s, v, aggressive);
    s.stats[0] = s.counter;
    for (int k = 0; k < 5; ++k) st[k] += s.stats[k];
    pcount[p] = s.counter;
    pblocks[p] = s.blocks;
    plens[p] = s.block_len;
    free(s.front);
    free(s.front_mark);
    free(s.conn);
    free(s.cand);
  }
  /* merge (multithread.hpp:107-143): aggregate offsets by partition */
  int64_t *poff = (int64_t *)calloc((size_t)nparts + 1, sizeof(int64_t));
  for (int64_t p = 0; p < nparts; ++p) poff[p + 1] = poff[p] + pcount[p];
  const int64_t ncoarse = poff[nparts];
  int64_t *lp = (int64_t *)malloc((size_t)(ncoarse + 1) * sizeof(int64_t));
  int64_t total = 0;
  for (int64_t p = 0; p < nparts; ++p)
    for (int64_t k = 0; k < pcount[p]; ++k) total += plens[p][k];
  int32_t *ls = (int32_t *)malloc((size_t)(total > 0 ? total : 1) * sizeof(int32_t));
  int64_t pos = 0, c = 0;
  for (int64_t p = 0; p < nparts; ++p) {
    const int64_t pb = lo_part_begin(n, nparts, p), pe = lo_part_begin(n, nparts, p + 1);
    for (int64_t v = pb; v < pe; ++v)
      if (agg[v] < LO_ISOLATED) agg[v] += (uint32_t)poff[p];
    for (int64_t k = 0; k < pcount[p]; ++k) {
      lp[c++] = pos;
      for (int32_t m = 0; m < plens[p][k]; ++m) ls[pos++] = pblocks[p][k * max_size + m];
    }
    free(pblocks[p]);
    free(plens[p]);
  }
  lp[ncoarse] = pos;
  free(pcount);
  free(poff);
  free(pblocks);
  free(plens);
  if (stats)
    for (int k = 0; k < 5; ++k) stats[k] = st[k];
  *list_ptr_out = lp;
  *list_out = ls;
  return ncoarse;
}

/* transport/matrix-shared.hpp:85-183 with the non-unique builder of
 * csr/shared.hpp:730-764: per coarse row, fine rows in aggregate-list order,
 * columns ascending; each value is cast to the coarse value type, then
 * accumulated in double per coarse column in first-encounter order; the row
 * is sorted by column and stored in the coarse value type.  Columns whose
 * fine vertex is isolated are dropped. */
/* one coarse row: distinct columns in first-encounter order with their
 * double sums; where[J] holds J's slot in cols (or -1) and is reset on
 * return.  Returns the column count. */
static int64_t galerkin_row(const lo_csr *a, const uint32_t *agg, const int64_t *list_ptr,
                            const int32_t *list, int coarse_f32, int64_t c, int64_t *where,
                            int64_t *cols, double *vals) {
  int64_t m = 0;
  for (int64_t k = list_ptr[c]; k < list_ptr[c + 1]; ++k) {
    const int64_t i = list[k];
    for (int64_t e = a->rowptr[i]; e < a->rowptr[i + 1]; ++e) {
      const uint32_t J = agg[a->col[e]];
      if (J >= LO_ISOLATED) continue;
      const double v = coarse_f32 ? (double)(float)a->val[e] : a->val[e];
      const int64_t f = where[J];
      if (f < 0) {
        where[J] = m;
        cols[m] = J;
        vals[m] = v;
        ++m;
      } else {
        vals[f] += v;
      }
    }
  }
  for (int64_t x = 0; x < m; ++x) where[cols[x]] = -1;
  return m;
}

int lo_amg_galerkin(const lo_csr *a, int64_t ncoarse, const uint32_t *agg, const int64_t *list_ptr,
                    const int32_t *list, int coarse_f32, lo_csr *out) {
  int64_t *cnt = (int64_t *)calloc((size_t)ncoarse + 1, sizeof(int64_t));
  int64_t maxrow = 0;
#pragma omp parallel for schedule(static) reduction(max : maxrow)
  for (int64_t c = 0; c < ncoarse; ++c) {
    int64_t u = 0;
    for (int64_t k = list_ptr[c]; k < list_ptr[c + 1]; ++k)
      u += a->rowptr[list[k] + 1] - a->rowptr[list[k]];
    if (u > maxrow) maxrow = u;
  }
  int failed = 0;
  /* pass 1: count distinct columns; pass 2: fill.  Rows are independent,
   * each thread keeps its own slot map and row buffers. */
  for (int pass = 0; pass < 2 && !failed; ++pass) {
    if (pass == 1) {
      int64_t nnz = 0;
      for (int64_t c = 0; c < ncoarse; ++c) nnz += cnt[c];
      if (lo_csr_alloc(out, ncoarse, nnz)) {
        failed = 1;
        break;
      }
      int64_t pos = 0;
      for (int64_t c = 0; c < ncoarse; ++c) {
        out->rowptr[c] = pos;
        pos += cnt[c];
      }
      out->rowptr[ncoarse] = pos;
    }
#pragma omp parallel
    {
      int64_t *where = (int64_t *)malloc((size_t)(ncoarse + 1) * sizeof(int64_t));
      int64_t *cols = (int64_t *)malloc((size_t)(maxrow + 1) * sizeof(int64_t));
      double *vals = (double *)malloc((size_t)(maxrow + 1) * sizeof(double));
      for (int64_t c = 0; c <= ncoarse; ++c) where[c] = -1;
#pragma omp for schedule(static)
      for (int64_t c = 0; c < ncoarse; ++c) {
        const int64_t m = galerkin_row(a, agg, list_ptr, list, coarse_f32, c, where, cols, vals);
        if (pass == 0) {
          cnt[c] = m;
          continue;
        }
        for (int64_t x = 1; x < m; ++x) { /* insertion sort by column */
          const int64_t cc = cols[x];
          const double vv = vals[x];
          int64_t y = x - 1;
          while (y >= 0 && cols[y] > cc) {
            cols[y + 1] = cols[y];
            vals[y + 1] = vals[y];
            --y;
          }
          cols[y + 1] = cc;
          vals[y + 1] = vv;
        }
        int64_t pos = out->rowptr[c];
        for (int64_t x = 0; x < m; ++x) {
          out->col[pos] = (int32_t)cols[x];
          out->val[pos] = coarse_f32 ? (double)(float)vals[x] : vals[x];
          ++pos;
        }
      }
      free(where);
      free(cols);
      free(vals);
    }
  }
  free(cnt);
  if (failed) return -1;
  out->symmetric = a->symmetric;
  out->is_f32 = coarse_f32;
  return 0;
}

static void csr_copy(const lo_csr *a, lo_csr *b) {
  const int64_t nnz = lo_csr_nnz(a);
  lo_csr_alloc(b, a->n, nnz);
  memcpy(b->rowptr, a->rowptr, (size_t)(a->n + 1) * sizeof(int64_t));
  memcpy(b->col, a->col, (size_t)nnz * sizeof(int32_t));
  memcpy(b->val, a->val, (size_t)nnz * sizeof(double));
  b->ncols = a->ncols;
  b->symmetric = a->symmetric;
  b->is_f32 = a->is_f32;
}

static void level_vectors(lo_amg_level *l, const lo_amg_params *p, int64_t idx,
                          const int32_t *given_colour, int32_t given_nc) {
  const int64_t n = l->a.n;
  l->b = (double *)calloc((size_t)n + 1, sizeof(double));
  l->x = (double *)calloc((size_t)n + 1, sizeof(double));
  l->r = (double *)calloc((size_t)n + 1, sizeof(double));
  l->order = NULL;
  l->colour = NULL;
  l->colour_ptr = NULL;
  l->ncolours = 0;
  if (p->smoother_parts == 0) {
    int32_t *colour = (int32_t *)malloc((size_t)(n + 1) * sizeof(int32_t));
    int32_t nc;
    if (given_colour) {
      memcpy(colour, given_colour, (size_t)n * sizeof(int32_t));
      nc = given_nc;
    } else {
      nc = p->coarse_smallest_last && idx > 0
             ? lo_colour_smallest_last(&l->a, colour)
             : lo_colour_jp(&l->a, p->colour_seed + (uint64_t)idx, colour);
    }
    l->order = (int32_t *)malloc((size_t)(n + 1) * sizeof(int32_t));
    lo_colour_order(n, colour, nc, l->order);
    l->colour = colour;
    l->ncolours = nc;
    if (lo_colouring_is_proper(&l->a, colour)) {
      l->colour_ptr = (int64_t *)calloc((size_t)nc + 1, sizeof(int64_t));
      for (int64_t i = 0; i < n; ++i) ++l->colour_ptr[colour[i] + 1];
      for (int32_t c = 0; c < nc; ++c) l->colour_ptr[c + 1] += l->colour_ptr[c];
    }
  }
}

int64_t lo_amg_partitions(int64_t n, int64_t level, const lo_amg_params *p) {
  double ps = (double)p->partition_size;
  for (int64_t l = 0; l < level; ++l) ps *= p->partition_growth;
  int64_t parts = ps >= 1.0 ? (int64_t)((double)n / ps) : n;
  const int64_t floor_parts = p->min_partitions < n / 1024 ? p->min_partitions : n / 1024;
  if (parts < floor_parts) parts = floor_parts;
  if (parts < 1) parts = 1;
  if (parts > p->max_partitions) parts = p->max_partitions;
  return parts;
}

/* hierarchy/wright.hpp:120-143 (level_action) and 146-309 (create_impl) */
int lo_agg_map_check(const lo_agg_map *m) {
  if (!m || m->n < 0 || m->ncoarse < 0 || (m->n > 0 && !m->agg) || !m->list_ptr ||
      (m->ncoarse > 0 && !m->list) || m->list_ptr[0] != 0)
    return LO_ERR_BAD_MAP;
  int64_t aggregated = 0;
  for (int64_t v = 0; v < m->n; ++v) {
    if (m->agg[v] == LO_ISOLATED) continue;
    if ((int64_t)m->agg[v] >= m->ncoarse) return LO_ERR_BAD_MAP;
    ++aggregated;
  }
  if (m->list_ptr[m->ncoarse] != aggregated) return LO_ERR_BAD_MAP;
  uint8_t *seen = (uint8_t *)calloc((size_t)m->n + 1, 1);
  int rc = 0;
  for (int64_t c = 0; c < m->ncoarse && rc == 0; ++c) {
    if (m->list_ptr[c + 1] <= m->list_ptr[c]) rc = LO_ERR_BAD_MAP;  /* empty aggregate */
    for (int64_t k = m->list_ptr[c]; k < m->list_ptr[c + 1] && rc == 0; ++k) {
      const int32_t v = m->list[k];
      if (v < 0 || v >= m->n || seen[v] || (int64_t)m->agg[v] != c) rc = LO_ERR_BAD_MAP;
      else seen[v] = 1;
    }
  }
  free(seen);
  return rc;
}

/* the level's aggregate map: computed (strength + aggregation), or copied
 * from a given map (FileAggregator, aggregation/independent.hpp:279-298) */
static int level_aggregates(const lo_csr *a, const lo_amg_params *p, int64_t level, int aggressive,
                            const lo_agg_map *given, lo_amg_level *fine, int64_t *nc_out) {
  if (given) {
    if (given->n != a->n) return LO_ERR_BAD_MAP;
    const int rc = lo_agg_map_check(given);
    if (rc) return rc;
    const int64_t nc = given->ncoarse, len = given->list_ptr[nc];
    fine->agg = (uint32_t *)malloc((size_t)(a->n + 1) * sizeof(uint32_t));
    fine->list_ptr = (int64_t *)malloc((size_t)(nc + 1) * sizeof(int64_t));
    fine->list = (int32_t *)malloc((size_t)(len + 1) * sizeof(int32_t));
    if (a->n) memcpy(fine->agg, given->agg, (size_t)a->n * sizeof(uint32_t));
    memcpy(fine->list_ptr, given->list_ptr, (size_t)(nc + 1) * sizeof(int64_t));
    if (len) memcpy(fine->list, given->list, (size_t)len * sizeof(int32_t));
    *nc_out = nc;
    return 0;
  }
  const int64_t nnz = lo_csr_nnz(a);
  uint8_t *dep = (uint8_t *)malloc((size_t)nnz + 1);
  uint8_t *inf = (uint8_t *)malloc((size_t)nnz + 1);
  uint8_t *iso = (uint8_t *)malloc((size_t)a->n + 1);
  lo_amg_strength(a, aggressive ? p->aggressive_threshold : p->strong_threshold, dep, inf, iso);
  fine->agg = (uint32_t *)malloc((size_t)(a->n + 1) * sizeof(uint32_t));
  int64_t stats[5];
  *nc_out = lo_amg_aggregate(a, dep, inf, iso, p->min_aggregate_size, p->max_aggregate_size,
                             lo_amg_partitions(a->n, level, p), aggressive, fine->agg,
                             &fine->list_ptr, &fine->list, stats);
  free(dep);
  free(inf);
  free(iso);
  return 0;
}

static int amg_setup(const lo_csr *a0, const lo_amg_params *p, const lo_agg_map *maps,
                     int64_t nmaps, const int32_t *colour0, int32_t nc0, lo_amg *h) {
  memset(h, 0, sizeof(*h));
  h->p = *p;
  csr_copy(a0, &h->lv[0].a);
  int aggressive = 0;
  int64_t level = 0;
  for (;;) {
    lo_amg_level *fine = &h->lv[level];
    const lo_csr *a = &fine->a;
    int64_t nc = 0;
    int rc = 0;
    if (maps && level >= nmaps) rc = LO_ERR_NO_MAP;
    else rc = level_aggregates(a, p, level, aggressive, maps ? &maps[level] : NULL, fine, &nc);
    if (rc) {
      h->nlevels = level + 1;  /* what lo_amg_free releases */
      return rc;
    }
    lo_amg_level *coarse = &h->lv[level + 1];
    lo_amg_galerkin(a, nc, fine->agg, fine->list_ptr, fine->list, p->coarse_f32, &coarse->a);
    level_vectors(fine, p, level, level == 0 ? colour0 : NULL, nc0);
    /* level_action: coarse < min size -> stop; too many levels -> stop;
     * factor * coarse > fine -> aggressive (or stop if already aggressive) */
    int stop = 0;
    const int64_t fsize = a->n, csize = coarse->a.n;
    if (csize < p->min_coarsen_size) {
      stop = 1;
    } else if (level + 1 >= p->max_level_num) {
      stop = 1;
    } else if (p->min_coarsen_factor * (double)csize > (double)fsize) {
      if (aggressive) stop = 1; else aggressive = 1;
    }
    ++level;
    if (stop || level + 1 >= 32) break;
  }
  h->nlevels = level + 1;
  lo_amg_level *last = &h->lv[level];
  last->b = (double *)calloc((size_t)last->a.n + 1, sizeof(double));
  last->x = (double *)calloc((size_t)last->a.n + 1, sizeof(double));
  last->r = (double *)calloc((size_t)last->a.n + 1, sizeof(double));
  h->chol = (double *)malloc((size_t)(last->a.n * last->a.n + 1) * sizeof(double));
  /* coarse solver: CholeskySolver for symmetric, LuSolver for nonsymmetric
   * hierarchies (test/aux/default.hpp:160-162) */
  return last->a.symmetric ? lo_cholesky_factor(&last->a, h->chol)
                           : lo_lu_factor(&last->a, h->chol);
}

int lo_amg_setup(const lo_csr *a, const lo_amg_params *p, lo_amg *h) {
  return amg_setup(a, p, NULL, 0, NULL, 0, h);
}

int lo_amg_setup_coloured(const lo_csr *a, const lo_amg_params *p, const int32_t *colour0,
                          int32_t ncolours0, lo_amg *h) {
  if (colour0) {
    for (int64_t i = 0; i < a->n; ++i)
      if (colour0[i] < 0 || colour0[i] >= ncolours0) {
        memset(h, 0, sizeof(*h));
        return LO_ERR_BAD_MAP;
      }
  }
  return amg_setup(a, p, NULL, 0, colour0, ncolours0, h);
}

int lo_amg_setup_given(const lo_csr *a, const lo_amg_params *p, const lo_agg_map *maps,
                       int64_t nmaps, lo_amg *h) {
  if (!maps || nmaps < 1) {
    memset(h, 0, sizeof(*h));
    return LO_ERR_NO_MAP;
  }
  return amg_setup(a, p, maps, nmaps, NULL, 0, h);
}

void lo_amg_free(lo_amg *h) {
  for (int64_t l = 0; l < h->nlevels; ++l) {
    lo_csr_free(&h->lv[l].a);
    free(h->lv[l].agg);
    free(h->lv[l].list_ptr);
    free(h->lv[l].list);
    free(h->lv[l].order);
    free(h->lv[l].colour);
    free(h->lv[l].colour_ptr);
    free(h->lv[l].b);
    free(h->lv[l].x);
    free(h->lv[l].r);
  }
  free(h->chol);
  memset(h, 0, sizeof(*h));
}

static void smooth(const lo_amg *h, const lo_amg_level *l, const double *x_in, double *x_out,
                   const double *b, int forward) {
  if (l->colour_ptr) {
    lo_sor_sweep_coloured(&l->a, h->p.smoother_relax, x_in, x_out, b, forward,
                          h->p.smoother_ultra, l->order, l->colour, l->colour_ptr, l->ncolours);
  } else if (l->order) {
    lo_sor_sweep_ordered(&l->a, h->p.smoother_relax, x_in, x_out, b, forward, h->p.smoother_ultra,
                         l->order);
  } else {
    lo_sor_sweep(&l->a, h->p.smoother_relax, x_in, x_out, b, forward, h->p.smoother_ultra,
                 h->p.smoother_parts);
  }
}

/* multigrid/solver.hpp:56-176 (REGULAR cycle, one iteration).  Pre-smoothing
 * is a forward SOR sweep from zero, the residual is restricted by aggregate
 * sums (vector-shared.hpp:49-56), the coarsest level is solved by Cholesky,
 * the correction is injected (vector-shared.hpp:121-134) scaled by 1/relax,
 * and post-smoothing is a backward SOR sweep in place. */
void lo_amg_vcycle(lo_amg *h, const double *b, double *x) {
  const int64_t L = h->nlevels;
  const double inv_relax = 1.0 / h->p.relax;
  for (int64_t l = 0; l + 1 < L; ++l) {
    lo_amg_level *lv = &h->lv[l];
    const double *bl = l == 0 ? b : lv->b;
    double *xl = l == 0 ? x : lv->x;
    smooth(h, lv, NULL, xl, bl, 1);
    lo_csr_residual(&lv->a, bl, xl, lv->r);
    lo_amg_level *cv = &h->lv[l + 1];
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < cv->a.n; ++c) {
      double s = 0.0;
      for (int64_t k = lv->list_ptr[c]; k < lv->list_ptr[c + 1]; ++k) s += lv->r[lv->list[k]];
      cv->b[c] = s;
    }
  }
  lo_amg_level *last = &h->lv[L - 1];
  if (last->a.symmetric)
    lo_cholesky_solve(last->a.n, h->chol, last->b, last->x);
  else
    lo_lu_solve(last->a.n, h->chol, last->b, last->x);
  for (int64_t l = L - 2; l >= 0; --l) {
    lo_amg_level *lv = &h->lv[l];
    const double *bl = l == 0 ? b : lv->b;
    double *xl = l == 0 ? x : lv->x;
    const double *xc = h->lv[l + 1].x;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < lv->a.n; ++i) {
      const uint32_t ag = lv->agg[i];
      const double ref = ag < LO_ISOLATED ? xc[ag] : 0.0;
      xl[i] = xl[i] + ref * inv_relax;
    }
    /* in-situ post smoothing: swap(sol, aux); sweep(aux -> sol) */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < lv->a.n; ++i) lv->r[i] = xl[i];
    smooth(h, lv, lv->r, xl, bl, 0);
  }
}
