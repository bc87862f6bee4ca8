/*
 * CPU restatement of lineal's shared-memory solve path (KurtBoehm/lineal).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle against which the
 * CUDA implementation in lineal_gb300/ is checked, and the CPU baseline that
 * bench.py times.  Nothing in the product links or calls it.
 *
 * Every routine names the reference file:line it restates (paths relative to
 * the lineal repository).  The reference itself cannot be built here (its
 * dependencies thesauros/grex are not vendored), so parity is pinned by the
 * reference's own golden data instead: test/python-reference/sor.py iterates,
 * test/python-reference/cholesky.py, test/data/UFZ_CT_02_{LHS.smf,RHS.dvf}
 * and the bound tables of test/shared-stencil.hpp / test/shared-csr.cpp.
 *
 * Floating-point conventions: compiled with -ffp-contract=off; wherever the
 * reference calls compat::fmadd / grex::fnmadd the restatement calls fma()
 * explicitly, everything else is a plain IEEE operation.
 */
#ifndef LINEAL_ORACLE_H
#define LINEAL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Aggregate sentinels, multigrid/types.hpp:87-88 (4-byte SizeByte). */
#define LO_UNAGGREGATED 0xFFFFFFFFu
#define LO_ISOLATED 0xFFFFFFFEu

/* CSR with sorted columns and a stored diagonal (csr/shared.hpp:258-262).
 * When is_f32 is set the values are exactly representable floats and
 * arithmetic that the reference performs in the matrix value type (AMG
 * strength, Galerkin storage) is done in float. */
typedef struct {
  int64_t n;
  int64_t ncols;
  int64_t *rowptr; /* n + 1 */
  int32_t *col;    /* nnz */
  double *val;     /* nnz */
  int symmetric;
  int is_f32;
} lo_csr;

void lo_csr_free(lo_csr *a);
int64_t lo_csr_nnz(const lo_csr *a);
int lo_csr_alloc(lo_csr *a, int64_t n, int64_t nnz);

/* Contiguous blocked partition of n items into p parts: part k starts at
 * k*(n/p) + min(k, n%p).  Stands in for thesauros' BlockedIndexSegmenter
 * (adaptive.hpp:266-268). */
int64_t lo_part_begin(int64_t n, int64_t p, int64_t k);
/* OpenMP threads of the later parallel loops (n > 0), and their number now */
void lo_set_threads(int n);
int lo_max_threads(void);

/* ---- geometry and valuators ---------------------------------------- */
/* box-equidistant.hpp:67-79 */
void lo_axis_quotients(const int64_t dims[3], const double lengths[3], double q[3]);
/* math/harmonic-mean.hpp:13-25 */
double lo_harmonic_mean(double a, double b);
/* test/aux/materials.hpp:217-233 (flow axis 0) */
void lo_material_diagonal_lines(const int64_t dims[3], int64_t max_material_num, uint8_t *mat);
/* test/python-reference/defs/materials.py:22-38 */
void lo_material_flow_cylinder_gap(const int64_t dims[3], double radius, uint8_t *mat);
/* lookup-wright.hpp:73-96: conn[d*16 + a*4 + b] = hm(c_a, c_b) * q_d */
void lo_lookup_tables(const double coeffs[4], const double q[3], double conn[48]);

/* 7-point diffusion stencil, one row (stencil/matrix/algorithm.hpp:93-227,
 * scalar valued unordered iteration; valuators stationary-diffusion-
 * {lookup,value}.hpp).  The cell value is k[cell] (value valuator) or
 * coeffs[mat[cell]] (lookup valuator; pass k=NULL).  Dirichlet borders only on
 * axis 0.  zero_to_one replaces a zero diagonal by 1. */
typedef struct {
  int64_t dims[3];
  double q[3];
  const double *k;        /* value valuator: conductivity per cell, or NULL */
  const uint8_t *mat;     /* lookup valuator: material per cell */
  double coeffs[4];       /* lookup valuator coefficients */
  double conn[48];        /* lookup tables (filled by lo_stencil_init) */
  double sol_start, sol_end;
  int zero_to_one;
  /* values valuator (stationary-diffusion-values.hpp:30-211): conductivity
   * per cell and axis, k for axis 0 (and the Dirichlet borders), k1 and k2
   * for axes 1 and 2; NULL: the value valuator's single k */
  const double *k1, *k2;
  /* HenryDiffusionLookupProvider (lookup-wright.hpp:38-60) when henry != 0:
   * diffusion factor hm(c_a f_b, c_b f_a), f = henry_constant for the
   * gaseous materials (bit m of gaseous_mask), else 1 */
  int henry;
  double henry_constant;
  int gaseous_mask;
} lo_stencil;

void lo_stencil_init(lo_stencil *s);
/* diffusion factor of materials a -> b (SymmetricDiffusionLookupProvider or
 * HenryDiffusionLookupProvider, lookup-wright.hpp:18-60) */
double lo_diffusion_factor(const lo_stencil *s, int a, int b);
/* EffDiffCalc (component-wise/sink/effective-diffusion.hpp:226-320): the
 * effective diffusivity of a solution through the middle planes of axis 0;
 * lengths are the axis lengths, none_mask flags "none" materials (bit m),
 * compress_map (NULL: identity) maps cells to solution rows (-1: removed).
 * *area_part (may be NULL) receives AreaPartSink's value. */
double lo_effective_diffusion(const lo_stencil *s, const double lengths[3], uint8_t none_mask,
                              const double *sol, const int64_t *compress_map,
                              double *area_part);
/* y = A x, products accumulated with fma in the scalar unordered order:
 * before (dims 0,1,2), after (dims 2,1,0), diagonal
 * (matrix-vector-product.hpp:71-82 applied to algorithm.hpp:178-225). */
void lo_stencil_spmv(const lo_stencil *s, const double *x, double *y);
/* diagonal entries (algorithm.hpp:346-357) */
void lo_stencil_diagonal(const lo_stencil *s, double *d);
/* Dirichlet right-hand side (stencil/vector/shared.hpp:181-205) */
void lo_stencil_rhs(const lo_stencil *s, double *b);
/* Stencil -> CSR (csr/create-from.hpp:37-239), zero off-diagonals dropped.
 * With zero_to_one == 0 rows whose diagonal is zero are removed and
 * compress_map[cell] gives the compressed row (or -1). */
int lo_stencil_to_csr(const lo_stencil *s, lo_csr *out, int64_t *compress_map);

/* 27-point variable-coefficient diffusion on a unit-spaced grid (no
 * reference counterpart; the reference stencil is 7-point).  Off-diagonal to
 * neighbour j at offset o: -hm(k_i, k_j) * w(|o|_1) with w = 1 (face),
 * 1/2 (edge), 1/4 (corner).  Diagonal: Dirichlet terms 2*k_i on both axis-0
 * faces first, then the off-diagonal weights in ascending column order. */
int lo_gen_27pt(const int64_t dims[3], const double *k, lo_csr *out);
/* 7-point variant of the same generator (value-valuator operator with q=1,
 * zero_to_one, assembled directly). */
int lo_gen_7pt(const int64_t dims[3], const double *k, lo_csr *out);
/* Upwind convection-diffusion 7-point (nonsymmetric), D=1, velocity v[3],
 * unit spacing, Dirichlet (zero) on all faces. */
int lo_gen_convdiff(const int64_t dims[3], const double v[3], lo_csr *out);

/* ---- CSR kernels ---------------------------------------------------- */
/* matrix-vector-product.hpp:71-82: sum = fma(a_ij, x_j, sum), columns ascending */
void lo_csr_spmv(const lo_csr *a, const double *x, double *y);
/* r = b - A x */
void lo_csr_residual(const lo_csr *a, const double *b, const double *x, double *r);
/* sequential-order reductions (accumulator.hpp:151-179 restated with a fixed order) */
/* fixed block partition of the reductions (thread-count independent) */
enum { LO_DOT_BLOCKS = 256 };
double lo_dot(int64_t n, const double *a, const double *b);
double lo_norm2sq(int64_t n, const double *a);
double lo_max_norm(int64_t n, const double *a);

/* ---- smoothers ------------------------------------------------------ */
/* jacobi/sweep.hpp:66-87.  x_in == NULL means a zero input vector. */
void lo_jacobi_sweep(const lo_csr *a, double relax, const double *x_in, double *x_out,
                     const double *b);
/* gauss-seidel-variant/sweep.hpp:134-200, scalar CSR path.
 * Rows are visited part by part (nparts contiguous blocked parts, each part
 * sequentially, forward or backward); a row reads the new value x_out[j] only
 * when j lies in its own part and before it in sweep order, otherwise x_in[j]
 * (thread-block-hybrid semantics, sweep.hpp:135-169).  ultra selects the l1
 * variant (sweep.hpp:170-173, 345-357).  x_in == NULL means zero. */
void lo_sor_sweep(const lo_csr *a, double relax, const double *x_in, double *x_out,
                  const double *b, int forward, int ultra, int64_t nparts);
/* The same sweep in an explicit row order: rows are processed in order[0..n)
 * (forward) or reversed (backward); a row reads x_out[j] when j was visited
 * before it, else x_in[j].  With order = colour classes this is the
 * multicolour sweep the GPU performs. */
void lo_sor_sweep_ordered(const lo_csr *a, double relax, const double *x_in, double *x_out,
                          const double *b, int forward, int ultra, const int32_t *order);
/* lo_sor_sweep_ordered for a proper colouring (no entry joins two rows of
 * one colour) whose order lists the rows colour by colour: colour_ptr[c] ..
 * colour_ptr[c + 1] index the rows of colour c in order.  Rows of one colour
 * do not read one another, so each colour runs in parallel and the result
 * equals lo_sor_sweep_ordered bit for bit. */
void lo_sor_sweep_coloured(const lo_csr *a, double relax, const double *x_in, double *x_out,
                           const double *b, int forward, int ultra, const int32_t *order,
                           const int32_t *colour, const int64_t *colour_ptr, int32_t ncolours);
/* 1 when no stored entry (i, j), i != j, has colour[i] == colour[j] */
int lo_colouring_is_proper(const lo_csr *a, const int32_t *colour);
/* lo_sor_sweep_ordered in float arithmetic on float-rounded values */
void lo_sor_sweep_ordered_f32(const lo_csr *a, float relax, const float *x_in, float *x_out,
                              const float *b, int forward, int ultra, const int32_t *order);

/* Jones-Plassmann colouring with priority hash(seed, i), ties by index.
 * Deterministic; returns the number of colours. */
int32_t lo_colour_jp(const lo_csr *a, uint64_t seed, int32_t *colour);
/* smallest-last greedy colouring (host restatement); returns the colours */
int32_t lo_colour_smallest_last(const lo_csr *a, int32_t *colour);
/* order = rows sorted by (colour, index) */
void lo_colour_order(int64_t n, const int32_t *colour, int32_t ncolours, int32_t *order);

/* ---- direct --------------------------------------------------------- */
/* cholesky/decomposition.hpp:52-107 (Cholesky-Banachiewicz), dense storage,
 * same operation order; l is n*n row-major lower.  Returns 0 on success. */
int lo_cholesky_factor(const lo_csr *a, double *l);
/* cholesky/solver.hpp:42-50, substitution.hpp:27-115 */
void lo_cholesky_solve(int64_t n, const double *l, const double *b, double *x);
/* lu/decomposition.hpp:31-122 (LU without pivoting), dense storage: L (unit
 * diagonal) below, U on and above the diagonal.  Returns 0 on success. */
int lo_lu_factor(const lo_csr *a, double *lu);
/* lu/solver.hpp:37-60 */
void lo_lu_solve(int64_t n, const double *lu, const double *b, double *x);

/* ---- AMG ------------------------------------------------------------ */
typedef struct {
  int32_t min_aggregate_size;     /* 6 */
  int32_t max_aggregate_size;     /* 9 */
  int64_t partition_size;         /* vertices per aggregation partition on level 0 */
  double partition_growth;        /* level l uses partition_size * growth^l */
  int64_t min_partitions;         /* 8: at least this many partitions while each keeps
                                     >= 1024 vertices */
  int64_t max_partitions;         /* upper clamp on the partition count */
  double strong_threshold;        /* 1/3 */
  double aggressive_threshold;    /* 1/3 */
  int64_t max_level_num;          /* 16 */
  int64_t min_coarsen_size;       /* 2000 (32 in the reference tests) */
  double min_coarsen_factor;      /* 1.2 */
  int coarse_f32;                 /* coarse matrices stored as float */
  double relax;                   /* MultiGridSolver relax (1.0) */
  double smoother_relax;          /* SOR relax (1.0) */
  int smoother_ultra;             /* SorVariant::ultra */
  int64_t smoother_parts;         /* >0: hybrid partitioned SOR with this many parts */
  uint64_t colour_seed;           /* used when smoother_parts == 0: colour-ordered SOR */
  int coarse_smallest_last;       /* with smoother_parts == 0: levels >= 1 coloured by
                                     lo_colour_smallest_last instead of Jones-Plassmann */
} lo_amg_params;

void lo_amg_default_params(lo_amg_params *p);
/* number of aggregation partitions for n vertices on `level`:
 * clamp(max(n / (partition_size * growth^level),
 *           min(min_partitions, n / 1024)), 1, max_partitions)
 * (independent.hpp:183-186 with partition_size in the role of min_per_thread
 * and max_partitions in the role of the thread count) */
int64_t lo_amg_partitions(int64_t n, int64_t level, const lo_amg_params *p);

/* dependency/criterion.hpp:35-78 with NegativeOffdiagonalTransform.
 * depends/influences are per CSR entry (diagonal entries left 0). */
void lo_amg_strength(const lo_csr *a, double theta, uint8_t *depends, uint8_t *influences,
                     uint8_t *isolated);
/* aggregation/base.hpp:532-677 + independent.hpp:123-208 +
 * aggregate-map/multithread.hpp:107-143.  agg[n] receives global aggregate
 * ids or LO_ISOLATED; list_ptr[ncoarse+1]/list[...] the coarse-to-fine lists.
 * list_ptr/list are malloc'ed.  stats[5] = aggregate_num, multi, single,
 * merged, isolated.  Returns the coarse size. */
int64_t lo_amg_aggregate(const lo_csr *a, const uint8_t *depends, const uint8_t *influences,
                         const uint8_t *isolated, int32_t min_size, int32_t max_size,
                         int64_t nparts, int aggressive, uint32_t *agg, int64_t **list_ptr,
                         int32_t **list, int64_t stats[5]);
/* transport/matrix-shared.hpp:85-183 + csr/shared.hpp:730-764 */
int lo_amg_galerkin(const lo_csr *a, int64_t ncoarse, const uint32_t *agg,
                    const int64_t *list_ptr, const int32_t *list, int coarse_f32, lo_csr *out);

typedef struct {
  lo_csr a;          /* level matrix (level 0 is a copy of the input) */
  uint32_t *agg;     /* fine -> coarse map (NULL on the coarsest level) */
  int64_t *list_ptr;
  int32_t *list;
  int32_t *order;    /* smoother row order (colour order) or NULL */
  int32_t *colour;   /* the colour of each row (with order) */
  int64_t *colour_ptr; /* rows of colour c: order[colour_ptr[c] .. colour_ptr[c+1]); NULL
                          when the colouring is not proper (sequential sweep) */
  int32_t ncolours;
  double *b, *x, *r; /* per-level work vectors */
} lo_amg_level;

typedef struct {
  int64_t nlevels;
  lo_amg_level lv[32];
  double *chol;      /* dense factor of the coarsest matrix: Cholesky lower
                        factor (symmetric), L and U of an LU (nonsymmetric) */
  lo_amg_params p;
} lo_amg;

/* hierarchy/wright.hpp:120-309 */
int lo_amg_setup(const lo_csr *a, const lo_amg_params *p, lo_amg *h);

/* An aggregate map of one level as BaseMultithreadAggregateMap holds it
 * (aggregate-map/multithread.hpp:42-45, 294-302): fine -> coarse ids (n;
 * LO_ISOLATED for isolated vertices) and the coarse -> fine lists
 * (list_ptr[ncoarse + 1], list[list_ptr[ncoarse]]). */
typedef struct {
  int64_t n, ncoarse;
  const uint32_t *agg;
  const int64_t *list_ptr;
  const int32_t *list;
} lo_agg_map;
enum { LO_ERR_NO_MAP = -2, LO_ERR_BAD_MAP = -3 };
/* 0 when the two maps agree: every id below ncoarse or LO_ISOLATED, every
 * aggregated vertex in exactly the list of its aggregate, no empty list;
 * LO_ERR_BAD_MAP otherwise */
int lo_agg_map_check(const lo_agg_map *m);
/* lo_amg_setup with the aggregation of level k replaced by maps[k]
 * (FileAggregator, aggregation/independent.hpp:279-298; the stop rules of
 * wright.hpp:120-143 unchanged).  Returns LO_ERR_NO_MAP when a level needs
 * a map beyond nmaps, LO_ERR_BAD_MAP when a map does not fit its level
 * (size or consistency), else as lo_amg_setup.  h is freeable on return. */
int lo_amg_setup_given(const lo_csr *a, const lo_amg_params *p, const lo_agg_map *maps,
                       int64_t nmaps, lo_amg *h);
/* lo_amg_setup with a given colouring of level 0 (colour[n], ncolours
 * classes) for the colour-ordered smoother (smoother_parts == 0) instead of
 * Jones-Plassmann, as a caller that hands the GPU hierarchy its finest
 * colouring does */
int lo_amg_setup_coloured(const lo_csr *a, const lo_amg_params *p, const int32_t *colour0,
                          int32_t ncolours0, lo_amg *h);
void lo_amg_free(lo_amg *h);
/* multigrid/solver.hpp:56-176, one REGULAR V-cycle from x_in = 0 */
void lo_amg_vcycle(lo_amg *h, const double *b, double *x);

/* ---- Krylov ----------------------------------------------------------- */
enum { LO_PRECON_NONE = 0, LO_PRECON_JACOBI = 1, LO_PRECON_SSOR = 2, LO_PRECON_AMG = 3 };
typedef struct {
  int kind;
  double relax;      /* Jacobi / SSOR relax */
  int ultra;
  int64_t nparts;    /* SSOR partitions */
  lo_amg *amg;
} lo_precon;

/* conjugate-gradients/solver.hpp:50-115.  Stops when ||r|| <= rtol * ||r0||
 * or after maxit iterations; rere_period > 0 recomputes the true residual
 * when iter > 0 && iter % rere_period == 0 (test/aux/iterative.hpp:97-99).
 * history (optional, maxit+1 entries) receives ||r|| per iteration.
 * Returns the iteration count. */
int64_t lo_pcg(const lo_csr *a, const double *b, double *x, const lo_precon *m, double rtol,
               int64_t maxit, int64_t rere_period, double *history);
/* bicgstab/solver.hpp:51-151 */
int64_t lo_pbicgstab(const lo_csr *a, const double *b, double *x, const lo_precon *m,
                     double rtol, int64_t maxit, int64_t rere_period, double *history);

#ifdef __cplusplus
}
#endif
#endif
