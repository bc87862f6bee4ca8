/*
 * lineal_gb300 C ABI: GB300 (sm_103a) implementation of lineal's solve path.
 *
 * lineal (KurtBoehm/lineal) is a header-only C++23 library whose operator
 * interface is a set of concepts (include/lineal/base/concept/range.hpp:17-40,
 * include/lineal/base/concept/solver.hpp:16-37).  This ABI is the device-side
 * boundary below the C++ wrappers in include/lineal_gb300/lineal.hpp, which
 * restate those concepts; every entry point names the reference interface it
 * replaces.
 *
 * Conventions
 *  - Every call returns lgx_status; lgx_last_error() holds a message for the
 *    calling thread.  No call throws and none traps on the device: breakdown
 *    and non-finite values are reported as statuses.
 *  - Pointers named d_* are device pointers; h_* are host pointers.  Vectors
 *    are plain arrays of double (or float where the name says f32).
 *  - Every call that launches work takes a cudaStream_t (0 = legacy default)
 *    and only enqueues on that stream, except where a host result is
 *    returned (documented per call).
 *  - Matrices are opaque handles owning device memory.  CSR input is
 *    row-major with sorted column indices per row and a stored diagonal
 *    (the invariants of include/lineal/tensor/dynamic/csr/shared.hpp:258-262).
 */
#ifndef LINEAL_GB300_H
#define LINEAL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *lgx_stream; /* == cudaStream_t */

typedef enum {
  LGX_OK = 0,
  LGX_ERR_INVALID = 1,     /* bad argument, size or handle */
  LGX_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  LGX_ERR_NOMEM = 3,       /* device allocation failed */
  LGX_ERR_BREAKDOWN = 4,   /* Krylov breakdown (zero denominator) */
  LGX_ERR_NONFINITE = 5,   /* NaN/Inf detected in a reduction */
  LGX_ERR_NOT_SPD = 6,     /* coarse Cholesky met a non-positive pivot */
  LGX_ERR_UNSUPPORTED = 7, /* operation not available for this matrix kind */
  LGX_ERR_NOT_CONVERGED = 8
} lgx_status;

const char *lgx_status_string(lgx_status s);
/* Message describing the last failure on the calling host thread. */
const char *lgx_last_error(void);
/* Library version string. */
const char *lgx_version(void);
/* Number of kernels this library has launched since it was loaded (every
 * launch site counts; used to report launches inside a timed region). */
uint64_t lgx_kernel_launches(void);

/* ------------------------------------------------------------------------
 * Matrices.  One handle type covers every matrix kind of the reference that
 * the solve path uses:
 *   LGX_MATRIX_CSR             CsrMatrix (tensor/dynamic/csr/shared.hpp:1114-1116)
 *   LGX_MATRIX_STENCIL_LOOKUP  AdjacentStencilMatrix<StationaryDiffusionLookupValuator>
 *   LGX_MATRIX_STENCIL_VALUE   AdjacentStencilMatrix<StationaryDiffusionValueValuator>
 *                              (tensor/dynamic/stencil/matrix/shared.hpp:34-358)
 * ---------------------------------------------------------------------- */
typedef struct lgx_matrix lgx_matrix;

typedef enum {
  LGX_MATRIX_CSR = 0,
  LGX_MATRIX_STENCIL_LOOKUP = 1,
  LGX_MATRIX_STENCIL_VALUE = 2
} lgx_matrix_kind;

typedef enum { LGX_F64 = 0, LGX_F32 = 1 } lgx_dtype;

/* Builds a CSR matrix from device arrays (copied).  values are stored in
 * `storage` precision (LGX_F32 rounds each value to float).  Replaces
 * CsrMatrix's RowWiseBuilder / MultithreadBuilder (csr/shared.hpp:424-903). */
lgx_status lgx_csr_create(int64_t n, int64_t nnz, const int64_t *d_rowptr, const int32_t *d_col,
                          const double *d_val, int symmetric, lgx_dtype storage, lgx_stream stream,
                          lgx_matrix **out);
/* Same from host arrays (uploaded with synchronous copies). */
lgx_status lgx_csr_create_host(int64_t n, int64_t nnz, const int64_t *h_rowptr,
                               const int32_t *h_col, const double *h_val, int symmetric,
                               lgx_dtype storage, lgx_matrix **out);
/* Copies the CSR arrays back to the host (sizes from lgx_matrix_info).
 * Synchronises `stream`. */
lgx_status lgx_csr_download(const lgx_matrix *a, int64_t *h_rowptr, int32_t *h_col,
                            double *h_val, lgx_stream stream);

/* Matrix-free 7-point diffusion stencil with Dirichlet values on both faces
 * of axis 0 and zero-flux elsewhere (valuator semantics of
 * stencil/valuator/stationary-diffusion-lookup.hpp:28-201 and
 * stationary-diffusion-value.hpp:31-204).  dims are cell counts (axis 2
 * fastest), q the axis quotients of BoxInfo (discretization/box-equidistant
 * .hpp:67-79).  Lookup: d_mat holds one material index (< 4) per cell and
 * coeffs the material conductivities.  Value: d_k holds one conductivity per
 * cell.  zero_to_one selects ZeroToOneTag (a zero diagonal becomes 1). */
/* BoxInfo (discretization/box-equidistant.hpp:57-110): an equidistant box of
 * cells[d] cells along axis d with axis lengths lengths[d].  The axis
 * quotients (67-79) are q_d = prod_{e != d} h_e / h_d with h = L / N, the
 * geometric factors the stencil valuators take as q.  Host-only; refuses
 * non-positive counts and non-positive or non-finite lengths. */
typedef struct {
  int64_t cells[3];
  double lengths[3];
} lgx_box_info;
lgx_status lgx_box_axis_quotients(const lgx_box_info *box, double q[3]);

lgx_status lgx_stencil_create_lookup(const int64_t dims[3], const double q[3],
                                     const double coeffs[4], const uint8_t *d_mat,
                                     double sol_start, double sol_end, int zero_to_one,
                                     lgx_stream stream, lgx_matrix **out);
/* The lookup valuator with HenryDiffusionLookupProvider (lookup-wright.hpp:
 * 38-60): the diffusion factor of materials a -> b is hm(c_a f_b, c_b f_a),
 * f = henry_constant for the materials flagged in gaseous_materials (bit m),
 * else 1; everything else as lgx_stencil_create_lookup. */
lgx_status lgx_stencil_create_lookup_henry(const int64_t dims[3], const double q[3],
                                           const double coeffs[4], uint8_t gaseous_materials,
                                           double henry_constant, const uint8_t *d_mat,
                                           double sol_start, double sol_end, int zero_to_one,
                                           lgx_stream stream, lgx_matrix **out);
lgx_status lgx_stencil_create_value(const int64_t dims[3], const double q[3], const double *d_k,
                                    double sol_start, double sol_end, int zero_to_one,
                                    lgx_stream stream, lgx_matrix **out);
/* StationaryDiffusionValuesValuator (stencil/valuator/stationary-diffusion-
 * values.hpp:30-211): a conductivity per cell and axis; the connection along
 * axis d is hm(k_d(from), k_d(to)) * q_d and the Dirichlet terms of axis 0
 * use k_0.  Same kernels and layout as the value valuator (matrix kind
 * LGX_MATRIX_STENCIL_VALUE); no effective diffusion (the reference valuator
 * has no diffusion coefficient). */
lgx_status lgx_stencil_create_values(const int64_t dims[3], const double q[3], const double *d_k0,
                                     const double *d_k1, const double *d_k2, double sol_start,
                                     double sol_end, int zero_to_one, lgx_stream stream,
                                     lgx_matrix **out);

lgx_status lgx_matrix_destroy(lgx_matrix *a);
/* kind, rows, stored non-zeros (stencils: the non-zeros of the assembled
 * matrix), symmetric flag (IsSymmetric, base/type-safe.hpp:11). */
lgx_status lgx_matrix_info(const lgx_matrix *a, int *kind, int64_t *n, int64_t *nnz,
                           int *symmetric);

/* y = A x (MatrixVectorProductExpr, component-wise/matrix-vector-product.hpp:
 * 34-140).  CSR rows accumulate fma(a_ij, x_j, sum) in ascending column order,
 * stencil rows in the scalar unordered order of stencil/matrix/algorithm.hpp
 * :178-225, so results equal the reference's scalar path bit for bit. */
lgx_status lgx_spmv(const lgx_matrix *a, const double *d_x, double *d_y, lgx_stream stream);
/* y = A x with float vectors (float-stored CSR; products accumulated in
 * float). */
lgx_status lgx_spmv_f32(const lgx_matrix *a, const float *d_x, float *d_y, lgx_stream stream);
/* r = b - A x, optionally d_norm2sq[0] = ||r||^2 (assign_expr +
 * euclidean_squared, conjugate-gradients/solver.hpp:59-61). */
lgx_status lgx_residual(const lgx_matrix *a, const double *d_b, const double *d_x, double *d_r,
                        double *d_norm2sq, lgx_stream stream);
/* diagonal of A (AdjacentStencilMatrix::diagonal_at, stencil/matrix/shared.hpp
 * :242-244; CsrMatrix row diagonal()). */
lgx_status lgx_diagonal(const lgx_matrix *a, double *d_diag, lgx_stream stream);
/* Right-hand side of a stencil system (AdjacentStencilVector,
 * stencil/vector/shared.hpp:181-205). */
lgx_status lgx_stencil_rhs(const lgx_matrix *a, double *d_b, lgx_stream stream);
/* Effective diffusivity of a solution (EffDiffCalc, component-wise/sink/
 * effective-diffusion.hpp:226-320): through the middle planes of axis 0,
 *   area_part = (filled cells of planes n0/2 and n0/2 + 1) / (n1 n2) / 2,
 *   eff = sum hm(c1, c2) (x(c2) - x(c1)) q0 / (area_part L1 L2) L0 / (u_end - u_start),
 * hm the harmonic mean of the two cells' coefficients; lengths = the axis
 * lengths L; none_materials flags "none" materials (bit m; lookup stencils;
 * every cell of a value stencil is filled); d_compress_map (may be NULL)
 * maps cells to the solution rows of a compressed system (-1: no row).
 * Synchronises `stream`; results on the host. */
lgx_status lgx_stencil_effective_diffusion(const lgx_matrix *a, const double lengths[3],
                                           uint8_t none_materials, const double *d_sol,
                                           const int64_t *d_compress_map, lgx_stream stream,
                                           double *h_eff, double *h_area_part);
/* Assembles a stencil matrix as CSR (csr_from_adjacent_stencil,
 * csr/create-from.hpp:37-246); zero off-diagonals are dropped.  With
 * zero_to_one == 0, rows with a zero diagonal are removed and d_compress_map
 * (cells entries, may be NULL) receives the compressed row or -1. */
lgx_status lgx_stencil_to_csr(const lgx_matrix *a, int64_t *d_compress_map, lgx_stream stream,
                              lgx_matrix **out);

/* Synthetic operators (no reference counterpart; the reference stencil is
 * 7-point).  d_k holds one conductivity per cell on a unit-spaced grid.
 * Off-diagonal to a neighbour at offset o: -hm(k_i, k_j) * w with w = 1
 * (face), 1/2 (edge), 1/4 (corner) and hm the harmonic mean of
 * math/harmonic-mean.hpp:13-25; the diagonal adds 2 k_i on both faces of
 * axis 0 and then the off-diagonal weights in ascending column order; a zero
 * diagonal becomes 1.  The 7-point variant keeps the faces only. */
lgx_status lgx_gen_27pt(const int64_t dims[3], const double *d_k, lgx_dtype storage,
                        lgx_stream stream, lgx_matrix **out);
lgx_status lgx_gen_7pt(const int64_t dims[3], const double *d_k, lgx_dtype storage,
                       lgx_stream stream, lgx_matrix **out);
/* Declares that a CSR matrix is a 27-point operator on an n0 x n1 x n2 grid
 * (row (i n1 + j) n2 + k couples the cell to its in-grid neighbours), as
 * lgx_gen_27pt's matrices are; an AMG hierarchy checks the structure on the
 * device before it relies on it.  No reference counterpart. */
lgx_status lgx_csr_set_grid27(lgx_matrix *a, const int64_t dims[3]);
/* The same for a 7-point operator (lgx_gen_7pt's matrices are declared). */
lgx_status lgx_csr_set_grid7(lgx_matrix *a, const int64_t dims[3]);

/* Configuration of the CSR row kernels (SpMV, residual, Jacobi, SOR) used by
 * later launches, process-wide; no reference counterpart (tuning):
 * 0-2 CTA tiles (two stages / one CTA per SM, one stage / two CTAs, two small
 * stages / two CTAs), 3-7 warp tiles (4 warps x 1 stage, 4 x 2, 8 x 1, 8 x 2
 * per CTA; 7: 4 x 1 with registers capped for seven CTAs per SM).  Every
 * configuration gives bit-identical results.  Default 3, or the environment
 * variable LGX_ROWS_CONFIG. */
lgx_status lgx_row_engine_set(int config);
int lgx_row_engine_get(void);

/* Kernel of the matrix-free stencil products (lgx_spmv, lgx_residual on
 * stencil matrices), process-wide; no reference counterpart: 0 thread per
 * cell (default), 1 plane march with the x planes of each 8 x 64 tile staged
 * through TMA (cp.async.bulk.tensor.3d, halo on both plane axes) into a
 * four-plane ring in shared memory (used when the axis-2 length is even and
 * x is 16-byte aligned; otherwise the thread-per-cell kernel runs).  Both
 * give bit-identical results.  Default 0, or 1 with LGX_STENCIL_PLANES=1. */
lgx_status lgx_stencil_engine_set(int engine);
int lgx_stencil_engine_get(void);

/* Autotuner of the row-engine configuration per matrix; no reference
 * counterpart (the reference's loops have a compile-time shape).  For each
 * (matrix, operation class, value type) it times all LGX_TUNE_CONFIGS
 * configurations with CUDA events on `stream` (two untimed launches, then
 * `reps` timed ones, reps in [1, 1000]) and keeps the fastest on that matrix;
 * later launches on the matrix use it instead of the process-wide
 * configuration.  Products and sweeps stay bit-identical; only the grouping
 * of norm reductions follows the grid.  Vectors are scratch (allocated and
 * freed by the call); matrix values are not touched.  Synchronises `stream`.
 * Tune before the first solve of a Krylov solver that captures CUDA graphs:
 * a captured iteration keeps the shapes it was recorded with. */
#define LGX_TUNE_CONFIGS 8
typedef struct lgx_tune_entry {
  int32_t level;       /* hierarchy level (0 for a single matrix) */
  int32_t op;          /* 0 products (SpMV, residual), 1 SOR sweeps */
  int32_t value_bytes; /* stored values read: 8 FP64, 4 FP32, 2 BF16 */
  int32_t config;      /* configuration kept (-1: nothing to tune) */
  int32_t fastest;     /* configuration with the least time in ms[] */
  float ms[LGX_TUNE_CONFIGS]; /* mean milliseconds of one operation per configuration */
} lgx_tune_entry;
/* y = A x with FP64 vectors on a CSR matrix (lgx_spmv's product): one
 * entry into *out (NULL skips the report). */
lgx_status lgx_matrix_autotune(lgx_matrix *a, int reps, lgx_tune_entry *out, lgx_stream stream);

/* ------------------------------------------------------------------------
 * Vector reductions and updates (component-wise/sink/accumulator.hpp:151-218,
 * vector-expression.hpp:67-92).  Reductions are deterministic: fixed block
 * partition, fixed-order second stage.  Results land in device memory; the
 * reductions synchronise `stream`.  Their partial sums are allocated once per
 * stream (9.7 KB, kept for the process), so repeated calls do not allocate.
 * ---------------------------------------------------------------------- */
lgx_status lgx_dot(int64_t n, const double *d_a, const double *d_b, double *d_out,
                   lgx_stream stream);
lgx_status lgx_norm2sq(int64_t n, const double *d_a, double *d_out, lgx_stream stream);

/* lgx_dot without any device allocation.  No reference counterpart: lineal's
 * dot (sink/accumulator.hpp:151-157) is a CPU reduction with no scratch.
 *
 * lgx_dot allocates its partial sums with cudaMalloc on the first call on
 * each stream (and keeps them).  Callers that must not allocate at all (code
 * whose device memory is all handed to its own pool, or that may run on a
 * fresh stream inside a region where an allocation would stall or fail) call
 * this instead: the partial sums live in a fixed static device array of the
 * library.
 *
 * - Result: the same as lgx_dot (same grid, same summation order), written to
 *   d_out in stream order; the call does not synchronise.
 * - Maximum size: n <= 2,097,152 elements (1024 partial sums of 2048
 *   elements); a larger n returns LGX_ERR_INVALID with a message.
 * - Set-up: the first call on each device looks up the scratch address
 *   (cudaGetSymbolAddress) with that device current; make that first call
 *   before any stream capture.
 * - The scratch is shared: two calls that overlap in time on one device (two
 *   streams, or two host threads) race on it and give wrong results.  Calls on
 *   one stream are ordered and safe.
 * - The scratch's arrival counter must be zero when a call starts; it is zero
 *   when the library loads and every completed call leaves it at zero.
 * - cudaDeviceReset ends the context whose scratch address the first call
 *   looked up; calls after a reset of that device are not supported. */
lgx_status lgx_dot_static(int64_t n, const double *d_a, const double *d_b, double *d_out,
                          lgx_stream stream);
lgx_status lgx_max_norm(int64_t n, const double *d_a, double *d_out, lgx_stream stream);
/* y = y + alpha * x */
lgx_status lgx_axpy(int64_t n, double alpha, const double *d_x, double *d_y, lgx_stream stream);
/* out = alpha x + beta y, each product and the sum rounded separately, so
 * that add(x, y) (alpha = beta = 1), subtract(x, y) (beta = -1),
 * scale(x, alpha) (d_y = NULL) and add/subtract of scaled vectors give the
 * bits of lineal's expression evaluation (component-wise/
 * vector-expression.hpp:67-91, 150-167).  out may be x or y. */
lgx_status lgx_lincomb(int64_t n, double alpha, const double *d_x, double beta,
                       const double *d_y, double *d_out, lgx_stream stream);
/* out = value everywhere (constant / constant_like, vector-expression.hpp:
 * 140-147, assigned) */
lgx_status lgx_fill(int64_t n, double value, double *d_out, lgx_stream stream);

/* ------------------------------------------------------------------------
 * Smoothers (linear-solver/iterative-stationary/).
 * ---------------------------------------------------------------------- */
/* One Jacobi sweep (jacobi/sweep.hpp:66-87); d_x_in == NULL means zero. */
lgx_status lgx_jacobi_sweep(const lgx_matrix *a, double relax, const double *d_x_in,
                            double *d_x_out, const double *d_b, lgx_stream stream);

/* A colouring of the matrix graph.  The GPU replaces the reference's
 * thread-block-hybrid SOR (gauss-seidel-variant/sweep.hpp:134-200) by a
 * multicolour sweep: colours are visited in ascending order (forward) or
 * descending order (backward); a row reads the values of already visited
 * colours from the output and all others from the input.  The result equals
 * the reference SOR applied in the order "rows sorted by (colour, index)". */
typedef struct lgx_colouring lgx_colouring;
/* Jones-Plassmann colouring with splitmix64 priorities (deterministic). */
lgx_status lgx_colouring_create_jp(const lgx_matrix *a, uint64_t seed, lgx_stream stream,
                                   lgx_colouring **out);
/* Smallest-last greedy colouring of a CSR pattern in host memory (rows as
 * adjacency lists, the diagonal ignored; a symmetric pattern gives a proper
 * colouring): host code only, deterministic, O(nnz).  On coarse AMG levels
 * it needs fewer colours than Jones-Plassmann (64^3 27-point hierarchy,
 * levels 1-2: 11 and 12 against 14 and 16).  colour[n] receives the
 * colours, *ncolours their number; pass the colours (copied to the device)
 * to lgx_colouring_create. */
lgx_status lgx_colour_smallest_last(int64_t n, const int64_t *rowptr, const int32_t *col,
                                    int32_t *colour, int32_t *ncolours);
/* Failure-detection self-test (no reference counterpart): launches a kernel
 * whose bounded wait on a shared-memory barrier can never complete (nothing
 * arrives), so the wait gives up after about one second of SM clock, records
 * the time-out in the device error flag and returns; the call then reports
 * it as LGX_ERR_CUDA ("a device wait ... timed out") and clears the flag,
 * the same path by which the staged kernels report a copy that never lands.
 * The context stays usable.  Synchronises `stream`. */
lgx_status lgx_wait_selftest(lgx_stream stream);

/* Red-black colouring of a stencil matrix, colour (p0 + p1 + p2) & 1: the
 * 7-point stencil's natural two-colouring.  lgx_sor_sweep then runs
 * matrix-free in natural order, one launch per colour, and equals lineal's
 * SOR of the assembled matrix in the row order sorted by (colour, index);
 * SSOR preconditioning of a stencil uses it too.  The permuted-order entry
 * points refuse it. */
lgx_status lgx_colouring_create_red_black(const lgx_matrix *a, lgx_stream stream,
                                          lgx_colouring **out);
/* User colouring (device array, one colour in [0, ncolours) per row; e.g.
 * the parity colouring of a structured grid).  Validated on the device. */
lgx_status lgx_colouring_create(const lgx_matrix *a, const int32_t *d_colour, int32_t ncolours,
                                lgx_stream stream, lgx_colouring **out);
/* Gives a parity colouring of a 27-point grid matrix (see
 * lgx_amg_params.grid27) the grid kernels for its sweeps through
 * lgx_sor_sweep_permuted[_f32]; with_float also prepares the float copy of
 * the values that lgx_sor_sweep_permuted_f32 reads.  The structure is
 * checked on the device: *attached (may be NULL) is 0 when it does not hold
 * and the CSR kernels stay.  Results are bit-identical either way.  No
 * reference counterpart. */
lgx_status lgx_colouring_grid27(lgx_colouring *c, const int64_t dims[3], int with_float,
                                lgx_stream stream, int *attached);
lgx_status lgx_colouring_destroy(lgx_colouring *c);
/* Copies the colour of every row to d_colour; *ncolours receives the count.
 * Synchronises `stream`. */
lgx_status lgx_colouring_export(const lgx_colouring *c, int32_t *d_colour, int32_t *ncolours,
                                lgx_stream stream);

/* One multicolour SOR sweep (SorSolver/SorBroom, gauss-seidel-variant/
 * solver.hpp:22-41, regular or ultra variant).  d_x_in == NULL means zero;
 * d_x_in may equal d_x_out (in situ). */
lgx_status lgx_sor_sweep(const lgx_matrix *a, const lgx_colouring *c, double relax, int forward,
                         int ultra, const double *d_x_in, double *d_x_out, const double *d_b,
                         lgx_stream stream);

/* Sweeps in the colouring's own row order: row r of the permuted space is
 * row perm[r] of the matrix, colours occupy contiguous ranges, and the sweep
 * updates d_x in place (the in-situ apply of broom.hpp:27-124) without the
 * gathers and scatters of lgx_sor_sweep.  lgx_colouring_permute /
 * lgx_colouring_unpermute move vectors between the natural and the permuted
 * order (dst[r] = src[perm[r]] and dst[perm[r]] = src[r]).  The _f32 sweep
 * computes in float with float values (the matrix's float storage, or a float
 * copy of its values made by the first call) -- the smoother of the
 * precision form. */
lgx_status lgx_colouring_permute(const lgx_colouring *c, const double *d_src, double *d_dst,
                                 lgx_stream stream);
lgx_status lgx_colouring_unpermute(const lgx_colouring *c, const double *d_src, double *d_dst,
                                   lgx_stream stream);
lgx_status lgx_sor_sweep_permuted(const lgx_colouring *c, double relax, int forward, int ultra,
                                  double *d_x, const double *d_b, lgx_stream stream);
lgx_status lgx_sor_sweep_permuted_f32(lgx_colouring *c, float relax, int forward, int ultra,
                                      float *d_x, const float *d_b, lgx_stream stream);

/* ------------------------------------------------------------------------
 * Aggregation AMG (linear-solver/multigrid/).
 * ---------------------------------------------------------------------- */
typedef struct {
  int32_t min_aggregate_size;  /* AggregationParams (aggregation/params.hpp:13-20) */
  int32_t max_aggregate_size;
  int64_t partition_size;      /* vertices per aggregation partition on the finest level */
  double partition_growth;     /* level l uses partition_size * growth^l: coarse levels
                                  keep partitions that span several fine planes */
  int64_t min_partitions;      /* but at least this many partitions (default 8) while each keeps
                                  1024 vertices (parallelism on coarse levels) */
  int64_t max_partitions;      /* clamp on the partition count */
  double strong_threshold;     /* DuneDependencyCriterion (dependency/criterion.hpp:103-118) */
  double aggressive_threshold;
  int64_t max_level_num;       /* HierarchyWrightParams (hierarchy/wright.hpp:46-55) */
  int64_t min_coarsen_size;
  double min_coarsen_factor;
  int coarse_f32;              /* coarse matrices stored as float, cycle arithmetic in
                                  double (the reference tests' CsrMatrix<f32> levels) */
  int cycle_f32;               /* precision form: every level stored as float and the
                                  whole cycle (smoothers, residuals, transfers) computed
                                  in float; the coarsest solve stays FP64 */
  double relax;                /* MultiGridSolver relax: correction scaled by 1/relax */
  double smoother_relax;       /* SOR relax */
  int smoother_ultra;          /* SorVariant::ultra */
  uint64_t colour_seed;        /* JP colouring seed of the coarse levels */
  int cycle_bf16;              /* with cycle_f32: smoothers and residuals read bfloat16
                                  values a_ij / a_ii with the diagonal a_ii as a per-row
                                  float scale (2 bytes per entry instead of 4) */
  int grid27;                  /* 1 (default): when the finest matrix is a 27-point
                                  operator on an even grid with the parity colouring, or a
                                  7-point operator (even n2) with the red-black colouring
                                  (lgx_gen_27pt / lgx_gen_7pt, or declared by
                                  lgx_csr_set_grid27 / lgx_csr_set_grid7), its products
                                  and sweeps compute the column indices from the grid
                                  instead of reading them (bit-identical results); 0:
                                  always the CSR kernels */
  int coarse_smallest_last;    /* 0 (default): Jones-Plassmann colourings on every
                                  level; 1: levels >= 1 coloured on the host by
                                  lgx_colour_smallest_last (fewer colours, so fewer
                                  sweep launches) */
} lgx_amg_params;

void lgx_amg_default_params(lgx_amg_params *p);

typedef struct lgx_amg lgx_amg;
/* HierarchyWrightInstance::create (hierarchy/wright.hpp:146-309): strength
 * (DuneDependencyCriterion), greedy aggregation per partition
 * (IndependentAggregationSink + BaseAggregator), Galerkin coarse matrices
 * (coarsen_matrix), multicolour SOR smoothers and a dense FP64 coarsest
 * solver.  finest_colouring may be NULL (JP colouring is computed).  The
 * finest matrix must stay alive while the hierarchy is used.  Synchronises
 * `stream` (level sizes decide the loop). */
lgx_status lgx_amg_setup(const lgx_matrix *a, const lgx_amg_params *p,
                         const lgx_colouring *finest_colouring, lgx_stream stream,
                         lgx_amg **out);
/* One level's aggregates in host memory, the two halves of
 * BaseMultithreadAggregateMap (aggregate-map/multithread.hpp:42-45,
 * 299-303): agg[n] fine->coarse ids (0xFFFFFFFE for an isolated vertex) and
 * the coarse->fine lists list_ptr[ncoarse + 1] / list[list_ptr[ncoarse]]. */
typedef struct lgx_agg_map {
  int64_t n;
  int64_t ncoarse;
  const uint32_t *agg;
  const int64_t *list_ptr;
  const int32_t *list;
} lgx_agg_map;
/* lgx_amg_setup with the strength and aggregation of level k replaced by
 * maps[k] (FileAggregator, aggregation/independent.hpp:279-298; the stop
 * rules of hierarchy/wright.hpp:120-143 unchanged).  Every map is checked on
 * the host before it is copied: fine size equal to the level's rows, ids
 * below ncoarse or isolated, every aggregated vertex in exactly the list of
 * its aggregate, no empty aggregate; LGX_ERR_INVALID otherwise, or when a
 * level needs a map beyond nmaps. */
/* The checks lgx_amg_setup_given applies to a map for a level of n rows,
 * on the host alone (no device work): LGX_OK or LGX_ERR_INVALID with the
 * reason in lgx_last_error. */
lgx_status lgx_agg_map_check(const lgx_agg_map *m, int64_t n);
lgx_status lgx_amg_setup_given(const lgx_matrix *a, const lgx_amg_params *p,
                               const lgx_colouring *finest_colouring, const lgx_agg_map *maps,
                               int64_t nmaps, lgx_stream stream, lgx_amg **out);
lgx_status lgx_amg_destroy(lgx_amg *h);
/* Number of levels, and per level (up to max_levels entries) rows and
 * stored non-zeros. */
lgx_status lgx_amg_info(const lgx_amg *h, int64_t *nlevels, int64_t *rows, int64_t *nnz,
                        int64_t max_levels);
/* Level matrix (natural ordering) and fine->coarse aggregate map of `level`
 * to host arrays (NULL pointers skip an array).  Synchronises `stream`. */
lgx_status lgx_amg_level_download(const lgx_amg *h, int64_t level, int64_t *h_rowptr,
                                  int32_t *h_col, double *h_val, uint32_t *h_agg,
                                  lgx_stream stream);
/* What lineal's hierarchy setup logs (hierarchy/wright.hpp:26-31, 120-143,
 * 210-225; aggregation/stats.hpp:16-32), per level in level order: the
 * dimensions, the stored non-zeros, the aggregation statistics of the level
 * (zero on the coarsest level and for levels built from given maps), and
 * whether the level was aggregated with the aggressive threshold; plus why
 * coarsening stopped.  Host data only. */
typedef struct lgx_amg_level_log {
  int64_t rows, columns, nnz;
  int64_t aggregate_num, multi_vertex_aggregate_num, single_vertex_aggregate_num,
    merged_aggregate_num, isolated_aggregate_num;
  int32_t aggressive;
  int32_t given_map;
} lgx_amg_level_log;
enum {
  LGX_STOP_TOO_SMALL = 1,       /* coarse size below min_coarsen_size */
  LGX_STOP_TOO_MANY_LEVELS = 2, /* max_level_num reached */
  LGX_STOP_TOO_SMALL_RATE = 3,  /* coarsening factor too small while aggressive */
  LGX_STOP_LEVEL_CAP = 4        /* this library's 32-level storage limit */
};
lgx_status lgx_amg_setup_log(const lgx_amg *h, lgx_amg_level_log *levels, int64_t max_levels,
                             int64_t *nlevels, int32_t *stop_reason);
/* Coarse->fine lists of `level`'s aggregates (BaseMultithreadAggregateMap::
 * coarse_row_to_fine_rows, aggregate-map/multithread.hpp:337-344; with the
 * fine->coarse map of lgx_amg_level_download, what to_file writes, 346-349):
 * h_list_ptr[ncoarse + 1] offsets and h_list[*list_len] fine vertices (natural
 * ordering, in the order aggregation added them).  NULL pointers skip an
 * output; *list_len = h_list_ptr[ncoarse] = the number of aggregated (not
 * isolated) vertices.  The coarsest level has no lists.  Synchronises
 * `stream`. */
lgx_status lgx_amg_level_lists(const lgx_amg *h, int64_t level, int64_t *h_list_ptr,
                               int32_t *h_list, int64_t *list_len, lgx_stream stream);
/* ---- Direct solver ------------------------------------------------------ */
/* CholeskySolver (direct/cholesky/solver.hpp:22-67, kind
 * LGX_DIRECT_CHOLESKY) or LuSolver (direct/lu/solver.hpp:21-66, kind
 * LGX_DIRECT_LU) as the dense FP64 solve the AMG uses on its coarsest level:
 * lgx_direct_create forms the inverse once -- Cholesky: the dense Cholesky
 * factor (every pivot positive, else LGX_ERR_NOT_SPD) and the inverse from
 * it; LU: Gauss-Jordan elimination without pivoting (every pivot nonzero,
 * finite and not tiny against its row, else LGX_ERR_BREAKDOWN — lineal's LU
 * does not pivot either) -- and synchronises `stream`; lgx_direct_solve
 * computes x = A^-1 b with one dense product (b and x distinct device
 * vectors of n doubles).  Dense storage: n <= LGX_DIRECT_MAX_ROWS.  Beyond
 * that, Cholesky factors in a band (lineal's factor, cholesky/decomposition
 * .hpp:52-107, fills the lower envelope of the natural order: the band of
 * width max_i (i - first column of row i)), at most 2^31 band values, and
 * each solve is a forward and a backward substitution; LU refuses. */
#define LGX_DIRECT_MAX_ROWS 8192
enum { LGX_DIRECT_CHOLESKY = 0, LGX_DIRECT_LU = 1 };
typedef struct lgx_direct lgx_direct;
lgx_status lgx_direct_create(const lgx_matrix *a, int kind, lgx_stream stream,
                             lgx_direct **out);
lgx_status lgx_direct_solve(const lgx_direct *d, const double *d_b, double *d_x,
                            lgx_stream stream);
lgx_status lgx_direct_destroy(lgx_direct *d);

/* One V-cycle from a zero initial guess: x = M^-1 b (MultiGridSolver::
 * Instance::apply, multigrid/solver.hpp:41-176, REGULAR cycle, 1 iteration). */
lgx_status lgx_amg_vcycle(lgx_amg *h, const double *d_b, double *d_x, lgx_stream stream);
/* Autotunes (see lgx_matrix_autotune) every smoothed level of a hierarchy:
 * its residual and its forward SOR sweep in the value and vector types its
 * cycles read, and with cycle_f32 also the finest level's FP64 product (the
 * outer Krylov SpMV).  A level keeps its fastest shapes only if a whole
 * V-cycle (graph replays, timed) is also faster with them than with the
 * process-wide configuration there; otherwise `config` reports the
 * process-wide one.  Writes up to max_out entries to *out and the number
 * of entries to *n_out (either may be NULL). */
lgx_status lgx_amg_autotune(lgx_amg *h, int reps, lgx_tune_entry *out, int max_out, int *n_out,
                            lgx_stream stream);
/* Drops the tuned choices: launches use the process-wide configuration. */
lgx_status lgx_amg_autotune_reset(lgx_amg *h);
/* 1 when the finest level runs the 27-point grid kernels (see
 * lgx_amg_params.grid27), else 0. */
int lgx_amg_grid27(const lgx_amg *h);

/* The individual setup steps, for parity checks.
 * Strength of connection (dependency/criterion.hpp:35-78): per stored entry
 * depends/influences bytes, per row the isolated byte. */
lgx_status lgx_amg_strength(const lgx_matrix *a, double theta, uint8_t *d_depends,
                            uint8_t *d_influences, uint8_t *d_isolated, lgx_stream stream);
/* Greedy aggregation in nparts contiguous partitions (aggregation/base.hpp:
 * 532-677, independent.hpp:47-216) followed by the aggregate-map merge
 * (aggregate-map/multithread.hpp:107-143).  d_agg receives global aggregate
 * ids, 0xFFFFFFFE for isolated vertices.  *ncoarse is written to host memory
 * (synchronises `stream`). */
lgx_status lgx_amg_aggregate(const lgx_matrix *a, const uint8_t *d_depends,
                             const uint8_t *d_influences, const uint8_t *d_isolated,
                             int32_t min_size, int32_t max_size, int64_t nparts, int aggressive,
                             uint32_t *d_agg, int64_t *ncoarse, lgx_stream stream);

/* ------------------------------------------------------------------------
 * Krylov solvers (linear-solver/conjugate-gradients/solver.hpp:24-225,
 * linear-solver/bicgstab/solver.hpp:25-263) driven as in run_iterative_solver
 * (linear-solver/runner.hpp:17-84): iterate until ||r|| <= rtol * ||r0|| or
 * maxit iterations.  The true residual is recomputed when iteration > 0 and
 * iteration % rere_period == 0 (the rere_controller of
 * test/aux/iterative.hpp:97-99).  Scalars stay on the device; the host
 * reads ||r||^2 once per iteration to decide termination.
 * ---------------------------------------------------------------------- */
typedef enum {
  LGX_PRECON_NONE = 0,
  LGX_PRECON_JACOBI = 1, /* one Jacobi sweep from zero */
  LGX_PRECON_SSOR = 2,   /* one multicolour SSOR sweep pair from zero */
  LGX_PRECON_AMG = 3     /* one V-cycle */
} lgx_precon_kind;

typedef struct {
  int precon;                   /* lgx_precon_kind */
  double relax;                 /* Jacobi / SSOR relax */
  int ultra;                    /* SSOR variant */
  const lgx_colouring *colouring; /* SSOR colouring (NULL: computed) */
  lgx_amg *amg;                 /* LGX_PRECON_AMG */
  double rtol;
  int64_t maxit;
  int64_t rere_period;          /* 0 disables true-residual recomputation */
  int use_graphs;               /* capture each iteration (SpMV, reductions, updates and
                                   the whole V-cycle) in a CUDA graph and replay it */
  int flexible;                 /* CG: flexible CG, beta = r+.(z+ - z) / r.z (Notay 2000),
                                   for preconditioners that are not exactly linear (the
                                   float V-cycle of the precision form); no counterpart
                                   in the reference's CG (solver.hpp:105-107) */
  int refine;                   /* lgx_pcg with an AMG hierarchy built with cycle_f32
                                   (precision form; no reference counterpart): CG on
                                   float vectors -- float finest-level products and
                                   float V-cycle, dot products accumulated and CG
                                   scalars kept in FP64 -- under an FP64 solution and
                                   FP64 residual; the solve stops on the FP64 residual.
                                   1: iterative refinement, each outer step solves
                                   A d = r / ||r|| from scratch to inner_rtol and adds
                                   ||r|| d to x.  2: reliable updates, one unbroken
                                   float recurrence whose accumulated update is folded
                                   into x, and r replaced by the FP64 residual, each
                                   time the recursive residual has fallen by inner_rtol
                                   (with flexible = 1 its beta is the flexible one).
                                   *iterations counts the float iterations (one product
                                   and one V-cycle each); h_history holds the float
                                   residual estimates and, at each FP64 residual, that
                                   residual */
  double inner_rtol;            /* refine 1: inner relative tolerance (1e-4); refine 2:
                                   reduction between FP64 residuals (1e-4) */
} lgx_solve_params;

void lgx_solve_default_params(lgx_solve_params *p);

/* Solve A x = b; x holds the initial guess on entry.  *iterations and
 * *final_rel_residual are host outputs; h_history (optional, maxit + 1
 * entries) receives ||r|| after each iteration.  Synchronises `stream`. */
lgx_status lgx_pcg(const lgx_matrix *a, const double *d_b, double *d_x,
                   const lgx_solve_params *p, lgx_stream stream, int64_t *iterations,
                   double *final_rel_residual, double *h_history);
lgx_status lgx_pbicgstab(const lgx_matrix *a, const double *d_b, double *d_x,
                         const lgx_solve_params *p, lgx_stream stream, int64_t *iterations,
                         double *final_rel_residual, double *h_history);

/* Blocked multi-right-hand-side AMG-PCG (batching form; no reference
 * counterpart): nrhs <= 32 systems A X = B with the same matrix and hierarchy,
 * d_b / d_x row-major n x nrhs blocks (entry (i, k) at i * nrhs + k), d_x the
 * initial guesses on entry.  Every pass over a matrix serves all columns;
 * each column runs its own CG recurrence (FP64 outer iteration and dots, the
 * hierarchy's V-cycle as preconditioner -- float for cycle_f32 hierarchies --
 * with the FP64 dense coarsest solve) and is frozen once
 * ||r_k|| <= rtol ||r0_k||.  The hierarchy must have been built from `a`.
 * The CG scalars of all columns stay on the device; with use_graphs != 0 the
 * second iteration is recorded as a CUDA graph (one per residual-recompute
 * variant: V-cycle, products, dots, scalars and updates) and replayed, the
 * host reading one small state block per iteration for the stopping test.
 * Both modes give bit-identical results.
 * Host outputs per column (optional): iterations and final relative residual.
 * Synchronises `stream`. */
lgx_status lgx_pcg_multi(const lgx_matrix *a, lgx_amg *amg, int32_t nrhs, const double *d_b,
                         double *d_x, double rtol, int64_t maxit, int use_graphs,
                         lgx_stream stream, int64_t *h_iterations, double *h_rel_residual);

/* Step-wise form of the same solvers: lgx_krylov_create performs the
 * SystemInstance construction (initial residual, first preconditioner
 * application), lgx_krylov_iterate one SystemInstance::iterate, and
 * lgx_krylov_state returns the iteration count, residual_norm() and rho()
 * (synchronised host copies).  lgx_krylov_solution writes the current
 * iterate to d_x (natural ordering).  b and the initial guess are copied at
 * creation, so d_b and d_x need not stay valid afterwards. */
typedef struct lgx_krylov lgx_krylov;
typedef enum { LGX_KRYLOV_CG = 0, LGX_KRYLOV_BICGSTAB = 1 } lgx_krylov_kind;
lgx_status lgx_krylov_create(int kind, const lgx_matrix *a, const double *d_b,
                             const double *d_x, const lgx_solve_params *p, lgx_stream stream,
                             lgx_krylov **out);
lgx_status lgx_krylov_iterate(lgx_krylov *k);
lgx_status lgx_krylov_state(const lgx_krylov *k, int64_t *iteration, double *residual_norm,
                            double *rho);
lgx_status lgx_krylov_solution(lgx_krylov *k, double *d_x);
lgx_status lgx_krylov_destroy(lgx_krylov *k);

/* ------------------------------------------------------------------------
 * Batching form: independent first-order upwind convection-diffusion
 * systems (D = 1, unit spacing, constant velocity v per system, zero
 * Dirichlet values outside the grid; the assembled row of cell i holds
 * -(1 + max(+-v_d, 0)) toward each neighbour and the sum of the six
 * magnitudes on the diagonal) solved by Jacobi-preconditioned BiCGStab
 * (bicgstab/solver.hpp:73-151, Jacobi from zero with `relax`) in one
 * persistent launch: each CTA solves whole systems taken from a work queue,
 * largest first, with the termination rule of run_iterative_solver
 * (runner.hpp:17-84) evaluated on the device.  No reference counterpart for
 * the batching itself.
 * ---------------------------------------------------------------------- */
typedef struct {
  int64_t dims[3];
  double v[3];
} lgx_convdiff_system;
/* d_b / d_x: the systems' vectors concatenated in list order (row-major
 * grids, last axis contiguous); d_x holds the initial guesses and receives the
 * solutions.  Host outputs per system (optional): iterations, final
 * ||r|| / ||r0||, status (0 converged, 1 breakdown, 2 non-finite, 3 maxit).
 * Returns LGX_ERR_BREAKDOWN / LGX_ERR_NONFINITE if any system hit one.
 * Synchronises `stream`. */
lgx_status lgx_batch_convdiff_bicgstab(int32_t nsys, const lgx_convdiff_system *h_systems,
                                       const double *d_b, double *d_x, double rtol, int64_t maxit,
                                       int64_t rere_period, double relax, lgx_stream stream,
                                       int64_t *h_iterations, double *h_rel_residual,
                                       int32_t *h_status);

/* ------------------------------------------------------------------------
 * Differentiation form: for x = A(theta)^-1 b and a loss L(x) the adjoint
 * lambda = A^-T dL/dx is one more Krylov solve (lgx_pcg when A is symmetric,
 * lgx_pbicgstab on the transpose otherwise) and dL/dtheta = -lambda^T
 * (dA/dtheta) x.  No reference counterpart (lineal has no derivatives).
 * ---------------------------------------------------------------------- */
/* d_out[e] = alpha * d_u[row(e)] * d_v[col(e)] for every stored entry e of
 * the CSR matrix a, in storage order: the outer product u v^T sampled on the
 * sparsity pattern (alpha = -1, u = lambda, v = x gives dL/dA on the
 * pattern).  d_out holds nnz doubles. */
lgx_status lgx_sampled_outer(const lgx_matrix *a, double alpha, const double *d_u,
                             const double *d_v, double *d_out, lgx_stream stream);
/* r = b - A x with each row summed by the compensated dot product Dot2
 * (Ogita, Rump, Oishi 2005): as accurate as twice-FP64 arithmetic rounded
 * once.  The residual of iterative refinement to full FP64 accuracy (FP64
 * CSR matrices only). */
lgx_status lgx_residual_compensated(const lgx_matrix *a, const double *d_b, const double *d_x,
                                   double *d_r, lgx_stream stream);
/* dL/dtheta for the 7-point operator of lgx_gen_7pt with k = exp(theta) per
 * cell (harmonic-mean faces, 2 k on axis-0 boundary faces), given
 * k, lambda and x: one deterministic pass, one thread per cell. */
lgx_status lgx_diffusion7_grad(const int64_t dims[3], const double *d_k, const double *d_lambda,
                               const double *d_x, double *d_grad, lgx_stream stream);

#ifdef __cplusplus
}
#endif
#endif
