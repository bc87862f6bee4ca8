// Krylov drivers: preconditioned CG (conjugate-gradients/solver.hpp:24-225)
// and BiCGStab (bicgstab/solver.hpp:25-263), run as run_iterative_solver does
// (runner.hpp:17-84).  Solver scalars (rho, alpha, beta, omega, ||r||^2) live
// in device memory and are produced by the last block of each deterministic
// reduction, so no scalar makes a host round trip; the host reads ||r||^2 once
// per iteration to decide termination.
//
// With an SSOR or AMG preconditioner on a CSR matrix the whole iteration runs
// in the colour-permuted ordering of the finest level (the smoother's native
// layout); b and x are permuted on entry and exit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "lgx_internal.cuh"

namespace lgx {
lgx_status amg_apply_permuted(lgx_amg &h, const double *b, double *x, cudaStream_t s);
const Csr &amg_finest_permuted(const lgx_amg &h);
lgx_colouring *amg_finest_colouring(lgx_amg &h);
bool amg_cycle_f32(const lgx_amg &h);
lgx_status amg_apply_permuted_f32(lgx_amg &h, const float *b, float *x, cudaStream_t s);
const float *amg_finest_values_f32(const lgx_amg &h);
}  // namespace lgx

namespace lgx {

struct KScalars {
  double rho, rho_old, alpha, beta, omega, res2, den, tmp;
  int flag;  // bit 0: breakdown, bit 1: non-finite
};

constexpr int kKT = 256;

__device__ __forceinline__ void set_flags(KScalars *ks, double num, double den) {
  if (!isfinite(num) || !isfinite(den)) ks->flag |= 2;
  if (den == 0.0) ks->flag |= 1;
}

enum Post { POST_ALPHA = 0, POST_RHO_BETA = 1, POST_OMEGA = 2, POST_RHO = 3, POST_FCG = 4 };

// dot(a, b) with a post operation in the last block
__global__ void __launch_bounds__(kKT)
  k_dot_post(int64_t n, const double *__restrict__ a, const double *__restrict__ b, int post,
             KScalars *ks, double *partials, unsigned *counter) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s = fma(a[i], b[i], s);
  double t;
  if (grid_reduce<kKT>(s, blockIdx.x, gridDim.x, partials, counter, &t) && threadIdx.x == 0) {
    if (post == POST_ALPHA) {  // alpha = rho / t
      set_flags(ks, ks->rho, t);
      ks->den = t;
      ks->alpha = ks->rho / t;
    } else if (post == POST_RHO_BETA) {  // rho_old = rho; rho = t; beta = rho / rho_old
      ks->rho_old = ks->rho;
      ks->rho = t;
      set_flags(ks, t, ks->rho_old);
      ks->beta = t / ks->rho_old;
    } else if (post == POST_RHO) {  // initial rho = z.r (solver.hpp:63-64)
      ks->rho = t;
      if (!isfinite(t)) ks->flag |= 2;
    }
  }
}

// two dots in one pass: t1 = a.b, t2 = c.d
__global__ void __launch_bounds__(kKT)
  k_dot2_post(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
              const double *__restrict__ c, const double *__restrict__ d, int post, KScalars *ks,
              double *partials, double *partials2, unsigned *counter, unsigned *counter2) {
  double s1 = 0.0, s2 = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    s1 = fma(a[i], b[i], s1);
    s2 = fma(c[i], d[i], s2);
  }
  double t1, t2;
  const bool l1 = grid_reduce<kKT>(s1, blockIdx.x, gridDim.x, partials, counter, &t1);
  if (l1 && threadIdx.x == 0) ks->tmp = t1;
  const bool l2 = grid_reduce<kKT>(s2, blockIdx.x, gridDim.x, partials2, counter2, &t2);
  if (l2 && threadIdx.x == 0) {
    __threadfence();
    const double u1 = ((volatile KScalars *)ks)->tmp;
    if (post == POST_OMEGA) {  // omega = (t.r) / (t.t)
      set_flags(ks, u1, t2);
      ks->omega = u1 / t2;
    } else if (post == POST_FCG) {  // rho = r.z, beta = (r.z - r.z_old) / rho_old
      ks->rho_old = ks->rho;
      ks->rho = u1;
      set_flags(ks, u1, ks->rho_old);
      ks->beta = (u1 - t2) / ks->rho_old;
    }
  }
}

// x += alpha p ; r -= alpha q ; res2 = ||r||^2 (CG, solver.hpp:87, 93-94)
// plain: also rho_old = rho, rho = res2, beta = rho / rho_old (solver.hpp:105-107)
__global__ void __launch_bounds__(kKT)
  k_cg_update(int64_t n, KScalars *ks, const double *__restrict__ p, const double *__restrict__ q,
              double *__restrict__ x, double *__restrict__ r, int update_r, int plain,
              double *partials, unsigned *counter) {
  const double alpha = ks->alpha;
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = fma(p[i], alpha, x[i]);
    if (update_r) {
      const double rv = fma(-alpha, q[i], r[i]);
      r[i] = rv;
      s = fma(rv, rv, s);
    }
  }
  if (!update_r) return;
  double t;
  if (grid_reduce<kKT>(s, blockIdx.x, gridDim.x, partials, counter, &t) && threadIdx.x == 0) {
    ks->res2 = t;
    if (!isfinite(t)) ks->flag |= 2;
    if (plain) {
      ks->rho_old = ks->rho;
      ks->rho = t;
      ks->beta = t / ks->rho_old;
    }
  }
}

// after a true-residual recomputation into ks->res2 (plain CG bookkeeping)
__global__ void k_cg_plain_rho(KScalars *ks) {
  ks->rho_old = ks->rho;
  ks->rho = ks->res2;
  ks->beta = ks->res2 / ks->rho_old;
}

// p = z + beta p
__global__ void k_xpby(int64_t n, const KScalars *ks, const double *__restrict__ z,
                       double *__restrict__ p) {
  const double beta = ks->beta;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = fma(p[i], beta, z[i]);
}

// p = z + beta p and z_old = z (flexible CG)
__global__ void k_xpby_save(int64_t n, const KScalars *ks, const double *__restrict__ z,
                            double *__restrict__ p, double *__restrict__ z_old) {
  const double beta = ks->beta;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double zi = z[i];
    p[i] = fma(p[i], beta, zi);
    z_old[i] = zi;
  }
}

// x += s y with s = ks->alpha (which == 0) or ks->omega (which == 1)
__global__ void k_axpy_ks(int64_t n, const KScalars *ks, int which, const double *__restrict__ y,
                          double *__restrict__ x) {
  const double s = which == 0 ? ks->alpha : ks->omega;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = fma(y[i], s, x[i]);
}

// BiCGStab: r -= omega t (unless recomputed); rho_new = r.r0, res2 = r.r;
// beta = (rho_new / rho) * (alpha / omega); p = r + beta (p - omega v)
__global__ void __launch_bounds__(kKT)
  k_bicg_r(int64_t n, KScalars *ks, int update_r, const double *__restrict__ t,
           double *__restrict__ r, const double *__restrict__ r0, double *partials,
           double *partials2, unsigned *counter, unsigned *counter2) {
  const double omega = ks->omega;
  double s1 = 0.0, s2 = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double rv = r[i];
    if (update_r) {
      rv = fma(-omega, t[i], rv);
      r[i] = rv;
    }
    s1 = fma(rv, r0[i], s1);
    s2 = fma(rv, rv, s2);
  }
  double t1, t2;
  const bool l1 = grid_reduce<kKT>(s1, blockIdx.x, gridDim.x, partials, counter, &t1);
  if (l1 && threadIdx.x == 0) ks->tmp = t1;
  const bool l2 = grid_reduce<kKT>(s2, blockIdx.x, gridDim.x, partials2, counter2, &t2);
  if (l2 && threadIdx.x == 0) {
    __threadfence();
    const double rho_new = ((volatile KScalars *)ks)->tmp;
    ks->rho_old = ks->rho;
    ks->rho = rho_new;
    ks->res2 = t2;
    set_flags(ks, rho_new, ks->omega);
    if (ks->rho_old == 0.0) ks->flag |= 1;
    ks->beta = (rho_new / ks->rho_old) * (ks->alpha / ks->omega);
  }
}

__global__ void k_bicg_p(int64_t n, const KScalars *ks, const double *__restrict__ r,
                         const double *__restrict__ v, double *__restrict__ p) {
  const double beta = ks->beta, omega = ks->omega;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = fma(fma(-omega, v[i], p[i]), beta, r[i]);
}

// r = b - A x already computed with its norm: rho = res2 (BiCGStab init)
__global__ void k_bicg_init(KScalars *ks) {
  ks->rho = ks->res2;
  ks->flag = 0;
}

// ---------------------------------------------------------------------------
// Operator / preconditioner plumbing
// ---------------------------------------------------------------------------
struct Solver {
  const lgx_matrix *m = nullptr;  // natural-order operator (when pcsr == nullptr)
  const Csr *pcsr = nullptr;      // permuted CSR operator
  const int32_t *perm = nullptr;  // permuted -> natural (when pcsr)
  int precon = LGX_PRECON_NONE;
  double relax = 1.0;
  int ultra = 0;
  lgx_colouring *col = nullptr;   // SSOR colouring (permuted space)
  lgx_amg *amg = nullptr;
  const double *diag = nullptr;   // Jacobi
  int64_t n = 0;
  cudaStream_t s = nullptr;
  DBuf<double> partials, partials2;
  DBuf<unsigned> counters;
  DBuf<KScalars> ks;

  lgx_status init() {
    const int64_t slots = std::max<int64_t>(
      {(int64_t)reduce_blocks(n), pcsr ? csr_partials(n) : matrix_partials(m), (int64_t)1});
    LGX_CHECK(partials.alloc(slots));
    LGX_CHECK(partials2.alloc(slots));
    LGX_CHECK(counters.alloc(2));
    LGX_CHECK(ks.alloc(1));
    LGX_CUDA(cudaMemsetAsync(counters.p, 0, 2 * sizeof(unsigned), s));
    LGX_CUDA(cudaMemsetAsync(ks.p, 0, sizeof(KScalars), s));
    return LGX_OK;
  }
  lgx_status apply(const double *x, double *y) {
    if (pcsr) {
      if (pcsr->storage == LGX_F64) return csr_spmv<double, double>(*pcsr, pcsr->v64.p, x, y, s);
      return csr_spmv<float, double>(*pcsr, pcsr->v32.p, x, y, s);
    }
    return matrix_spmv(m, x, y, s);
  }
  lgx_status residual(const double *b, const double *x, double *r, double *norm) {
    if (pcsr) {
      if (pcsr->storage == LGX_F64)
        return csr_residual<double, double>(*pcsr, pcsr->v64.p, b, x, r, norm, partials.p,
                                            counters.p, s);
      return csr_residual<float, double>(*pcsr, pcsr->v32.p, b, x, r, norm, partials.p,
                                         counters.p, s);
    }
    return matrix_residual(m, b, x, r, norm, partials.p, counters.p, s);
  }
  lgx_status precondition(const double *r, double *z) {
    switch (precon) {
      case LGX_PRECON_JACOBI: return jacobi_diag_zero(n, diag, relax, r, z, s);
      case LGX_PRECON_SSOR: {
        if (col->stencil_rb) {
          // SsorBroom: forward from zero into z, backward in place
          LGX_CHECK(stencil_sor_sweep(m, relax, 1, ultra, nullptr, z, r, s));
          return stencil_sor_sweep(m, relax, 0, ultra, z, z, r, s);
        }
        // forward sweep from zero (x need not be cleared), backward in place
        const Csr &p = col->pcsr;
        if (p.storage == LGX_F64) {
          LGX_CHECK(mc_sor_sweep<double, double>(*col, p.v64.p, relax, 1, ultra, r, z, s, 1));
          return mc_sor_sweep<double, double>(*col, p.v64.p, relax, 0, ultra, r, z, s);
        }
        LGX_CHECK(mc_sor_sweep<float, double>(*col, p.v32.p, relax, 1, ultra, r, z, s, 1));
        return mc_sor_sweep<float, double>(*col, p.v32.p, relax, 0, ultra, r, z, s);
      }
      case LGX_PRECON_AMG: return amg_apply_permuted(*amg, r, z, s);
      default:
        LGX_CUDA(cudaMemcpyAsync(z, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        return LGX_OK;
    }
  }
  unsigned vgrid() const { return (unsigned)std::min<int64_t>(grid_for(n, 256), 16384); }
  lgx_status read(KScalars &h) {
    LGX_CUDA(cudaMemcpyAsync(&h, ks.p, sizeof(KScalars), cudaMemcpyDeviceToHost, s));
    LGX_CUDA(cudaStreamSynchronize(s));
    return LGX_OK;
  }
};

static lgx_status setup_solver(const lgx_matrix *a, const lgx_solve_params *p, cudaStream_t s,
                               Solver &S, std::unique_ptr<lgx_colouring> &own_col) {
  S.n = a->n;
  S.s = s;
  S.precon = p->precon;
  S.relax = p->relax;
  S.ultra = p->ultra;
  S.m = a;
  switch (p->precon) {
    case LGX_PRECON_NONE: break;
    case LGX_PRECON_JACOBI:
      LGX_CHECK(matrix_diagonal(const_cast<lgx_matrix *>(a), s, &S.diag));
      break;
    case LGX_PRECON_SSOR: {
      if (a->kind != LGX_MATRIX_CSR) {
        // matrix-free red-black SSOR in natural order
        lgx_colouring *c = const_cast<lgx_colouring *>(p->colouring);
        if (!c) {
          lgx_colouring *made = nullptr;
          LGX_CHECK(lgx_colouring_create_red_black(a, s, &made));
          own_col.reset(made);
          c = made;
        }
        if (!c->stencil_rb || c->n != a->n)
          return fail(LGX_ERR_INVALID, "a stencil's SSOR needs its red-black colouring");
        S.col = c;
        break;
      }
      lgx_colouring *c = const_cast<lgx_colouring *>(p->colouring);
      if (!c) {
        own_col = std::make_unique<lgx_colouring>();
        int32_t nc = 0;
        LGX_CHECK(colouring_jp(a->csr, 0x5eed, s, own_col->colour, nc));
        LGX_CHECK(colouring_build(a->csr, own_col->colour.p, nc, s, *own_col));
        c = own_col.get();
      }
      if (c->n != a->n) return fail(LGX_ERR_INVALID, "colouring does not match the matrix");
      S.col = c;
      S.pcsr = &c->pcsr;
      S.perm = c->perm.p;
      break;
    }
    case LGX_PRECON_AMG: {
      if (!p->amg) return fail(LGX_ERR_INVALID, "AMG preconditioner without a hierarchy");
      S.amg = p->amg;
      lgx_colouring *c = amg_finest_colouring(*p->amg);
      if (c) {
        if (c->n != a->n) return fail(LGX_ERR_INVALID, "hierarchy does not match the matrix");
        if (c->stencil_rb) {
          // matrix-free finest level: the iteration runs in natural order on
          // the stencil itself
          if (a->kind == LGX_MATRIX_CSR)
            return fail(LGX_ERR_INVALID, "the hierarchy was built on a stencil matrix");
        } else {
          S.pcsr = &c->pcsr;
          S.perm = c->perm.p;
        }
      }
      break;
    }
    default: return fail(LGX_ERR_INVALID, "unknown preconditioner");
  }
  return S.init();
}

struct Vecs {
  std::vector<DBuf<double>> v;
  lgx_status alloc(int count, int64_t n) {
    v.resize(count);
    for (auto &b : v) LGX_CHECK(b.alloc(n));
    return LGX_OK;
  }
  double *operator[](int i) { return v[i].p; }
};

static lgx_status check_flags(const KScalars &h, int64_t it) {
  if (h.flag & 2)
    return fail(LGX_ERR_NONFINITE, "non-finite value in iteration " + std::to_string(it));
  if (h.flag & 1)
    return fail(LGX_ERR_BREAKDOWN, "zero denominator in iteration " + std::to_string(it));
  return LGX_OK;
}

}  // namespace lgx

// Krylov solver state: the SystemInstance of the reference solvers.
struct lgx_krylov {
  int kind = LGX_KRYLOV_CG;
  lgx_solve_params p{};
  lgx::Solver S;
  std::unique_ptr<lgx_colouring> own_col;
  lgx::Vecs V;
  lgx::KScalars h{};
  int64_t it = 0;
  double r0 = 0.0;
  // captured iterations: [0] regular, [1] with true-residual recomputation
  cudaStream_t user_stream = nullptr;
  cudaStream_t capture_stream = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  uint64_t graph_kernels[2] = {0, 0};  // kernels recorded in each graph
  ~lgx_krylov() {
    for (auto &g : graph)
      if (g) cudaGraphExecDestroy(g);
    if (capture_stream) cudaStreamDestroy(capture_stream);
  }
};

namespace lgx {

// CG vectors: 0 b, 1 x, 2 r, 3 p, 4 q/z.  BiCGStab: 0 b, 1 x, 2 r, 3 r0, 4 p,
// 5 v, 6 t, 7 px.
static lgx_status krylov_init(lgx_krylov &K, const double *d_b, const double *d_x) {
  Solver &S = K.S;
  const int64_t n = S.n;
  const bool cg = K.kind == LGX_KRYLOV_CG;
  const bool flexible = cg && K.p.flexible && S.precon != LGX_PRECON_NONE;
  LGX_CHECK(K.V.alloc(cg ? (flexible ? 6 : 5) : 8, n));
  double *b = K.V[0], *x = K.V[1], *r = K.V[2];
  cudaStream_t s = S.s;
  if (S.perm) {
    LGX_CHECK(gather<double, double>(n, S.perm, d_b, b, s));
    LGX_CHECK(gather<double, double>(n, S.perm, d_x, x, s));
  } else {
    LGX_CUDA(cudaMemcpyAsync(b, d_b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    LGX_CUDA(cudaMemcpyAsync(x, d_x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  }
  KScalars *ks = S.ks.p;
  const unsigned rg = (unsigned)reduce_blocks(n);
  LGX_CHECK(S.residual(b, x, r, &ks->res2));
  if (cg) {
    // conjugate-gradients/solver.hpp:50-73
    double *pd = K.V[3];
    if (S.precon != LGX_PRECON_NONE) {
      LGX_CHECK(S.precondition(r, pd));
      k_dot_post<<<rg, kKT, 0, s>>>(n, pd, r, POST_RHO, ks, S.partials.p, S.counters.p);
      LGX_LAUNCH_CHECK();
      if (flexible)
        LGX_CUDA(cudaMemcpyAsync(K.V[5], pd, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    } else {
      LGX_CUDA(cudaMemcpyAsync(pd, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      k_cg_plain_rho<<<1, 1, 0, s>>>(ks);
      LGX_LAUNCH_CHECK();
    }
  } else {
    // bicgstab/solver.hpp:51-71
    LGX_CUDA(cudaMemcpyAsync(K.V[3], r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    LGX_CUDA(cudaMemcpyAsync(K.V[4], r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    k_bicg_init<<<1, 1, 0, s>>>(ks);
    LGX_LAUNCH_CHECK();
  }
  LGX_CHECK(S.read(K.h));
  if (!std::isfinite(K.h.res2) || !std::isfinite(K.h.rho))
    return fail(LGX_ERR_NONFINITE, "non-finite initial residual or preconditioned residual");
  K.r0 = std::sqrt(K.h.res2);
  K.it = 0;
  return LGX_OK;
}

// conjugate-gradients/solver.hpp:75-115
static lgx_status cg_iterate(lgx_krylov &K) {
  Solver &S = K.S;
  const int64_t n = S.n;
  cudaStream_t s = S.s;
  double *b = K.V[0], *x = K.V[1], *r = K.V[2], *pd = K.V[3], *q = K.V[4];
  KScalars *ks = S.ks.p;
  const unsigned rg = (unsigned)reduce_blocks(n);
  const bool precon = S.precon != LGX_PRECON_NONE;
  LGX_CHECK(S.apply(pd, q));
  k_dot_post<<<rg, kKT, 0, s>>>(n, pd, q, POST_ALPHA, ks, S.partials.p, S.counters.p);
  LGX_LAUNCH_CHECK();
  const bool rere = K.p.rere_period > 0 && K.it > 0 && K.it % K.p.rere_period == 0;
  k_cg_update<<<rg, kKT, 0, s>>>(n, ks, pd, q, x, r, rere ? 0 : 1, precon ? 0 : 1, S.partials.p,
                                 S.counters.p);
  LGX_LAUNCH_CHECK();
  if (rere) {
    LGX_CHECK(S.residual(b, x, r, &ks->res2));
    if (!precon) {
      k_cg_plain_rho<<<1, 1, 0, s>>>(ks);
      LGX_LAUNCH_CHECK();
    }
  }
  if (precon && K.p.flexible) {
    double *z_old = K.V[5];
    LGX_CHECK(S.precondition(r, q));
    k_dot2_post<<<rg, kKT, 0, s>>>(n, r, q, r, z_old, POST_FCG, ks, S.partials.p,
                                   S.partials2.p, S.counters.p, S.counters.p + 1);
    LGX_LAUNCH_CHECK();
    k_xpby_save<<<S.vgrid(), 256, 0, s>>>(n, ks, q, pd, z_old);
  } else if (precon) {
    LGX_CHECK(S.precondition(r, q));
    k_dot_post<<<rg, kKT, 0, s>>>(n, r, q, POST_RHO_BETA, ks, S.partials.p, S.counters.p);
    LGX_LAUNCH_CHECK();
    k_xpby<<<S.vgrid(), 256, 0, s>>>(n, ks, q, pd);
  } else {
    k_xpby<<<S.vgrid(), 256, 0, s>>>(n, ks, r, pd);
  }
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

// bicgstab/solver.hpp:73-151
static lgx_status bicgstab_iterate(lgx_krylov &K) {
  Solver &S = K.S;
  const int64_t n = S.n;
  cudaStream_t s = S.s;
  double *b = K.V[0], *x = K.V[1], *r = K.V[2], *r0 = K.V[3], *pd = K.V[4], *v = K.V[5],
         *t = K.V[6], *px = K.V[7];
  KScalars *ks = S.ks.p;
  const unsigned rg = (unsigned)reduce_blocks(n);
  const bool precon = S.precon != LGX_PRECON_NONE;
  double *partials2 = S.partials2.p;
  unsigned *c1 = S.counters.p, *c2 = S.counters.p + 1;
  const double *y = pd;
  if (precon) {
    LGX_CHECK(S.precondition(pd, px));
    y = px;
  }
  LGX_CHECK(S.apply(y, v));
  k_dot_post<<<rg, kKT, 0, s>>>(n, r0, v, POST_ALPHA, ks, S.partials.p, c1);
  LGX_LAUNCH_CHECK();
  k_cg_update<<<rg, kKT, 0, s>>>(n, ks, y, v, x, r, 1, 0, S.partials.p, c1);
  LGX_LAUNCH_CHECK();
  const double *z = r;
  if (precon) {
    LGX_CHECK(S.precondition(r, px));
    z = px;
  }
  LGX_CHECK(S.apply(z, t));
  k_dot2_post<<<rg, kKT, 0, s>>>(n, t, r, t, t, POST_OMEGA, ks, S.partials.p, partials2, c1, c2);
  LGX_LAUNCH_CHECK();
  k_axpy_ks<<<S.vgrid(), 256, 0, s>>>(n, ks, 1, z, x);
  LGX_LAUNCH_CHECK();
  const bool rere = K.p.rere_period > 0 && K.it > 0 && K.it % K.p.rere_period == 0;
  if (rere) LGX_CHECK(S.residual(b, x, r, nullptr));
  k_bicg_r<<<rg, kKT, 0, s>>>(n, ks, rere ? 0 : 1, t, r, r0, S.partials.p, partials2, c1, c2);
  LGX_LAUNCH_CHECK();
  k_bicg_p<<<S.vgrid(), 256, 0, s>>>(n, ks, r, v, pd);
  LGX_LAUNCH_CHECK();
  return LGX_OK;
}

static lgx_status iterate_body(lgx_krylov &K) {
  return K.kind == LGX_KRYLOV_CG ? cg_iterate(K) : bicgstab_iterate(K);
}

// Records one iteration (the variant selected by `rere`) into a CUDA graph.
// Capture runs on a private stream (the legacy default stream cannot be
// captured); the graph is then launched on the caller's stream.
static lgx_status capture_iteration(lgx_krylov &K, int rere) {
  if (!K.capture_stream)
    LGX_CUDA(cudaStreamCreateWithFlags(&K.capture_stream, cudaStreamNonBlocking));
  const int64_t saved_it = K.it;
  // the rere decision inside the bodies depends on K.it: pick a representative
  K.it = rere ? K.p.rere_period : 1;
  K.S.s = K.capture_stream;
  cudaGraph_t g = nullptr;
  const uint64_t before = launch_count();
  cudaError_t e = cudaStreamBeginCapture(K.capture_stream, cudaStreamCaptureModeThreadLocal);
  lgx_status st = e == cudaSuccess ? iterate_body(K) : cuda_fail(e, "cudaStreamBeginCapture");
  // recording does not launch: move the count to the replays
  K.graph_kernels[rere] = launch_count() - before;
  count_launches(0 - K.graph_kernels[rere]);
  cudaError_t e2 = cudaStreamEndCapture(K.capture_stream, &g);
  K.S.s = K.user_stream;
  K.it = saved_it;
  if (st != LGX_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&K.graph[rere], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return LGX_OK;
}

static lgx_status krylov_iterate(lgx_krylov &K) {
  const bool rere = K.p.rere_period > 0 && K.it > 0 && K.it % K.p.rere_period == 0;
  if (K.p.use_graphs && K.it > 0) {
    // the first iteration ran eagerly (it also initialises per-kernel
    // attributes); later iterations replay captured graphs
    if (!K.graph[rere]) LGX_CHECK(capture_iteration(K, rere ? 1 : 0));
    LGX_CUDA(cudaGraphLaunch(K.graph[rere], K.user_stream));
    count_launches(K.graph_kernels[rere]);
  } else {
    LGX_CHECK(iterate_body(K));
  }
  ++K.it;
  LGX_CHECK(K.S.read(K.h));
  return check_flags(K.h, K.it);
}

static lgx_status krylov_solution(lgx_krylov &K, double *d_x) {
  const int64_t n = K.S.n;
  if (K.S.perm) {
    LGX_CHECK(scatter<double, double>(n, K.S.perm, K.V[1], d_x, K.S.s));
  } else {
    LGX_CUDA(cudaMemcpyAsync(d_x, K.V[1], sizeof(double) * n, cudaMemcpyDeviceToDevice, K.S.s));
  }
  LGX_CUDA(cudaStreamSynchronize(K.S.s));
  return LGX_OK;
}

static lgx_status krylov_create(int kind, const lgx_matrix *a, const double *d_b,
                                const double *d_x, const lgx_solve_params *p, cudaStream_t s,
                                std::unique_ptr<lgx_krylov> &out) {
  auto K = std::make_unique<lgx_krylov>();
  K->kind = kind;
  K->p = *p;
  K->user_stream = s;
  LGX_CHECK(setup_solver(a, p, s, K->S, K->own_col));
  LGX_CHECK(krylov_init(*K, d_b, d_x));
  out = std::move(K);
  return LGX_OK;
}

static lgx_status run_solve(int kind, const lgx_matrix *a, const double *d_b, double *d_x,
                            const lgx_solve_params *p, cudaStream_t s, int64_t *iterations,
                            double *final_rel, double *history) {
  std::unique_ptr<lgx_krylov> K;
  LGX_CHECK(krylov_create(kind, a, d_b, d_x, p, s, K));
  if (history) history[0] = K->r0;
  double res = K->r0;
  lgx_status st = LGX_OK;
  // run_iterative_solver with the stopping rule ||r|| <= rtol ||r0||, maxit, rho == 0
  while (K->it < p->maxit && res > p->rtol * K->r0 && K->h.rho != 0.0) {
    st = krylov_iterate(*K);
    res = std::sqrt(K->h.res2);
    if (history) history[K->it] = res;
    if (st != LGX_OK) break;
  }
  const lgx_status st2 = krylov_solution(*K, d_x);
  if (iterations) *iterations = K->it;
  if (final_rel) *final_rel = K->r0 > 0 ? res / K->r0 : 0.0;
  return st != LGX_OK ? st : st2;
}

// ---------------------------------------------------------------------------
// FP64 iterative refinement over a float inner PCG (the precision form; no
// reference counterpart).  The inner CG runs the recurrence of
// conjugate-gradients/solver.hpp:75-115 on float vectors: float products of
// the finest level (grid or row kernels on the cycle's float values) and the
// float V-cycle, with every dot product compensated (Dot2f below) and the CG
// scalars kept in FP64 (KScalars).  The outer loop forms the FP64 residual,
// hands the inner solve r / ||r|| (so the float vectors stay O(1) however far
// the residual has fallen), adds ||r|| d to x in FP64 and stops on the FP64
// residual.
// ---------------------------------------------------------------------------

// Per-thread dot products of float vectors, compensated in FP32 (Ogita,
// Rump & Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26,
// 2005, Algorithm Dot2): each product is split exactly into p + e by an
// fma (TwoProduct), each running sum exactly into s + q (TwoSum), and the
// errors e + q are summed in a second float.  The result is as accurate as
// a sum in twice the working precision; it leaves the thread as s + c in
// FP64 and the partials meet in FP64.  On GB300 the FP32 pipe has 64 times
// the FP64 rate, and FP64 accumulation (two float-to-double conversions and
// a DFMA per element) made these dot kernels FP64-pipe bound.  The
// operations are the _rn intrinsics, which the compiler does not contract.
struct Dot2f {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float q = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    s = t;
    c = __fadd_rn(c, __fadd_rn(q, e));
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// dot(a, b) of float vectors (compensated, FP64 partials) with a post operation in the last block
__global__ void __launch_bounds__(kKT)
  k_fdot_post(int64_t n, const float *__restrict__ a, const float *__restrict__ b, int post,
              KScalars *ks, double *partials, unsigned *counter) {
  Dot2f acc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    acc.add(a[i], b[i]);
  double t;
  if (grid_reduce<kKT>(acc.value(), blockIdx.x, gridDim.x, partials, counter, &t) &&
      threadIdx.x == 0) {
    if (post == POST_ALPHA) {
      set_flags(ks, ks->rho, t);
      ks->den = t;
      ks->alpha = ks->rho / t;
    } else if (post == POST_RHO_BETA) {
      ks->rho_old = ks->rho;
      ks->rho = t;
      set_flags(ks, t, ks->rho_old);
      ks->beta = t / ks->rho_old;
    } else if (post == POST_RHO) {
      ks->rho = t;
      if (!isfinite(t)) ks->flag |= 2;
    }
  }
}

// r -= alpha q ; res2 = ||r||^2 (float vectors, FP64 alpha rounded once to
// float, compensated sum).  The iterate's d += alpha p waits for the
// direction kernel (k_fxpby_d), which reads p anyway.
__global__ void __launch_bounds__(kKT)
  k_fcg_update(int64_t n, KScalars *ks, const float *__restrict__ q, float *__restrict__ r,
               double *partials, unsigned *counter) {
  const float alpha = (float)ks->alpha;
  Dot2f acc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float rv = fmaf(-alpha, q[i], r[i]);
    r[i] = rv;
    acc.add(rv, rv);
  }
  double t;
  if (grid_reduce<kKT>(acc.value(), blockIdx.x, gridDim.x, partials, counter, &t) &&
      threadIdx.x == 0) {
    ks->res2 = t;
    if (!isfinite(t)) ks->flag |= 2;
  }
}

// d += alpha p (the deferred iterate update, before an FP64 residual)
__global__ void k_faxpy_alpha(int64_t n, const KScalars *ks, const float *__restrict__ p,
                              float *__restrict__ d) {
  const float alpha = (float)ks->alpha;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] = fmaf(p[i], alpha, d[i]);
}

// d += alpha p (this iteration's alpha), then p = z + beta p (float)
__global__ void k_fxpby_d(int64_t n, const KScalars *ks, const float *__restrict__ z,
                          float *__restrict__ p, float *__restrict__ d) {
  const float alpha = (float)ks->alpha;
  const float beta = (float)ks->beta;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float pi = p[i];
    d[i] = fmaf(pi, alpha, d[i]);
    p[i] = fmaf(pi, beta, z[i]);
  }
}

// flexible CG on float vectors: t1 = r.z, t2 = r.z_old (compensated sums), then
// rho_old = rho, rho = t1, beta = (t1 - t2) / rho_old (Notay 2000)
__global__ void __launch_bounds__(kKT)
  k_fdot2_fcg(int64_t n, const float *__restrict__ r, const float *__restrict__ z,
              const float *__restrict__ zold, KScalars *ks, double *partials, double *partials2,
              unsigned *counter, unsigned *counter2) {
  Dot2f acc1, acc2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float ri = r[i];
    acc1.add(ri, z[i]);
    acc2.add(ri, zold[i]);
  }
  double t1, t2;
  const bool l1 = grid_reduce<kKT>(acc1.value(), blockIdx.x, gridDim.x, partials, counter, &t1);
  if (l1 && threadIdx.x == 0) ks->tmp = t1;
  const bool l2 =
    grid_reduce<kKT>(acc2.value(), blockIdx.x, gridDim.x, partials2, counter2, &t2);
  if (l2 && threadIdx.x == 0) {
    __threadfence();
    const double u1 = ((volatile KScalars *)ks)->tmp;
    ks->rho_old = ks->rho;
    ks->rho = u1;
    set_flags(ks, u1, ks->rho_old);
    ks->beta = (u1 - t2) / ks->rho_old;
  }
}

// rf = float(r * inv_scale), d = 0
__global__ void k_refine_start(int64_t n, const double *__restrict__ r, double inv_scale,
                               float *__restrict__ rf, float *__restrict__ d) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    rf[i] = (float)(r[i] * inv_scale);
    d[i] = 0.0f;
  }
}

// x += scale * d (FP64)
__global__ void k_refine_add(int64_t n, const float *__restrict__ d, double scale,
                             double *__restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = fma((double)d[i], scale, x[i]);
}

struct Refiner {
  Solver S;
  std::unique_ptr<lgx_colouring> own_col;
  DBuf<double> b, x, r;
  DBuf<float> rf, df, pf, qf, zf, zf2;
  const float *v32 = nullptr;
  bool flexible = false;  // flexible beta (Notay 2000) for the float V-cycle
  // flexible CG needs the previous preconditioned residual: the V-cycle
  // writes z into zbuf(par) while zbuf(par ^ 1) still holds the previous z
  // (the buffers alternate instead of z being copied every iteration)
  int par = 0;
  float *zbuf(int k) { return k ? zf2.p : zf.p; }
  cudaStream_t user_stream = nullptr, capture_stream = nullptr;
  // graphs of the two halves of an inner iteration: [0] product and update,
  // [1 + par] preconditioner and new direction
  cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
  uint64_t graph_kernels[3] = {0, 0, 0};
  ~Refiner() {
    for (auto &g : graph)
      if (g) cudaGraphExecDestroy(g);
    if (capture_stream) cudaStreamDestroy(capture_stream);
  }

  // first half of a CG iteration on the float vectors: q = A p,
  // alpha = rho / p.q, r -= alpha q, ||r||^2 (d += alpha p follows in the
  // second half, or in fold_alpha before an FP64 residual)
  lgx_status half_update() {
    const int64_t n = S.n;
    cudaStream_t s = S.s;
    KScalars *ks = S.ks.p;
    const unsigned rg = (unsigned)reduce_blocks(n);
    LGX_CHECK((csr_spmv<float, float>(*S.pcsr, v32, pf.p, qf.p, s)));
    k_fdot_post<<<rg, kKT, 0, s>>>(n, pf.p, qf.p, POST_ALPHA, ks, S.partials.p, S.counters.p);
    LGX_LAUNCH_CHECK();
    k_fcg_update<<<rg, kKT, 0, s>>>(n, ks, qf.p, rf.p, S.partials.p, S.counters.p);
    LGX_LAUNCH_CHECK();
    return LGX_OK;
  }
  // second half: z = M r, rho = r.z, beta, d += alpha p, p = z + beta p
  lgx_status half_direction() {
    const int64_t n = S.n;
    cudaStream_t s = S.s;
    KScalars *ks = S.ks.p;
    const unsigned rg = (unsigned)reduce_blocks(n);
    float *z = flexible ? zbuf(par) : zf.p;
    LGX_CHECK(amg_apply_permuted_f32(*S.amg, rf.p, z, s));
    if (flexible) {
      k_fdot2_fcg<<<rg, kKT, 0, s>>>(n, rf.p, z, zbuf(par ^ 1), ks, S.partials.p,
                                     S.partials2.p, S.counters.p, S.counters.p + 1);
    } else {
      k_fdot_post<<<rg, kKT, 0, s>>>(n, rf.p, z, POST_RHO_BETA, ks, S.partials.p,
                                     S.counters.p);
    }
    LGX_LAUNCH_CHECK();
    k_fxpby_d<<<S.vgrid(), 256, 0, s>>>(n, ks, z, pf.p, df.p);
    LGX_LAUNCH_CHECK();
    return LGX_OK;
  }
  lgx_status half(int which) { return which == 0 ? half_update() : half_direction(); }

  // the float vectors of a solve of n rows
  lgx_status alloc(int64_t n) {
    LGX_CHECK(rf.alloc(n));
    LGX_CHECK(df.alloc(n));
    LGX_CHECK(pf.alloc(n));
    LGX_CHECK(qf.alloc(n));
    LGX_CHECK(zf.alloc(n));
    if (flexible) LGX_CHECK(zf2.alloc(n));
    return LGX_OK;
  }

  // d += alpha p now (the last update's alpha), and alpha = 0 so that the
  // direction kernel that follows adds nothing more
  lgx_status fold_alpha() {
    k_faxpy_alpha<<<S.vgrid(), 256, 0, S.s>>>(S.n, S.ks.p, pf.p, df.p);
    LGX_LAUNCH_CHECK();
    LGX_CUDA(cudaMemsetAsync(&S.ks.p->alpha, 0, sizeof(double), S.s));
    return LGX_OK;
  }

  lgx_status capture(int slot, int which) {
    if (!capture_stream)
      LGX_CUDA(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking));
    S.s = capture_stream;
    cudaGraph_t g = nullptr;
    const uint64_t before = launch_count();
    cudaError_t e = cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal);
    lgx_status st = e == cudaSuccess ? half(which) : cuda_fail(e, "cudaStreamBeginCapture");
    graph_kernels[slot] = launch_count() - before;
    count_launches(0 - graph_kernels[slot]);
    cudaError_t e2 = cudaStreamEndCapture(capture_stream, &g);
    S.s = user_stream;
    if (st != LGX_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&graph[slot], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return LGX_OK;
  }

  // one half, eagerly the first time (it also sets per-kernel attributes),
  // then replayed from its graph
  lgx_status run_half(int which, bool use_graphs, bool &first) {
    const int slot = which == 0 ? 0 : 1 + (flexible ? par : 0);
    if (use_graphs && !first) {
      if (!graph[slot]) LGX_CHECK(capture(slot, which));
      LGX_CUDA(cudaGraphLaunch(graph[slot], user_stream));
      count_launches(graph_kernels[slot]);
    } else {
      if (which == 1) first = false;
      LGX_CHECK(half(which));
    }
    if (which == 1 && flexible) par ^= 1;
    return LGX_OK;
  }
};

static lgx_status run_refined(const lgx_matrix *a, const double *d_b, double *d_x,
                              const lgx_solve_params *p, cudaStream_t s, int64_t *iterations,
                              double *final_rel, double *history) {
  if (p->precon != LGX_PRECON_AMG || !p->amg)
    return fail(LGX_ERR_UNSUPPORTED, "refinement needs the AMG preconditioner");
  if (!amg_cycle_f32(*p->amg))
    return fail(LGX_ERR_UNSUPPORTED, "refinement needs a float-cycle hierarchy (cycle_f32)");
  if (!(p->inner_rtol > 0.0 && p->inner_rtol < 1.0))
    return fail(LGX_ERR_INVALID, "inner_rtol must lie in (0, 1)");
  Refiner R;
  R.user_stream = s;
  LGX_CHECK(setup_solver(a, p, s, R.S, R.own_col));
  Solver &S = R.S;
  if (!S.pcsr) return fail(LGX_ERR_UNSUPPORTED, "refinement needs a CSR finest level");
  const int64_t n = S.n;
  R.v32 = amg_finest_values_f32(*S.amg);
  LGX_CHECK(R.b.alloc(n));
  LGX_CHECK(R.x.alloc(n));
  LGX_CHECK(R.r.alloc(n));
  LGX_CHECK(R.alloc(n));
  LGX_CHECK(gather<double, double>(n, S.perm, d_b, R.b.p, s));
  LGX_CHECK(gather<double, double>(n, S.perm, d_x, R.x.p, s));
  KScalars *ks = S.ks.p;
  KScalars h{};
  const unsigned rg = (unsigned)reduce_blocks(n);
  LGX_CHECK(S.residual(R.b.p, R.x.p, R.r.p, &ks->res2));
  LGX_CHECK(S.read(h));
  if (!std::isfinite(h.res2)) return fail(LGX_ERR_NONFINITE, "non-finite initial residual");
  const double r0 = std::sqrt(h.res2);
  double res = r0;
  if (history) history[0] = r0;
  int64_t it = 0;
  bool first = true;
  lgx_status st = LGX_OK;
  while (st == LGX_OK && it < p->maxit && res > p->rtol * r0 && res > 0.0) {
    // inner solve of A d = r / ||r|| to the tolerance this step needs
    const double scale = res;
    const double tol = std::max(p->inner_rtol, 0.5 * p->rtol * r0 / res);
    k_refine_start<<<S.vgrid(), 256, 0, s>>>(n, R.r.p, 1.0 / scale, R.rf.p, R.df.p);
    LGX_LAUNCH_CHECK();
    LGX_CHECK(amg_apply_permuted_f32(*S.amg, R.rf.p, R.zf.p, s));
    k_fdot_post<<<rg, kKT, 0, s>>>(n, R.rf.p, R.zf.p, POST_RHO, ks, S.partials.p, S.counters.p);
    LGX_LAUNCH_CHECK();
    LGX_CUDA(cudaMemcpyAsync(R.pf.p, R.zf.p, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    R.par = R.flexible ? 1 : 0;  // this solve's first z is the previous z of its first step
    LGX_CHECK(S.read(h));
    LGX_CHECK(check_flags(h, it));
    double inner = 1.0;
    while (it < p->maxit && inner > tol && h.rho != 0.0) {
      st = R.run_half(0, p->use_graphs != 0, first);
      if (st == LGX_OK) st = R.run_half(1, p->use_graphs != 0, first);
      if (st != LGX_OK) break;
      ++it;
      LGX_CHECK(S.read(h));
      st = check_flags(h, it);
      inner = std::sqrt(h.res2);
      if (history) history[it] = scale * inner;
      if (st != LGX_OK) break;
    }
    if (st != LGX_OK) break;
    k_refine_add<<<S.vgrid(), 256, 0, s>>>(n, R.df.p, scale, R.x.p);
    LGX_LAUNCH_CHECK();
    LGX_CHECK(S.residual(R.b.p, R.x.p, R.r.p, &ks->res2));
    LGX_CHECK(S.read(h));
    if (!std::isfinite(h.res2)) {
      st = fail(LGX_ERR_NONFINITE, "non-finite residual after refinement step");
      break;
    }
    const double prev = res;
    res = std::sqrt(h.res2);
    if (history) history[it] = res;
    // an inner solve that no longer reduces the FP64 residual (float
    // precision reached on an operator the float cycle cannot resolve) ends
    // the refinement
    if (res >= prev) break;
  }
  LGX_CHECK(scatter<double, double>(n, S.perm, R.x.p, d_x, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  if (iterations) *iterations = it;
  if (final_rel) *final_rel = r0 > 0 ? res / r0 : 0.0;
  return st;
}

// Reliable updates (refine == 2; H. A. van der Vorst, Q. Ye, "Residual
// replacement strategies for Krylov subspace iterative methods for the
// convergence of true residuals", SIAM J. Sci. Comput. 22 (2000), in the
// mixed-precision form of M. A. Clark et al., "Solving lattice QCD systems of
// equations using mixed precision solvers on GPUs", Comput. Phys. Commun. 181
// (2010)): one CG recurrence on float vectors, never restarted.  The float
// iterate d accumulates updates to the FP64 solution x; whenever the
// recursive residual has fallen by reliable_delta since the last FP64
// residual (and when it reaches the tolerance), x += d, d = 0 and r is
// replaced by the FP64 residual b - A x before the next preconditioner
// application.  The search direction is kept, so the iteration count stays
// the FP64 recurrence's while the products, V-cycles and vector updates run
// in float; the solve stops on the FP64 residual.
static lgx_status run_reliable(const lgx_matrix *a, const double *d_b, double *d_x,
                               const lgx_solve_params *p, cudaStream_t s, int64_t *iterations,
                               double *final_rel, double *history) {
  if (p->precon != LGX_PRECON_AMG || !p->amg)
    return fail(LGX_ERR_UNSUPPORTED, "refinement needs the AMG preconditioner");
  if (!amg_cycle_f32(*p->amg))
    return fail(LGX_ERR_UNSUPPORTED, "refinement needs a float-cycle hierarchy (cycle_f32)");
  if (!(p->inner_rtol > 0.0 && p->inner_rtol < 1.0))
    return fail(LGX_ERR_INVALID, "inner_rtol must lie in (0, 1)");
  Refiner R;
  R.user_stream = s;
  LGX_CHECK(setup_solver(a, p, s, R.S, R.own_col));
  Solver &S = R.S;
  if (!S.pcsr) return fail(LGX_ERR_UNSUPPORTED, "refinement needs a CSR finest level");
  const int64_t n = S.n;
  R.v32 = amg_finest_values_f32(*S.amg);
  LGX_CHECK(R.b.alloc(n));
  LGX_CHECK(R.x.alloc(n));
  LGX_CHECK(R.r.alloc(n));
  R.flexible = p->flexible != 0;
  LGX_CHECK(R.alloc(n));
  LGX_CHECK(gather<double, double>(n, S.perm, d_b, R.b.p, s));
  LGX_CHECK(gather<double, double>(n, S.perm, d_x, R.x.p, s));
  KScalars *ks = S.ks.p;
  KScalars h{};
  const unsigned rg = (unsigned)reduce_blocks(n);
  LGX_CHECK(S.residual(R.b.p, R.x.p, R.r.p, &ks->res2));
  LGX_CHECK(S.read(h));
  if (!std::isfinite(h.res2)) return fail(LGX_ERR_NONFINITE, "non-finite initial residual");
  const double r0 = std::sqrt(h.res2);
  double res = r0, last = r0;
  if (history) history[0] = r0;
  int64_t it = 0;
  lgx_status st = LGX_OK;
  if (r0 > 0.0 && p->maxit > 0) {
    // r = float(b - A x), d = 0, z = M r, rho = r.z, p = z
    k_refine_start<<<S.vgrid(), 256, 0, s>>>(n, R.r.p, 1.0, R.rf.p, R.df.p);
    LGX_LAUNCH_CHECK();
    LGX_CHECK(amg_apply_permuted_f32(*S.amg, R.rf.p, R.zf.p, s));
    k_fdot_post<<<rg, kKT, 0, s>>>(n, R.rf.p, R.zf.p, POST_RHO, ks, S.partials.p, S.counters.p);
    LGX_LAUNCH_CHECK();
    LGX_CUDA(cudaMemcpyAsync(R.pf.p, R.zf.p, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    R.par = R.flexible ? 1 : 0;  // z is the previous z of the first step
    LGX_CHECK(S.read(h));
    LGX_CHECK(check_flags(h, 0));
  }
  bool first = true, pending = false;
  const bool graphs = p->use_graphs != 0;
  while (st == LGX_OK && it < p->maxit && res > p->rtol * r0 && h.rho != 0.0) {
    st = R.run_half(0, graphs, first);
    if (st != LGX_OK) break;
    ++it;
    pending = true;
    LGX_CHECK(S.read(h));
    st = check_flags(h, it);
    if (st != LGX_OK) break;
    const double est = std::sqrt(h.res2);
    if (history) history[it] = est;
    if (est <= p->inner_rtol * last || est <= p->rtol * r0 || it == p->maxit) {
      // reliable update: fold d into x and replace r by the FP64 residual
      LGX_CHECK(R.fold_alpha());
      k_refine_add<<<S.vgrid(), 256, 0, s>>>(n, R.df.p, 1.0, R.x.p);
      LGX_LAUNCH_CHECK();
      LGX_CHECK(S.residual(R.b.p, R.x.p, R.r.p, &ks->res2));
      k_refine_start<<<S.vgrid(), 256, 0, s>>>(n, R.r.p, 1.0, R.rf.p, R.df.p);
      LGX_LAUNCH_CHECK();
      LGX_CHECK(S.read(h));
      if (!std::isfinite(h.res2)) {
        st = fail(LGX_ERR_NONFINITE, "non-finite residual at a reliable update");
        break;
      }
      res = last = std::sqrt(h.res2);
      pending = false;
      if (history) history[it] = res;
      if (res <= p->rtol * r0 || it == p->maxit) break;
    }
    st = R.run_half(1, graphs, first);
  }
  if (st == LGX_OK && pending) {
    // a breakdown (rho = 0) ended the recurrence between updates
    k_refine_add<<<S.vgrid(), 256, 0, s>>>(n, R.df.p, 1.0, R.x.p);
    LGX_LAUNCH_CHECK();
    LGX_CHECK(S.residual(R.b.p, R.x.p, R.r.p, &ks->res2));
    LGX_CHECK(S.read(h));
    res = std::sqrt(h.res2);
    if (history) history[it] = res;
  }
  LGX_CHECK(scatter<double, double>(n, S.perm, R.x.p, d_x, s));
  LGX_CUDA(cudaStreamSynchronize(s));
  if (iterations) *iterations = it;
  if (final_rel) *final_rel = r0 > 0 ? res / r0 : 0.0;
  return st;
}

}  // namespace lgx

using namespace lgx;

extern "C" {

void lgx_solve_default_params(lgx_solve_params *p) {
  if (!p) return;
  p->precon = LGX_PRECON_NONE;
  p->relax = 1.0;
  p->ultra = 0;
  p->colouring = nullptr;
  p->amg = nullptr;
  p->rtol = 1e-8;
  p->maxit = 1000;
  p->rere_period = 8;
  p->use_graphs = 1;
  p->flexible = 0;
  p->refine = 0;
  p->inner_rtol = 1e-4;
}

lgx_status lgx_pcg(const lgx_matrix *a, const double *d_b, double *d_x,
                   const lgx_solve_params *p, lgx_stream stream, int64_t *iterations,
                   double *final_rel_residual, double *h_history) {
  if (!a || !p || (a->n > 0 && (!d_b || !d_x))) return fail(LGX_ERR_INVALID, "null argument");
  if (p->refine == 2)
    return run_reliable(a, d_b, d_x, p, stream, iterations, final_rel_residual, h_history);
  if (p->refine == 1)
    return run_refined(a, d_b, d_x, p, stream, iterations, final_rel_residual, h_history);
  if (p->refine)
    return fail(LGX_ERR_INVALID, "refine must be 0, 1 (restarted inner solves) or 2 (reliable "
                                 "updates)");
  return run_solve(LGX_KRYLOV_CG, a, d_b, d_x, p, stream, iterations, final_rel_residual,
                   h_history);
}

lgx_status lgx_pbicgstab(const lgx_matrix *a, const double *d_b, double *d_x,
                         const lgx_solve_params *p, lgx_stream stream, int64_t *iterations,
                         double *final_rel_residual, double *h_history) {
  if (!a || !p || (a->n > 0 && (!d_b || !d_x))) return fail(LGX_ERR_INVALID, "null argument");
  if (p->refine) return fail(LGX_ERR_UNSUPPORTED, "refinement is a CG option");
  return run_solve(LGX_KRYLOV_BICGSTAB, a, d_b, d_x, p, stream, iterations, final_rel_residual,
                   h_history);
}

lgx_status lgx_krylov_create(int kind, const lgx_matrix *a, const double *d_b,
                             const double *d_x, const lgx_solve_params *p, lgx_stream stream,
                             lgx_krylov **out) {
  if (!a || !p || !out || (a->n > 0 && (!d_b || !d_x)))
    return fail(LGX_ERR_INVALID, "null argument");
  if (kind != LGX_KRYLOV_CG && kind != LGX_KRYLOV_BICGSTAB)
    return fail(LGX_ERR_INVALID, "unknown Krylov method");
  if (p->refine) return fail(LGX_ERR_UNSUPPORTED, "refinement runs through lgx_pcg only");
  std::unique_ptr<lgx_krylov> K;
  LGX_CHECK(krylov_create(kind, a, d_b, d_x, p, stream, K));
  *out = K.release();
  return LGX_OK;
}

lgx_status lgx_krylov_iterate(lgx_krylov *k) {
  if (!k) return fail(LGX_ERR_INVALID, "null solver");
  return krylov_iterate(*k);
}

lgx_status lgx_krylov_state(const lgx_krylov *k, int64_t *iteration, double *residual_norm,
                            double *rho) {
  if (!k) return fail(LGX_ERR_INVALID, "null solver");
  if (iteration) *iteration = k->it;
  if (residual_norm) *residual_norm = std::sqrt(k->h.res2);
  if (rho) *rho = k->h.rho;
  return LGX_OK;
}

lgx_status lgx_krylov_solution(lgx_krylov *k, double *d_x) {
  if (!k || !d_x) return fail(LGX_ERR_INVALID, "null argument");
  return krylov_solution(*k, d_x);
}

lgx_status lgx_krylov_destroy(lgx_krylov *k) {
  delete k;
  return LGX_OK;
}

}  // extern "C"
