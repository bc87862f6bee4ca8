// Autotuner of the CSR row-engine configuration (block and tile shapes).
//
// The row engine (lgx_rows.cuh) has eight configurations: three CTA-tile
// shapes and five warp-tile shapes (warps per CTA x pipeline stages x CTAs
// per SM).  Which one is fastest depends on the matrix (rows, entries per
// row, how many rows there are to spread over 152 SMs) and on the
// operation: a product
// streams values once, an SOR sweep runs one launch per colour over a
// fraction of the rows.  The tuner times every configuration on the matrix
// itself (replays of a CUDA graph of the operation, timed with CUDA events,
// the way a captured solver iteration runs it) and records the fastest in
// the matrix's Csr::tuned slot for that operation class and value type;
// launch_rows reads the slot on every later launch.  Every configuration forms each row in the
// same order, so a tuned matrix gives bit-identical products and sweeps.
//
// The reference has no counterpart: its kernels are CPU loops whose shape
// is fixed at compile time.

#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>

#include "lgx_amg.cuh"
#include "lgx_internal.cuh"

namespace lgx {

lgx_status amg_apply_permuted(lgx_amg &h, const double *b, double *x, cudaStream_t s);
int rows_config();

constexpr int kTuneConfigs = 8;
static_assert(kTuneConfigs == LGX_TUNE_CONFIGS, "tuning space and ABI disagree");

namespace {

struct TuneObjects {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaStream_t capture = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
  ~TuneObjects() {
    drop_graph();
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (capture) cudaStreamDestroy(capture);
  }
};

// `reps` operations recorded as one CUDA graph, replayed once untimed and
// once timed on `s`: the time is the device-side cost of the launches as a
// captured solver iteration sees it, without host launch overhead
template <class Run>
lgx_status time_graph(TuneObjects &o, int reps, cudaStream_t s, Run &run, float *ms,
                      int replays = 1) {
  o.drop_graph();
  cudaError_t e = cudaStreamBeginCapture(o.capture, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
  lgx_status st = LGX_OK;
  const uint64_t before = launch_count();
  for (int r = 0; r < reps && st == LGX_OK; ++r) st = run(o.capture);
  // recording launches nothing: the count moves to the two replays
  const uint64_t recorded = launch_count() - before;
  count_launches(0 - recorded);
  e = cudaStreamEndCapture(o.capture, &o.graph);
  LGX_CHECK(st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  LGX_CUDA(cudaGraphInstantiate(&o.exec, o.graph, 0));
  LGX_CUDA(cudaGraphLaunch(o.exec, s));
  float best = FLT_MAX;
  for (int k = 0; k < replays; ++k) {
    LGX_CUDA(cudaEventRecord(o.a, s));
    LGX_CUDA(cudaGraphLaunch(o.exec, s));
    LGX_CUDA(cudaEventRecord(o.b, s));
    LGX_CUDA(cudaEventSynchronize(o.b));
    float t = 0.f;
    LGX_CUDA(cudaEventElapsedTime(&t, o.a, o.b));
    best = std::min(best, t);
  }
  count_launches((uint64_t)(replays + 1) * recorded);
  *ms = best / (float)reps;
  return LGX_OK;
}

lgx_status tune_objects(TuneObjects &o) {
  LGX_CUDA(cudaEventCreate(&o.a));
  LGX_CUDA(cudaEventCreate(&o.b));
  LGX_CUDA(cudaStreamCreateWithFlags(&o.capture, cudaStreamNonBlocking));
  return LGX_OK;
}

// Times `run` (one operation on the stream it is given) under every
// configuration with the slot set to it, then leaves the slot at the fastest.
template <class Run>
lgx_status tune_slot(int8_t &slot, int reps, cudaStream_t s, lgx_tune_entry &e, Run run) {
  TuneObjects o;
  LGX_CHECK(tune_objects(o));
  const int8_t before = slot;
  float best = FLT_MAX;
  int best_cfg = -1;
  for (int cfg = 0; cfg < kTuneConfigs; ++cfg) {
    slot = (int8_t)cfg;
    // one eager launch first: kernel attributes are set outside the capture
    lgx_status st = run(s);
    float ms = 0.f;
    if (st == LGX_OK) st = time_graph(o, reps, s, run, &ms);
    if (st != LGX_OK) {
      slot = before;
      return st;
    }
    e.ms[cfg] = ms;
    if (ms < best) {
      best = ms;
      best_cfg = cfg;
    }
  }
  // a wait that ran out inside the engine is reported, not tuned around
  const lgx_status st = check_device_error(s);
  if (st != LGX_OK) {
    slot = before;
    return st;
  }
  slot = (int8_t)best_cfg;
  e.config = best_cfg;
  e.fastest = best_cfg;
  return LGX_OK;
}

lgx_tune_entry blank_entry(int level, int op, int value_bytes) {
  lgx_tune_entry e{};
  e.level = level;
  e.op = op;
  e.value_bytes = value_bytes;
  e.config = -1;
  e.fastest = -1;
  return e;
}

// stored-value bytes the V-cycle of `h` reads on a level with colouring `c`
int cycle_value_bytes(const lgx_amg &h, const lgx_colouring &c) {
  if (!h.f32) return c.pcsr.storage == LGX_F64 ? 8 : 4;
  return h.p.cycle_bf16 ? 2 : 4;
}

// One V-cycle (zero right-hand side; the work does not depend on values),
// recorded and replayed: minimum of three timed replays.
lgx_status time_cycle(lgx_amg &h, TuneObjects &o, const double *b, double *x, int reps,
                      cudaStream_t s, float *ms) {
  auto run = [&](cudaStream_t cs) { return amg_apply_permuted(h, b, x, cs); };
  LGX_CHECK(run(s));  // eager: attributes of newly chosen shapes are set outside the capture
  return time_graph(o, reps, s, run, ms, 3);
}

// The isolated timings rank each level's shapes.  Inside the cycle a kernel
// shares the SMs with its early-scheduled successor, so a level's winners
// are kept only when the whole V-cycle is also faster with them than with
// the process-wide configuration at that level.
lgx_status confirm_in_cycle(lgx_amg &h, std::vector<lgx_tune_entry> &all, int reps,
                            cudaStream_t s) {
  const int L = (int)h.lv.size();
  if (L < 2) return LGX_OK;
  const int64_t n = h.lv[0]->a->n;
  DBuf<double> b, x;
  LGX_CHECK(b.alloc(n));
  LGX_CHECK(x.alloc(n));
  LGX_CUDA(cudaMemsetAsync(b.p, 0, sizeof(double) * (size_t)n, s));
  TuneObjects o;
  LGX_CHECK(tune_objects(o));
  const int def = rows_config();
  for (int l = 0; l + 1 < L; ++l) {
    lgx_amg_level &lv = *h.lv[l];
    if (!lv.col) continue;
    Csr &p = lv.col->pcsr;
    const int vb = cycle_value_bytes(h, *lv.col);
    const int vi = vb == 8 ? 0 : vb == 4 ? 1 : 2;
    std::vector<lgx_tune_entry *> changed;
    for (auto &e : all)
      if (e.level == l && e.value_bytes == vb && e.config >= 0 && e.config != def)
        changed.push_back(&e);
    if (changed.empty()) continue;
    float t_win = 0.f, t_def = 0.f;
    LGX_CHECK(time_cycle(h, o, b.p, x.p, reps, s, &t_win));
    for (auto *e : changed) p.tuned[e->op][vi] = -1;
    LGX_CHECK(time_cycle(h, o, b.p, x.p, reps, s, &t_def));
    if (t_win < t_def) {
      for (auto *e : changed) p.tuned[e->op][vi] = (int8_t)e->config;
    } else {
      for (auto *e : changed) e->config = def;
    }
  }
  return check_device_error(s);
}

template <typename XT>
struct Scratch {
  DBuf<XT> b, x, r;
  lgx_status alloc(int64_t n, cudaStream_t s) {
    LGX_CHECK(b.alloc(n));
    LGX_CHECK(x.alloc(n));
    LGX_CHECK(r.alloc(n));
    // zero vectors: the timed work does not depend on the values
    LGX_CUDA(cudaMemsetAsync(b.p, 0, sizeof(XT) * (size_t)n, s));
    LGX_CUDA(cudaMemsetAsync(x.p, 0, sizeof(XT) * (size_t)n, s));
    return LGX_OK;
  }
};

// residual (class 0) and forward SOR sweep (class 1) of one level in the
// value type VT and vector type XT its cycle reads
template <typename VT, typename XT>
lgx_status tune_level(lgx_colouring &c, const VT *val, const float *scale, double relax, int ultra,
                      int level, int reps, cudaStream_t s, std::vector<lgx_tune_entry> &out) {
  Csr &p = c.pcsr;
  Scratch<XT> v;
  LGX_CHECK(v.alloc(p.n, s));
  const int vi = tune_value_index<VT>();
  lgx_tune_entry e = blank_entry(level, 0, (int)sizeof(VT));
  LGX_CHECK(tune_slot(p.tuned[0][vi], reps, s, e, [&](cudaStream_t cs) {
    return csr_residual<VT, XT>(p, val, v.b.p, v.x.p, v.r.p, nullptr, nullptr, nullptr, cs,
                                scale);
  }));
  out.push_back(e);
  e = blank_entry(level, 1, (int)sizeof(VT));
  LGX_CHECK(tune_slot(p.tuned[1][vi], reps, s, e, [&](cudaStream_t cs) {
    return mc_sor_sweep<VT, XT>(c, val, relax, 1, ultra, v.b.p, v.x.p, cs, 0, scale);
  }));
  out.push_back(e);
  return LGX_OK;
}

// y = A x with FP64 vectors (the outer Krylov product and lgx_spmv)
lgx_status tune_product64(Csr &a, int level, int reps, cudaStream_t s,
                          std::vector<lgx_tune_entry> &out) {
  Scratch<double> v;
  LGX_CHECK(v.alloc(a.n, s));
  const bool f64 = a.storage == LGX_F64;
  lgx_tune_entry e = blank_entry(level, 0, f64 ? 8 : 4);
  LGX_CHECK(tune_slot(a.tuned[0][f64 ? 0 : 1], reps, s, e, [&](cudaStream_t cs) {
    return f64 ? csr_spmv<double, double>(a, a.v64.p, v.x.p, v.r.p, cs)
               : csr_spmv<float, double>(a, a.v32.p, v.x.p, v.r.p, cs);
  }));
  out.push_back(e);
  return LGX_OK;
}

lgx_status copy_out(const std::vector<lgx_tune_entry> &all, lgx_tune_entry *out, int max_out,
                    int *n_out) {
  if (n_out) *n_out = (int)all.size();
  if (out)
    std::copy_n(all.begin(), std::min<size_t>(all.size(), (size_t)std::max(max_out, 0)), out);
  return LGX_OK;
}

}  // namespace
}  // namespace lgx

using namespace lgx;

lgx_status lgx_matrix_autotune(lgx_matrix *a, int reps, lgx_tune_entry *out, lgx_stream stream) {
  if (!a) return fail(LGX_ERR_INVALID, "null matrix");
  if (a->kind != LGX_MATRIX_CSR) return fail(LGX_ERR_UNSUPPORTED, "autotune needs a CSR matrix");
  if (reps < 1 || reps > 1000) return fail(LGX_ERR_INVALID, "reps must be in [1, 1000]");
  std::vector<lgx_tune_entry> all;
  if (a->csr.n > 0) LGX_CHECK(tune_product64(a->csr, 0, reps, (cudaStream_t)stream, all));
  else all.push_back(blank_entry(0, 0, a->csr.storage == LGX_F64 ? 8 : 4));
  return copy_out(all, out, 1, nullptr);
}

lgx_status lgx_amg_autotune(lgx_amg *h, int reps, lgx_tune_entry *out, int max_out, int *n_out,
                            lgx_stream stream) {
  if (!h) return fail(LGX_ERR_INVALID, "null hierarchy");
  if (reps < 1 || reps > 1000) return fail(LGX_ERR_INVALID, "reps must be in [1, 1000]");
  if (out && max_out < 0) return fail(LGX_ERR_INVALID, "max_out must not be negative");
  const cudaStream_t s = (cudaStream_t)stream;
  const double relax = h->p.smoother_relax;
  const int ultra = h->p.smoother_ultra;
  std::vector<lgx_tune_entry> all;
  const int L = (int)h->lv.size();
  for (int l = 0; l < L; ++l) {
    lgx_amg_level &lv = *h->lv[l];
    // the coarsest level is solved densely; it has no smoother; a
    // grid level runs its own kernels, not the row engine
    if (!lv.col || l == L - 1 || lv.col->pcsr.n == 0 || lv.col->pcsr.grid) continue;
    lgx_colouring &c = *lv.col;
    if (l == 0 && c.pcsr.storage == LGX_F64 && h->f32)
      LGX_CHECK(tune_product64(c.pcsr, 0, reps, s, all));
    if (!h->f32) {
      if (c.pcsr.storage == LGX_F64)
        LGX_CHECK((tune_level<double, double>(c, c.pcsr.v64.p, nullptr, relax, ultra, l, reps, s,
                                              all)));
      else
        LGX_CHECK((tune_level<float, double>(c, c.pcsr.v32.p, nullptr, relax, ultra, l, reps, s,
                                             all)));
    } else if (h->p.cycle_bf16) {
      LGX_CHECK((tune_level<bf16, float>(c, c.pv16.p, c.pscale.p, relax, ultra, l, reps, s,
                                         all)));
    } else {
      const float *v = c.pcsr.storage == LGX_F32 ? c.pcsr.v32.p : c.pv32.p;
      LGX_CHECK((tune_level<float, float>(c, v, nullptr, relax, ultra, l, reps, s, all)));
    }
  }
  LGX_CHECK(confirm_in_cycle(*h, all, reps, s));
  return copy_out(all, out, max_out, n_out);
}

lgx_status lgx_amg_autotune_reset(lgx_amg *h) {
  if (!h) return fail(LGX_ERR_INVALID, "null hierarchy");
  for (auto &lv : h->lv)
    if (lv->col)
      for (auto &cls : lv->col->pcsr.tuned)
        for (auto &slot : cls) slot = -1;
  return LGX_OK;
}
