// Internal layout of an aggregation-AMG hierarchy, shared by the setup and
// V-cycle (lgx_amg.cu) and the multi-right-hand-side cycle (lgx_multi.cu).
#pragma once

#include <memory>
#include <vector>

#include "lgx_internal.cuh"

namespace lgx {

// aggregation of one level: fine -> coarse map and per-aggregate member lists
struct AggResult {
  int64_t ncoarse = 0;
  DBuf<uint32_t> agg;
  DBuf<int64_t> list_ptr;
  DBuf<int32_t> list;
  int64_t stats[5] = {0, 0, 0, 0, 0};
};

}  // namespace lgx

struct lgx_amg_level {
  lgx::Csr own;                      // natural-order matrix (levels >= 1)
  const lgx::Csr *a = nullptr;       // natural-order matrix of this level
  lgx::AggResult agg;                // this level -> next (non-coarsest levels)
  std::unique_ptr<lgx_colouring> col;  // smoother colouring and permuted matrix
  lgx::DBuf<uint32_t> agg_p;         // permuted fine -> permuted coarse
  lgx::DBuf<int64_t> rptr;           // permuted coarse row -> fine rows (permuted)
  lgx::DBuf<int32_t> rlist;
  lgx::DBuf<double> b64, x64, r64;   // cycle vectors (permuted order)
  lgx::DBuf<float> b32, x32, r32;
  // level 0 of a hierarchy built on a stencil matrix: the smoother and the
  // residual run matrix-free on it (red-black, natural order); `own` then
  // keeps only the sizes of the assembled matrix the setup used
  const lgx_matrix *stencil = nullptr;
};

struct lgx_amg {
  lgx_amg_params p{};
  std::vector<std::unique_ptr<lgx_amg_level>> lv;
  lgx::DBuf<double> inv;             // dense inverse of the coarsest matrix
  int64_t stats[32][5] = {};
  uint8_t aggressive[32] = {};       // level aggregated with the aggressive threshold
  uint8_t given[32] = {};            // level took a given aggregate map
  int32_t stop_reason = 0;           // LGX_STOP_* (hierarchy/wright.hpp:26-28)
  lgx::DBuf<double> nat_b, nat_x;    // natural-order staging for lgx_amg_vcycle
  bool f32 = false;
};

