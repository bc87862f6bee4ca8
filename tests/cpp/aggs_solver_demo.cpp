// MultiGridSolver with lineal's aggregate-map file options: a hierarchy
// written through AggregationParams::base_agg_map_path (RefinedAggregator,
// aggregation/independent.hpp:243-272) and rebuilt through
// file_agg_map_path (FileAggregator, 279-298) with other partitioning
// parameters applies the same V-cycle bit for bit.
//
// Usage: aggs_solver_demo <base>.  Output: "aggs_solver_demo ok levels=<L>"
// (exit status 0) or the failure (exit status 1).
#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "lineal_gb300/lineal.hpp"

namespace lg = lineal::gb300;

int main(int argc, char **argv) {
  if (argc != 2) return 2;
  try {
    const lg::Environment env{};
    const int64_t dims[3] = {12, 14, 16};
    const std::size_t n = 12 * 14 * 16;
    std::mt19937_64 rng(3);
    std::normal_distribution<double> normal;
    std::uniform_real_distribution<double> uni(-1.0, 1.0);
    std::vector<double> k(n), b(n);
    for (auto &v : k) v = std::exp(1.5 * normal(rng));
    for (auto &v : b) v = uni(rng);
    lg::DenseVector<double> kd(n, env), rhs(n, env), x1(n, env), x2(n, env);
    kd.upload(k, env);
    rhs.upload(b, env);
    const auto lhs = lg::CsrMatrix::diffusion_27pt(dims, kd, env);

    lg::MultiGridSolver writer;
    writer.hierarchy.min_coarsen_size = 64;
    writer.aggregation.partition_size = 512;
    writer.aggregation.base_agg_map_path = std::string(argv[1]);
    const auto first = writer.instantiate(lhs, env);

    lg::MultiGridSolver reader;
    reader.hierarchy.min_coarsen_size = 64;
    reader.aggregation.partition_size = 1 << 24;  // its own aggregation would differ
    reader.file_agg_map_path = std::string(argv[1]);
    const auto second = reader.instantiate(lhs, env);

    first.apply(x1, rhs, env);
    second.apply(x2, rhs, env);
    const auto h1 = x1.download(env), h2 = x2.download(env);
    const std::size_t levels = first.level_num();
    if (levels != second.level_num() || levels < 3 || h1 != h2) {
      std::printf("aggs_solver_demo failed: levels %zu / %zu, cycles %s\n", levels,
                  second.level_num(), h1 == h2 ? "equal" : "differ");
      return 1;
    }
    for (std::size_t l = 0; l + 1 < levels; ++l) {
      const auto a = first.aggregate_map(l, env), c = second.aggregate_map(l, env);
      const auto f = lg::read_aggs(lg::aggs_path(argv[1], l));
      if (a.agg != c.agg || a.list != c.list || a.list != f.list || a.agg != f.agg) {
        std::printf("aggs_solver_demo failed: level %zu maps differ\n", l);
        return 1;
      }
    }
    std::printf("aggs_solver_demo ok levels=%zu\n", levels);
    return 0;
  } catch (const std::exception &e) {
    std::printf("aggs_solver_demo error: %s\n", e.what());
    return 1;
  }
}
