// Aggregate-map files from the C++ concept layer (write_aggs / read_aggs /
// read_aggregates, the files of lineal's RefinedAggregator and
// FileAggregator, aggregation/independent.hpp:237-298), host side only: no
// device work, so it runs without a GPU.
//
//   aggs_io_demo write <base>  writes <base>0.aggs and <base>1.aggs
//   aggs_io_demo read <base>   reads <base>0.aggs, <base>1.aggs, ... and prints
//                              per level "level <k> n <n> nc <nc> sum <s>",
//                              s = sum over agg + 3 * sum over lists
//   aggs_io_demo refuse <path> exits 0 when reading <path> throws
#include <cstdio>
#include <string>

#include "lineal_gb300/lineal.hpp"

namespace lg = lineal::gb300;

namespace {

// 10 fine vertices in 3 aggregates (lists in aggregation order), vertex 4
// isolated; then the 3 coarse vertices in one aggregate
lg::AggregateMap level0() {
  lg::AggregateMap m;
  m.agg = {1, 1, 0, 0, 0xFFFFFFFEu, 2, 2, 0, 1, 2};
  m.list_ptr = {0, 3, 6, 9};
  m.list = {3, 2, 7, 8, 0, 1, 9, 5, 6};
  return m;
}
lg::AggregateMap level1() {
  lg::AggregateMap m;
  m.agg = {0, 0, 0};
  m.list_ptr = {0, 3};
  m.list = {1, 0, 2};
  return m;
}

long long checksum(const lg::AggregateMap &m) {
  long long s = 0;
  for (auto v : m.agg) s += v;
  for (auto v : m.list) s += 3LL * v;
  return s;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  const std::string mode = argv[1], path = argv[2];
  try {
    if (mode == "write") {
      lg::write_aggs(lg::aggs_path(path, 0), level0());
      lg::write_aggs(lg::aggs_path(path, 1), level1());
      return 0;
    }
    if (mode == "read") {
      const auto maps = lg::read_aggregates(path);
      for (std::size_t k = 0; k < maps.size(); ++k)
        std::printf("level %zu n %zu nc %zu sum %lld\n", k, maps[k].agg.size(),
                    maps[k].list_ptr.size() - 1, checksum(maps[k]));
      return 0;
    }
    if (mode == "refuse") {
      try {
        (void)lg::read_aggs(path);
      } catch (const lg::Error &e) {
        std::printf("refused: %s\n", e.what());
        return 0;
      }
      return 1;
    }
  } catch (const std::exception &e) {
    std::printf("aggs_io_demo error: %s\n", e.what());
    return 1;
  }
  return 2;
}
