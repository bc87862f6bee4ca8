// Host element access of the C++ concept layer: DenseVector's operator[],
// compute and store (dense/vector/shared.hpp:268-310) and the ConstRow
// interface of a CSR matrix's rows (csr/shared.hpp:120-333) on a host
// snapshot, against the host arrays the matrix was built from.
//
// Output: one line "access_demo ok" (exit status 0) or the first mismatch
// (exit status 1).
#include <cstdio>
#include <optional>
#include <random>
#include <stdexcept>
#include <vector>

#include "lineal_gb300/lineal.hpp"

namespace lg = lineal::gb300;

namespace {

int fail(const char *what) {
  std::printf("access_demo failed: %s\n", what);
  return 1;
}

}  // namespace

int main() {
  try {
    const lg::Environment env{};
    // a nonsymmetric band matrix with a stored diagonal, 64 rows
    const int64_t n = 64;
    std::vector<int64_t> rowptr{0};
    std::vector<int32_t> col;
    std::vector<double> val;
    std::mt19937_64 rng(3);
    std::uniform_real_distribution<double> uni(-1.0, 1.0);
    for (int64_t i = 0; i < n; ++i) {
      for (int64_t j = i - 2; j <= i + 3; ++j) {
        if (j < 0 || j >= n || (j == i + 1 && i % 3 == 0)) continue;
        col.push_back((int32_t)j);
        val.push_back(j == i ? 8.0 + uni(rng) : uni(rng));
      }
      rowptr.push_back((int64_t)col.size());
    }
    const auto m = lg::CsrMatrix::from_host(rowptr, col, val, lg::IsSymmetric{false});
    const auto h = lg::HostCsr::download(m, env);
    if (h.row_num() != (std::size_t)n || h.non_zero_num() != col.size()) return fail("sizes");
    if (h.row_offsets() != rowptr || h.column_indices() != col || h.entries() != val)
      return fail("arrays");
    for (int64_t i = 0; i < n; ++i) {
      const auto row = h[(std::size_t)i];
      const auto len = (std::size_t)(rowptr[i + 1] - rowptr[i]);
      if (row.index() != (std::size_t)i || row.size() != len) return fail("row size");
      if (row.offdiagonal_num() != len - 1) return fail("offdiagonal_num");
      const auto cols = row.column_indices();
      for (std::size_t k = 0; k < len; ++k) {
        const int32_t c = col[(std::size_t)rowptr[i] + k];
        if (cols[k] != c) return fail("column indices");
        if (row[c] != val[(std::size_t)rowptr[i] + k]) return fail("value by column");
        if (!row.find(c) || *row.find(c) != k) return fail("find");
      }
      if (row.contains((int32_t)(i + 5)) || row.find((int32_t)(i + 5))) return fail("absent");
      if (row.diagonal() != h.diagonal_at((std::size_t)i) ||
          h.entry_at((std::size_t)i, (int32_t)i) != row[(int32_t)i])
        return fail("diagonal");
      // off-diagonal positions skip the diagonal
      std::size_t off = 0;
      for (std::size_t q = 0; q < len; ++q) {
        const int32_t c = col[(std::size_t)rowptr[i] + q];
        if (c == i) continue;
        if (row.offdiagonal_index_within(c) != off++) return fail("offdiagonal_index_within");
      }
      // the full walk in column order
      std::size_t k = 0;
      bool ordered = true;
      row.iterate([&](int32_t c, double v) {
        ordered = ordered && c == col[(std::size_t)rowptr[i] + k] &&
                  v == val[(std::size_t)rowptr[i] + k];
        ++k;
      });
      if (!ordered || k != len) return fail("iterate");
      // split around the diagonal
      std::size_t nb = 0, nd = 0, na = 0;
      double diag = 0.0;
      row.iterate([&](int32_t c, double) { nb += c < i; },
                  [&](int32_t, double v) {
                    ++nd;
                    diag = v;
                  },
                  [&](int32_t c, double) { na += c > i; });
      std::size_t wb = 0, wa = 0;
      for (std::size_t q = 0; q < len; ++q) {
        wb += col[(std::size_t)rowptr[i] + q] < i;
        wa += col[(std::size_t)rowptr[i] + q] > i;
      }
      if (nb != wb || nd != 1 || na != wa || diag != row[(int32_t)i]) return fail("split walk");
      // a valued return ends the walk: the first column right of the diagonal
      const auto first_after = row.iterate([&](int32_t c, double) -> std::optional<int32_t> {
        if (c > i) return c;
        return std::nullopt;
      });
      std::optional<int32_t> want;
      for (std::size_t q = 0; q < len && !want; ++q)
        if (col[(std::size_t)rowptr[i] + q] > i) want = col[(std::size_t)rowptr[i] + q];
      if (first_after != want) return fail("valued return");
    }
    bool threw = false;
    try {
      (void)h[(std::size_t)n];
    } catch (const std::out_of_range &) {
      threw = true;
    }
    if (!threw) return fail("row range");

    // vector elements
    lg::DenseVector<double> v(10, 1.5, env);
    v[3] = 2.25;
    v.store(7, -4.0, env);
    const lg::DenseVector<double> &cv = v;
    if (cv[3] != 2.25 || v.compute(7, env) != -4.0 || cv[0] != 1.5) return fail("elements");
    v[2] = v[3];
    const auto all = v.download(env);
    const std::vector<double> want{1.5, 1.5, 2.25, 2.25, 1.5, 1.5, 1.5, -4.0, 1.5, 1.5};
    if (all != want) return fail("element writes");
    threw = false;
    try {
      (void)cv[10];
    } catch (const std::out_of_range &) {
      threw = true;
    }
    if (!threw) return fail("element range");
    std::printf("access_demo ok\n");
    return 0;
  } catch (const std::exception &e) {
    std::printf("access_demo failed: %s\n", e.what());
    return 1;
  }
}
