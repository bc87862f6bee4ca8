// Drives the direct solvers of the C++ concept layer the way lineal's tests
// drive CholeskySolver and LuSolver (instantiate(lhs, env), then
// solve(sol, rhs, aux, env)): a symmetric positive definite tridiagonal
// system (the matrix of test/python-reference/cholesky.py, n = 32) and a
// nonsymmetric convection-diffusion tridiagonal one, each solved and checked
// on the host against b - A x.
//
// Output: one line "direct_demo ok spd=<r> nonsym=<r>" (exit status 0) or an
// error message (exit status 1).
#include <cmath>
#include <cstdio>
#include <tuple>
#include <vector>

#include "lineal_gb300/lineal.hpp"

namespace lg = lineal::gb300;

static_assert(lg::DirectSolver<lg::CholeskySolver>);
static_assert(lg::DirectSolver<lg::LuSolver>);

namespace {

struct Tridiagonal {
  std::vector<int64_t> rowptr{0};
  std::vector<int32_t> col;
  std::vector<double> val;
};

// rows i: lower a_{i,i-1}, diagonal d, upper a_{i,i+1}
Tridiagonal tridiagonal(int n, double lower, double diag, double upper) {
  Tridiagonal t;
  for (int i = 0; i < n; ++i) {
    if (i > 0) t.col.push_back(i - 1), t.val.push_back(lower);
    t.col.push_back(i), t.val.push_back(diag);
    if (i + 1 < n) t.col.push_back(i + 1), t.val.push_back(upper);
    t.rowptr.push_back((int64_t)t.col.size());
  }
  return t;
}

template <typename TSolver>
double solve_and_check(const Tridiagonal &t, lg::IsSymmetric sym, const lg::Environment &env) {
  const std::size_t n = t.rowptr.size() - 1;
  const auto lhs = lg::CsrMatrix::from_host(t.rowptr, t.col, t.val, sym);
  std::vector<double> b(n);
  for (std::size_t i = 0; i < n; ++i) b[i] = 1.0 + 0.25 * (double)(i % 7);
  lg::DenseVector<double> rhs(n, env), sol(n, 0.0, env);
  rhs.upload(b, env);
  const TSolver solver{};
  const auto inst = solver.instantiate(lhs, env);
  inst.solve(sol, rhs, std::tuple<>{}, env);
  const auto x = sol.download(env);
  double num = 0.0, den = 0.0;
  for (std::size_t i = 0; i < n; ++i) {
    double ax = 0.0;
    for (int64_t e = t.rowptr[i]; e < t.rowptr[i + 1]; ++e) ax += t.val[e] * x[t.col[e]];
    num += (b[i] - ax) * (b[i] - ax);
    den += b[i] * b[i];
  }
  return std::sqrt(num / den);
}

}  // namespace

int main() {
  try {
    const lg::Environment env{};
    const double spd = solve_and_check<lg::CholeskySolver>(tridiagonal(32, -1.0, 2.0, -1.0),
                                                           lg::IsSymmetric{true}, env);
    const double nonsym = solve_and_check<lg::LuSolver>(tridiagonal(200, -1.3, 2.0, -0.7),
                                                        lg::IsSymmetric{false}, env);
    // symmetric indefinite (pivots 0.5, -1.5, ...): LuSolver solves it,
    // CholeskySolver refuses it with LGX_ERR_NOT_SPD
    const Tridiagonal indefinite = tridiagonal(8, -1.0, 0.5, -1.0);
    const double indef = solve_and_check<lg::LuSolver>(indefinite, lg::IsSymmetric{true}, env);
    lgx_status refused = LGX_OK;
    try {
      (void)solve_and_check<lg::CholeskySolver>(indefinite, lg::IsSymmetric{true}, env);
    } catch (const lg::Error &e) {
      refused = e.status;
    }
    // relative residuals of an explicit inverse: about cond(A) * eps (cond
    // 441, 839 and 16 here), so 1e-12 leaves a margin
    if (!(spd <= 1e-12) || !(nonsym <= 1e-12) || !(indef <= 1e-12) ||
        refused != LGX_ERR_NOT_SPD) {
      std::printf("direct_demo failed: spd %.3e nonsym %.3e indefinite %.3e refused %d\n", spd,
                  nonsym, indef, (int)refused);
      return 1;
    }
    std::printf("direct_demo ok spd=%.3e nonsym=%.3e indefinite=%.3e\n", spd, nonsym, indef);
    return 0;
  } catch (const std::exception &e) {
    std::printf("direct_demo error: %s\n", e.what());
    return 1;
  }
}
