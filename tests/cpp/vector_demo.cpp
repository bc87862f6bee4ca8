// The free vector operations of the C++ concept layer (component-wise/
// vector-expression.hpp: add, subtract, scale, operator+ - *, constant,
// constant_like; sink/swap.hpp: swap; sink/accumulator.hpp: multiconsume
// with its consumers) against host arithmetic with lineal's rounding: every
// product and every sum rounded on its own; and the aux-tuple call shapes of
// the stationary solvers (iterative-stationary/broom.hpp:36-51).
//
// Output: one line "vector_demo ok" (exit status 0) or the first mismatch
// (exit status 1).
#include <cmath>
#include <cstdio>
#include <functional>
#include <random>
#include <tuple>
#include <vector>

#include "lineal_gb300/lineal.hpp"

namespace lg = lineal::gb300;

namespace {

// the bits lineal computes for s1 * x + s2 * y (volatile: no contraction)
double lincomb(double s1, double x, double s2, double y) {
  volatile double p = s1 * x;
  volatile double q = s2 * y;
  volatile double r = p + q;
  return r;
}

bool same(const std::vector<double> &got, const std::function<double(std::size_t)> &want,
          const char *what) {
  for (std::size_t i = 0; i < got.size(); ++i) {
    if (got[i] != want(i)) {
      std::printf("vector_demo failed: %s at %zu: %.17g != %.17g\n", what, i, got[i], want(i));
      return false;
    }
  }
  return true;
}

}  // namespace

int main() {
  try {
    const lg::Environment env{};
    const auto pol = env.execution_policy();
    const std::size_t n = 100003;
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> uni(-3.0, 3.0);
    std::vector<double> a(n), b(n);
    for (auto &v : a) v = uni(rng);
    for (auto &v : b) v = uni(rng);
    lg::DenseVector<double> da(n, env), db(n, env), out(n, env);
    da.upload(a, env);
    db.upload(b, env);
    const double s = 0.7071067811865476, t = -1.25e-3;
    bool ok = true;

    lg::assign(out, da + db, pol);
    ok = ok && same(out.download(env), [&](std::size_t i) { return a[i] + b[i]; }, "a + b");
    lg::assign(out, lg::subtract(da, db), pol);
    ok = ok && same(out.download(env), [&](std::size_t i) { return a[i] - b[i]; }, "a - b");
    lg::assign(out, s * da, pol);
    ok = ok && same(out.download(env), [&](std::size_t i) { return lincomb(s, a[i], 0, 0); },
                    "s * a");
    lg::assign(out, da - db * s, pol);
    ok = ok && same(out.download(env), [&](std::size_t i) { return lincomb(1, a[i], -s, b[i]); },
                    "a - b s");
    lg::assign(out, lg::add(lg::scale(da, s), t * db), pol);
    ok = ok && same(out.download(env), [&](std::size_t i) { return lincomb(s, a[i], t, b[i]); },
                    "s a + t b");
    // in place: out = out + a
    lg::assign(out, out + da, pol);
    ok = ok && same(out.download(env),
                    [&](std::size_t i) {
                      volatile double r = lincomb(s, a[i], t, b[i]) + a[i];
                      return (double)r;
                    },
                    "out + a");
    lg::assign(out, lg::constant_like(out, -2.5), pol);
    ok = ok && same(out.download(env), [](std::size_t) { return -2.5; }, "constant");

    // swap exchanges the contents
    lg::swap(da, db, pol);
    ok = ok && same(da.download(env), [&](std::size_t i) { return b[i]; }, "swap");
    lg::swap(da, db, pol);

    // multiconsume = the single reductions
    const auto [d, e2, en, mx] = lg::multiconsume(
      std::tuple{lg::dot_consumer<double, 0, 1>(), lg::euclidean_squared_consumer<double, 1>(),
                 lg::euclidean_norm_consumer<double, 0>(), lg::max_norm_consumer<double, 1>()},
      std::tie(da, db), pol);
    if (d != lg::dot(da, db, pol) || e2 != lg::euclidean_squared(db, pol) ||
        en != lg::euclidean_norm(da, pol) || mx != lg::max_norm(db, pol)) {
      std::printf("vector_demo failed: multiconsume\n");
      ok = false;
    }
    double maxb = 0.0;
    for (double v : b) maxb = std::fmax(maxb, std::fabs(v));
    if (mx != maxb) {
      std::printf("vector_demo failed: max_norm %.17g != %.17g\n", mx, maxb);
      ok = false;
    }
    // sizes must agree
    bool refused = false;
    try {
      lg::DenseVector<double> small(n - 1, env);
      lg::assign(small, da + db, pol);
    } catch (const lg::Error &) {
      refused = true;
    }
    // lineal's stationary-solver call shapes with an aux tuple (broom.hpp:
    // 36-51): in situ equals ex situ bit for bit, and aux receives the old
    // solution; MultiGridSolver from constant_like(out, 0)
    {
      const int64_t dims[3] = {8, 8, 8};
      const std::size_t m = 512;
      std::vector<double> k(m), x0(m), rb(m);
      for (auto &v : k) v = std::exp(uni(rng));
      for (auto &v : x0) v = uni(rng);
      for (auto &v : rb) v = uni(rng);
      lg::DenseVector<double> kd(m, env), rhs(m, env), in(m, env), ex(m, env), sol(m, env),
        tmp(m, env);
      kd.upload(k, env);
      rhs.upload(rb, env);
      in.upload(x0, env);
      const auto lhs = lg::CsrMatrix::diffusion_27pt(dims, kd, env);
      auto check_shapes = [&](const auto &inst, const char *what) {
        inst.apply(in, ex, rhs, std::tuple<>{}, env);
        sol.upload(x0, env);
        inst.apply(sol, rhs, std::tie(tmp), env);
        const auto want = ex.download(env);
        ok = ok && same(sol.download(env), [&](std::size_t i) { return want[i]; }, what);
        ok = ok && same(tmp.download(env), [&](std::size_t i) { return x0[i]; }, what);
      };
      check_shapes(lg::JacobiSolver{0.8}.instantiate(lhs, env), "jacobi in situ");
      check_shapes(lg::SorSolver<lg::forward_tag_t>{1.0}.instantiate(lhs, env), "sor in situ");
      lg::MultiGridSolver mg;
      mg.hierarchy.min_coarsen_size = 20;
      const auto amg = mg.instantiate(lhs, env);
      amg.apply(lg::constant_like(ex, 0.0), ex, rhs, std::tuple<>{}, env);
      amg.apply(sol, rhs, env);
      const auto want = sol.download(env);
      ok = ok && same(ex.download(env), [&](std::size_t i) { return want[i]; }, "amg apply");
      bool nonzero_refused = false;
      try {
        amg.apply(lg::constant_like(ex, 1.0), ex, rhs, std::tuple<>{}, env);
      } catch (const lg::Error &) {
        nonzero_refused = true;
      }
      ok = ok && nonzero_refused;
    }
    if (!ok || !refused) return 1;
    std::printf("vector_demo ok\n");
    return 0;
  } catch (const std::exception &e) {
    std::printf("vector_demo error: %s\n", e.what());
    return 1;
  }
}
