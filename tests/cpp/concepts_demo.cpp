// Drives lineal_gb300 through the C++ concept layer the way lineal's own test
// helpers drive lineal (test/aux/iterative.hpp:25-45): build the operator,
// instantiate ConjugateGradientsSolver with a MultiGridSolver preconditioner,
// and run run_iterative_solver with a caller-side stopping rule.
//
// Output: one line "concepts_demo ok iterations=<k> residual=<r> levels=<L>"
// (exit status 0) or an error message (exit status 1).
#include <cmath>
#include <cstdio>
#include <optional>
#include <random>
#include <vector>

#include "lineal_gb300/lineal.hpp"

namespace lg = lineal::gb300;

static_assert(lg::AnyMatrix<lg::CsrMatrix>);
static_assert(lg::AnyMatrix<lg::StencilMatrix>);
static_assert(lg::AnyVector<lg::DenseVector<double>>);
static_assert(lg::StationaryIterativeSolver<lg::MultiGridSolver>);
static_assert(lg::StationaryIterativeSolver<lg::JacobiSolver>);
static_assert(lg::NonStationaryIterativeSolver<lg::ConjugateGradientsSolver<lg::MultiGridSolver>>);
static_assert(lg::Env<lg::Environment>);

int main() {
  try {
    const lg::Environment env{};
    const int64_t dims[3] = {24, 24, 24};
    const std::size_t n = (std::size_t)(dims[0] * dims[1] * dims[2]);
    std::mt19937_64 rng(1);
    std::normal_distribution<double> normal;
    std::uniform_real_distribution<double> uni(-1.0, 1.0);
    std::vector<double> k(n), b(n);
    for (auto &v : k) v = std::exp(1.5 * normal(rng));
    for (auto &v : b) v = uni(rng);

    lg::DenseVector<double> kd(n, env), rhs(n, env), sol(n, 0.0, env);
    kd.upload(k, env);
    rhs.upload(b, env);
    const auto lhs = lg::CsrMatrix::diffusion_27pt(dims, kd, env);

    lg::MultiGridSolver precon;
    precon.hierarchy.min_coarsen_size = 200;
    precon.aggregation.partition_size = 1024;
    const lg::ConjugateGradientsSolver<lg::MultiGridSolver> solver{precon};

    // test::cg (test/aux/iterative.hpp:25-45) with a relative-residual rule
    double r0 = -1.0;
    std::size_t iters = 0;
    const double res = lg::run_iterative_solver(
      solver, lhs, sol, rhs, env, [&](std::size_t iter, auto &inst, const auto &) {
        const double r = inst.residual_norm();
        if (r0 < 0) r0 = r;
        iters = iter;
        using Out = std::optional<double>;
        return (r <= 1e-8 * r0 || inst.rho() == 0 || iter > 500) ? Out{r / r0} : Out{};
      });

    // FP64 check of the returned solution: ||b - A x|| / ||b||
    lg::DenseVector<double> ax(n, env);
    lg::assign(ax, lhs * sol, env.execution_policy());
    const auto hx = ax.download(env);
    double num = 0, den = 0;
    for (std::size_t i = 0; i < n; ++i) {
      num += (b[i] - hx[i]) * (b[i] - hx[i]);
      den += b[i] * b[i];
    }
    const double true_rel = std::sqrt(num / den);
    auto inst = solver.instantiate(lhs, env);
    const auto levels = inst.amg->level_num();
    // the block/tile-shape autotuner reports two entries per smoothed level
    const auto report = inst.amg->autotune(env, 2);
    bool tuned_ok = report.size() == 2 * (levels - 1);
    for (const auto &e : report) tuned_ok = tuned_ok && e.config >= 0 && e.config < LGX_TUNE_CONFIGS;
    if (!tuned_ok) {
      std::printf("concepts_demo failed: autotune report of %zu entries\n", report.size());
      return 1;
    }
    if (!(res <= 1e-8) || !(true_rel <= 1.1e-8)) {
      std::printf("concepts_demo failed: residual %.3e true %.3e\n", res, true_rel);
      return 1;
    }
    std::printf("concepts_demo ok iterations=%zu residual=%.3e true=%.3e levels=%zu\n", iters, res,
                true_rel, levels);
    return 0;
  } catch (const std::exception &e) {
    std::printf("concepts_demo error: %s\n", e.what());
    return 1;
  }
}
