"""Batching form: many upwind convection-diffusion systems of uneven sizes
solved by Jacobi-BiCGStab in one persistent launch, each checked against the
oracle's BiCGStab on the assembled CSR (iteration count within 5 %,
FP64-verified residual)."""

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu


def _systems(count, lo_edge, hi_edge, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        dims = tuple(int(e) for e in rng.integers(lo_edge, hi_edge + 1, 3))
        v = tuple(float(c) for c in rng.uniform(-20.0, 20.0, 3))
        out.append((dims, v))
    return out


def test_batch_matches_oracle_per_system(cuda):
    systems = _systems(24, 3, 14) + [((1, 5, 7), (0.0, 20.0, -20.0))]
    rng = np.random.default_rng(11)
    bs = [rng.uniform(-1, 1, int(np.prod(d))) for d, _ in systems]
    res = cuda.batch_convdiff_bicgstab(systems, np.concatenate(bs), rtol=1e-8, maxit=1000)
    assert (res.status == 0).all(), res.status
    x = res.x.cpu().numpy()
    off = 0
    for s, ((dims, v), b) in enumerate(zip(systems, bs)):
        n = b.size
        a = lo.gen_convdiff(dims, v)
        xs = x[off:off + n]
        off += n
        _, it, _ = lo.pbicgstab(a, b, precon=lo.PRECON_JACOBI, rtol=1e-8, maxit=1000)
        assert abs(int(res.iterations[s]) - it) <= max(1, int(0.05 * it + 0.999)), (s, dims)
        assert res.rel_residual[s] <= 1e-8
        assert np.linalg.norm(b - lo.spmv(a, xs)) <= 1.1e-8 * np.linalg.norm(b), (s, dims)


def test_batch_initial_guess_and_empty(cuda):
    systems = _systems(5, 6, 9, seed=4)
    n = sum(int(np.prod(d)) for d, _ in systems)
    b = np.random.default_rng(2).uniform(-1, 1, n)
    first = cuda.batch_convdiff_bicgstab(systems, b, rtol=1e-10)
    # a start at half the solution converges to the same solutions
    again = cuda.batch_convdiff_bicgstab(systems, b, x0=0.5 * first.x, rtol=1e-10)
    assert (first.status == 0).all() and (again.status == 0).all()
    x1, x2 = first.x.cpu().numpy(), again.x.cpu().numpy()
    assert np.linalg.norm(x2 - x1) <= 1e-7 * np.linalg.norm(x1)
    empty = cuda.batch_convdiff_bicgstab([], np.zeros(0))
    assert empty.iterations.size == 0


def test_batch_exact_alpha_step(cuda):
    """A 1x1x1 system is solved (to rounding) by the first alpha step; the
    batch reports it converged with x = b / a_11 (the reference's omega would
    be 0 / 0 there when the step is exact)."""
    systems = [((1, 1, 1), (5.0, -3.0, 0.0)), ((6, 7, 8), (1.0, 2.0, 3.0))]
    b = np.random.default_rng(8).uniform(-1, 1, 1 + 336)
    res = cuda.batch_convdiff_bicgstab(systems, b, rtol=1e-8)
    assert (res.status == 0).all()
    diag = lo.gen_convdiff((1, 1, 1), (5.0, -3.0, 0.0)).val[0]
    assert abs(res.x.cpu().numpy()[0] - b[0] / diag) <= 4e-16 * abs(b[0] / diag)
    assert res.iterations[0] <= 2
