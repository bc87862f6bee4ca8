"""Blocked multi-right-hand-side AMG-PCG (batching form): every column of a
32-column block reaches the tolerance, verified in FP64 on the oracle, in
the iteration count of its own single-vector solve."""

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu

PARAMS = dict(min_coarsen_size=64, partition_size=512)


def _case(dims=(18, 17, 16), seed=5):
    n = int(np.prod(dims))
    k = np.exp(1.5 * np.random.default_rng(seed).standard_normal(n))
    return lo.gen_27pt(dims, k), k


@pytest.mark.parametrize("cycle_f32", [False, True])
@pytest.mark.parametrize("nrhs", [1, 5, 32])
def test_blocked_pcg_matches_single_solves(cuda, cycle_f32, nrhs):
    import torch

    dims = (18, 17, 16)
    ref, k = _case(dims)
    m = cuda.gen_27pt(dims, k)
    h = cuda.HierarchyWright(cycle_f32=cycle_f32, **PARAMS).instantiate(m)
    B = np.random.default_rng(nrhs).uniform(-1, 1, (ref.n, nrhs))
    X, its, rels = cuda.pcg_multi(m, h, B, rtol=1e-8, maxit=500)
    Xh = X.cpu().numpy()
    for c in range(nrhs):
        single = cuda.pcg(m, B[:, c], precon=cuda.PRECON_AMG, amg=h, rtol=1e-8, maxit=500)
        assert rels[c] <= 1e-8
        assert abs(int(its[c]) - single.iterations) <= max(1, int(0.05 * single.iterations + 0.999))
        r = B[:, c] - lo.spmv(ref, Xh[:, c])
        assert np.linalg.norm(r) <= 1.1e-8 * np.linalg.norm(B[:, c])
        xs = single.x.cpu().numpy()
        assert np.linalg.norm(Xh[:, c] - xs) <= 1e-6 * np.linalg.norm(xs)


def test_blocked_pcg_initial_guess_and_errors(cuda):
    dims = (10, 9, 8)
    ref, k = _case(dims, seed=6)
    m = cuda.gen_27pt(dims, k)
    h = cuda.HierarchyWright(**PARAMS).instantiate(m)
    B = np.random.default_rng(1).uniform(-1, 1, (ref.n, 3))
    X, its, _ = cuda.pcg_multi(m, h, B, rtol=1e-10)
    # a start at the solution stays there
    X2, _, _ = cuda.pcg_multi(m, h, B, x0=X, rtol=1e-2)
    x1, x2 = X.cpu().numpy(), X2.cpu().numpy()
    assert np.linalg.norm(x2 - x1) <= 1e-8 * np.linalg.norm(x1)
    with pytest.raises(cuda.LinealError):
        cuda.pcg_multi(m, h, np.zeros((ref.n, 33)))
    other = cuda.gen_27pt(dims, k)
    with pytest.raises(cuda.LinealError):
        cuda.pcg_multi(other, h, B)


@pytest.mark.parametrize("cycle_f32", [False, True])
def test_blocked_pcg_graph_replay_bitexact(cuda, cycle_f32):
    """The captured iteration replays exactly what the eager loop launches."""
    dims = (16, 15, 14)
    ref, k = _case(dims, seed=8)
    m = cuda.gen_27pt(dims, k)
    h = cuda.HierarchyWright(cycle_f32=cycle_f32, **PARAMS).instantiate(m)
    B = np.random.default_rng(9).uniform(-1, 1, (ref.n, 7))
    Xg, itg, relg = cuda.pcg_multi(m, h, B, rtol=1e-9, use_graphs=True)
    Xe, ite, rele = cuda.pcg_multi(m, h, B, rtol=1e-9, use_graphs=False)
    # past 8 iterations both graph variants (with and without the residual
    # recomputation) have replayed
    assert itg.min() > 8
    np.testing.assert_array_equal(itg, ite)
    np.testing.assert_array_equal(relg, rele)
    np.testing.assert_array_equal(Xg.cpu().numpy(), Xe.cpu().numpy())
