"""The AMG option coarse_smallest_last (levels >= 1 coloured on the host by
lgx_colour_smallest_last) against the oracle's AMG with the same option:
V-cycle within 1e-11 and AMG-PCG iterations as the oracle's; and a
standalone smallest-last colouring driving the multicolour SOR sweep."""

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu

PARAMS = dict(min_coarsen_size=64, partition_size=512, max_partitions=1 << 30)


def _case(dims=(14, 15, 16), seed=1):
    n = int(np.prod(dims))
    k = np.exp(1.5 * np.random.default_rng(seed).standard_normal(n))
    return lo.gen_27pt(dims, k), k


def test_coarse_smallest_last_matches_oracle(cuda):
    ref, _ = _case()
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    h = cuda.HierarchyWright(coarse_smallest_last=True, **PARAMS).instantiate(m)
    oh = lo.Amg(ref, smoother_parts=0, coarse_smallest_last=1, **PARAMS)
    assert h.level_num() == oh.nlevels >= 3
    b = np.random.default_rng(3).uniform(-1, 1, ref.n)
    got = h.vcycle(b).cpu().numpy()
    want = oh.vcycle(b)
    assert np.abs(got - want).max() <= 1e-11 * np.abs(want).max()
    # the option changes the cycle (other colour orders on the coarse levels)
    plain = cuda.HierarchyWright(**PARAMS).instantiate(m).vcycle(b).cpu().numpy()
    assert not np.array_equal(plain, got)
    res = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=1e-8, maxit=300)
    _, it, hist = lo.pcg(ref, b, precon=lo.PRECON_AMG, amg=oh, rtol=1e-8, maxit=300)
    assert res.rel_residual <= 1e-8
    assert abs(res.iterations - it) <= max(1, int(0.05 * it + 0.999))
    np.testing.assert_allclose(res.history[:5], hist[:5], rtol=1e-9)


def test_standalone_smallest_last_sweep(cuda):
    ref, _ = _case((10, 11, 12), 5)
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    colour, nc = cuda.colour_smallest_last(ref.rowptr, ref.col)
    col = cuda.Colouring.from_array(m, colour, nc)
    rng = np.random.default_rng(6)
    b, x0 = rng.uniform(-1, 1, ref.n), rng.uniform(-1, 1, ref.n)
    x = cuda.sor_sweep(m, col, b, x_in=x0).cpu().numpy()
    want = lo.sor_sweep(ref, b, x_in=x0, order=lo.colour_order(colour, nc))
    np.testing.assert_allclose(x, want, rtol=1e-13, atol=1e-13)
