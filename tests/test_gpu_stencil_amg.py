"""AMG with a matrix-free finest level: a hierarchy built on a stencil
matrix assembles the finest matrix only for its setup, then smooths (red-
black SOR) and forms residuals on the stencil itself.  Levels and V-cycles
agree with the oracle's hierarchy on the assembled matrix in red-black
order, and lineal's pcg_amg / pbicgstab_amg suite entries
(test/aux/iterative.hpp:162-181) meet their bound tables on the stencils."""

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu


def _rb(dims):
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    return ((i + j + k) % 2).ravel().astype(np.int32)


def _lookup(cuda, dims, mat, coeffs=(0.5, 1.0, 2.0, 3.0)):
    m = cuda.StencilMatrix.lookup(cuda.BoxInfo(dims, dims), None, coeffs, mat, 1.0, 0.0)
    ref = lo.Stencil(dims, mat=mat, coeffs=coeffs, sol_start=1.0, sol_end=0.0)
    return m, ref


def _value(cuda, dims, k):
    m = cuda.StencilMatrix.value(cuda.BoxInfo(dims, dims), None, k, 1.0, 0.0)
    ref = lo.Stencil(dims, k=k, sol_start=1.0, sol_end=0.0)
    return m, ref


PARAMS = dict(min_coarsen_size=64, partition_size=512)


@pytest.mark.parametrize("kind", ["lookup", "value"])
@pytest.mark.parametrize("dims", [(12, 11, 10), (9, 16, 7)])
def test_stencil_hierarchy_and_vcycle_match_oracle(cuda, kind, dims):
    n = int(np.prod(dims))
    rng = np.random.default_rng(4)
    if kind == "lookup":
        m, ref = _lookup(cuda, dims, rng.integers(0, 4, n).astype(np.uint8))
    else:
        m, ref = _value(cuda, dims, np.exp(1.5 * rng.standard_normal(n)))
    csr, _ = ref.to_csr()
    h = cuda.HierarchyWright(**PARAMS).instantiate(m)
    oh = lo.Amg(csr, finest_colours=_rb(dims), ncolours=2, smoother_parts=0, **PARAMS)
    rows, _ = h.sizes()
    assert rows == [oh.level_size(l) for l in range(oh.nlevels)]
    assert len(rows) >= 3
    b = rng.uniform(-1, 1, n)
    got = h.vcycle(b).cpu().numpy()
    want = oh.vcycle(b)
    # same aggregation, level matrices and colour orders; the finest residual
    # sums the stencil row in its own order and the coarsest solve is a dense
    # inverse on the GPU
    assert np.abs(got - want).max() <= 1e-11 * np.abs(want).max()


def test_stencil_amg_pcg_matches_oracle_iterations(cuda):
    dims = (24, 22, 20)
    n = int(np.prod(dims))
    m, ref = _value(cuda, dims, np.exp(1.5 * np.random.default_rng(1).standard_normal(n)))
    csr, _ = ref.to_csr()
    b = np.random.default_rng(0).uniform(-1, 1, n)
    h = cuda.HierarchyWright(**PARAMS).instantiate(m)
    res = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=1e-8, maxit=300)
    oh = lo.Amg(csr, finest_colours=_rb(dims), ncolours=2, smoother_parts=0, **PARAMS)
    _, it, hist = lo.pcg(csr, b, precon=lo.PRECON_AMG, amg=oh, rtol=1e-8, maxit=300)
    x = res.x.cpu().numpy()
    assert np.linalg.norm(b - lo.spmv(csr, x)) <= 1.01e-8 * np.linalg.norm(b)
    assert abs(res.iterations - it) <= max(1, int(0.05 * it + 0.999))
    np.testing.assert_allclose(res.history[:5], hist[:5], rtol=1e-9)


# bounds of test/shared-stencil.hpp:157-224 (x = 2 / real rhs), 33 iterations
@pytest.mark.parametrize("kind", ["lookup", "value"])
@pytest.mark.parametrize("fn,bound_x2,bound_rhs", [("pcg", 1e-13, 2e-14),
                                                   ("pbicgstab", 1e-13, 1e-13)])
def test_stencil_suite_amg_bounds(cuda, kind, fn, bound_x2, bound_rhs):
    dims = (4, 9, 7)
    mat = lo.material_diagonal_lines(dims, 4)
    coeffs = (0.0, 1.0, 2.0, 3.0)
    if kind == "lookup":
        m, ref = _lookup(cuda, dims, mat, coeffs)
    else:
        m, ref = _value(cuda, dims, np.asarray(coeffs)[mat])
    csr, _ = ref.to_csr()
    h = cuda.HierarchyWright(min_coarsen_size=32, partition_size=126,
                             coarse_f32=True).instantiate(m)
    solve = getattr(cuda, fn)
    b2 = lo.spmv(csr, np.full(ref.n, 2.0))
    res = solve(m, b2, precon=cuda.PRECON_AMG, amg=h, rtol=0.0, maxit=33)
    x = res.x.cpu().numpy()
    assert res.history[-1] <= bound_x2 and np.abs(x - 2).max() <= bound_x2
    b = ref.rhs()
    res = solve(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=0.0, maxit=33)
    x = res.x.cpu().numpy()
    assert res.history[-1] <= bound_rhs and np.abs(lo.spmv(csr, x) - b).max() <= bound_rhs


def test_stencil_hierarchy_refusals(cuda):
    dims = (8, 8, 8)
    m, ref = _lookup(cuda, dims, np.ones(512, dtype=np.uint8))
    with pytest.raises(cuda.LinealError):
        cuda.HierarchyWright(cycle_f32=True, **PARAMS).instantiate(m)
    h = cuda.HierarchyWright(min_coarsen_size=16, partition_size=64).instantiate(m)
    with pytest.raises(cuda.LinealError):
        h.level(0)
    csr, _ = ref.to_csr()
    c = cuda.CsrMatrix.from_host(csr.rowptr, csr.col, csr.val)
    with pytest.raises(cuda.LinealError):
        cuda.pcg(c, np.ones(512), precon=cuda.PRECON_AMG, amg=h)
