"""Matrix-free red-black SOR and SSOR on stencil matrices (lookup and value
valuators): every sweep equals the oracle's SOR of the assembled matrix in
the red-black row order bit for bit, and lineal's suite entries sor, ssor1,
sor5, ssor5, pcg_ssor1 and pbicgstab_ssor1 (test/aux/iterative.hpp:115-160)
meet the bound tables of test/shared-stencil.hpp:157-224 on the stencils
themselves, without assembling a matrix."""

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu


def _rb(dims):
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    return ((i + j + k) % 2).ravel().astype(np.int32)


def _pair(cuda, kind, dims, mat=None, seed=3):
    """(GPU stencil, oracle stencil) on a box of unit cells"""
    n = int(np.prod(dims))
    coeffs = (0.0, 1.0, 2.0, 3.0)
    if mat is None:
        mat = np.random.default_rng(seed).integers(0, 4, n).astype(np.uint8)
    box = cuda.BoxInfo(dims, dims)
    if kind == "lookup":
        m = cuda.StencilMatrix.lookup(box, None, coeffs, mat, 1.0, 0.0)
        ref = lo.Stencil(dims, mat=mat, coeffs=coeffs, sol_start=1.0, sol_end=0.0)
    else:
        k = np.asarray(coeffs)[mat]
        m = cuda.StencilMatrix.value(box, None, k, 1.0, 0.0)
        ref = lo.Stencil(dims, k=k, sol_start=1.0, sol_end=0.0)
    return m, ref


@pytest.mark.parametrize("kind", ["lookup", "value"])
@pytest.mark.parametrize("dims", [(4, 9, 7), (6, 5, 8), (1, 5, 3), (7, 1, 6)])
@pytest.mark.parametrize("forward", [True, False])
@pytest.mark.parametrize("ultra", [False, True])
@pytest.mark.parametrize("relax", [1.0, 0.9])
@pytest.mark.parametrize("start", ["zero", "given", "in_situ"])
def test_stencil_sor_sweep_bitexact(cuda, kind, dims, forward, ultra, relax, start):
    m, ref = _pair(cuda, kind, dims)
    csr, _ = ref.to_csr()
    col = cuda.Colouring.red_black(m)
    colours, nc = col.export()
    np.testing.assert_array_equal(colours.cpu().numpy(), _rb(dims))
    assert nc == 2
    order = lo.colour_order(_rb(dims), 2)
    rng = np.random.default_rng(11)
    b = rng.uniform(-1, 1, ref.n)
    x0 = rng.uniform(-1, 1, ref.n)
    want = lo.sor_sweep(csr, b, None if start == "zero" else x0, relax=relax, forward=forward,
                        ultra=ultra, order=order)
    if start == "in_situ":
        x = cuda._dvec(x0).clone()
        got = cuda.sor_sweep(m, col, b, x_in=x, relax=relax, forward=forward, ultra=ultra, out=x)
    else:
        got = cuda.sor_sweep(m, col, b, x_in=None if start == "zero" else x0, relax=relax,
                             forward=forward, ultra=ultra)
    np.testing.assert_array_equal(got.cpu().numpy(), want)


# (entry, sweeps per iteration, symmetric, bound with x = 2, bound with the real rhs)
SWEEP_CASES = [("sor", 1, False, 1e-8, 1e-9), ("ssor1", 1, True, 1e-13, 1.1e-14),
               ("sor5", 5, False, 1e-13, 1e-14), ("ssor5", 5, True, 1e-13, 1.1e-14)]


def _suite_system():
    dims = (4, 9, 7)
    return dims, lo.material_diagonal_lines(dims, 4)


@pytest.mark.parametrize("kind", ["lookup", "value"])
@pytest.mark.parametrize("ultra", [False, True])
@pytest.mark.parametrize("entry,per,sym,bound_x2,bound_rhs", SWEEP_CASES)
def test_stencil_suite_sweep_bounds(cuda, kind, ultra, entry, per, sym, bound_x2, bound_rhs):
    dims, mat = _suite_system()
    m, ref = _pair(cuda, kind, dims, mat)
    csr, _ = ref.to_csr()
    col = cuda.Colouring.red_black(m)
    for rhs_kind in ("x2", "rhs"):
        b = lo.spmv(csr, np.full(ref.n, 2.0)) if rhs_kind == "x2" else ref.rhs()
        x = cuda._dvec(np.zeros(ref.n)).clone()
        for _ in range(129):
            for _ in range(per):
                cuda.sor_sweep(m, col, b, x_in=x, ultra=ultra, out=x)
                if sym:
                    cuda.sor_sweep(m, col, b, x_in=x, forward=False, ultra=ultra, out=x)
        xh = x.cpu().numpy()
        r = lo.spmv(csr, xh) - b
        bound = bound_x2 if rhs_kind == "x2" else bound_rhs
        assert np.linalg.norm(r) <= bound, (entry, rhs_kind, np.linalg.norm(r))
        err = np.abs(xh - 2.0).max() if rhs_kind == "x2" else np.abs(r).max()
        assert err <= bound, (entry, rhs_kind, err)


@pytest.mark.parametrize("kind", ["lookup", "value"])
@pytest.mark.parametrize("fn,bound_x2,bound_rhs", [("pcg", 1e-13, 1e-13),
                                                   ("pbicgstab", 1e-12, 1e-13)])
def test_stencil_suite_ssor_preconditioned_bounds(cuda, kind, fn, bound_x2, bound_rhs):
    dims, mat = _suite_system()
    m, ref = _pair(cuda, kind, dims, mat)
    csr, _ = ref.to_csr()
    solve = getattr(cuda, fn)
    for rhs_kind, bound in (("x2", bound_x2), ("rhs", bound_rhs)):
        b = lo.spmv(csr, np.full(ref.n, 2.0)) if rhs_kind == "x2" else ref.rhs()
        res = solve(m, b, precon=cuda.PRECON_SSOR, rtol=0.0, maxit=129)
        x = res.x.cpu().numpy()
        assert res.history[-1] <= bound
        if rhs_kind == "x2":
            assert np.abs(x - 2.0).max() <= bound
        else:
            assert np.abs(lo.spmv(csr, x) - b).max() <= bound


def test_stencil_ssor_preconditioner_is_the_red_black_pair(cuda):
    """One SSOR preconditioner application (PCG's first direction) equals a
    forward red-black sweep from zero followed by a backward sweep in place,
    as the oracle computes them on the assembled matrix."""
    dims, mat = (6, 7, 8), None
    m, ref = _pair(cuda, "lookup", dims, mat, seed=5)
    csr, _ = ref.to_csr()
    order = lo.colour_order(_rb(dims), 2)
    b = np.random.default_rng(2).uniform(-1, 1, ref.n)
    z = lo.sor_sweep(csr, b, None, order=order)
    z = lo.sor_sweep(csr, b, z, forward=False, order=order)
    res = cuda.pcg(m, b, precon=cuda.PRECON_SSOR, rtol=0.0, maxit=1)
    # x1 = alpha z with alpha = (z.r) / (z.A z): the direction is z
    x = res.x.cpu().numpy()
    alpha = (z @ b) / (z @ lo.spmv(csr, z))
    np.testing.assert_allclose(x, alpha * z, rtol=1e-12, atol=1e-14 * np.abs(x).max())


def test_stencil_colouring_refusals(cuda):
    dims = (4, 5, 6)
    m, ref = _pair(cuda, "lookup", dims)
    csr, _ = ref.to_csr()
    c = cuda.CsrMatrix.from_host(csr.rowptr, csr.col, csr.val)
    with pytest.raises(cuda.LinealError):
        cuda.Colouring.red_black(c)
    jp = cuda.Colouring.jp(c)
    b = np.ones(ref.n)
    with pytest.raises(cuda.LinealError):
        cuda.sor_sweep(m, jp, b)
    rb = cuda.Colouring.red_black(m)
    with pytest.raises(cuda.LinealError):
        cuda.sor_sweep(c, rb, b)
    with pytest.raises(cuda.LinealError):
        cuda.sor_sweep_permuted(rb, b, cuda._dvec(np.zeros(ref.n)).clone())
