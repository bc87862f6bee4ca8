"""The finest level of a parity-coloured 27-point grid matrix runs kernels
that compute column indices from the grid: V-cycles and AMG-PCG solves must
equal the CSR kernels' bit for bit, in every precision form, and the grid
path must stay off wherever the structure does not hold."""

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu

PARAMS = dict(min_coarsen_size=64, partition_size=512, max_partitions=1 << 30)
FORMS = {"fp64": {}, "f32": dict(cycle_f32=True), "bf16": dict(cycle_f32=True, cycle_bf16=True),
         "f32_coarse": dict(coarse_f32=True, cycle_f32=True)}


def _parity(dims):
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    return ((i % 2) * 4 + (j % 2) * 2 + (k % 2)).ravel().astype(np.int32)


def _k(dims, seed=3):
    return np.exp(1.5 * np.random.default_rng(seed).standard_normal(int(np.prod(dims))))


def _pair(cuda, m, dims, **kw):
    col = cuda.Colouring.from_array(m, _parity(dims), 8)
    hg = cuda.HierarchyWright(grid27=True, **PARAMS, **kw).instantiate(m, finest_colouring=col)
    hc = cuda.HierarchyWright(grid27=False, **PARAMS, **kw).instantiate(m, finest_colouring=col)
    return hg, hc


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("dims", [(8, 10, 12), (16, 16, 16), (2, 4, 6)])
def test_grid_vcycle_equals_csr(cuda, form, dims):
    m = cuda.gen_27pt(dims, _k(dims))
    hg, hc = _pair(cuda, m, dims, **FORMS[form])
    assert hg.grid27_active() and not hc.grid27_active()
    b = np.random.default_rng(5).uniform(-1, 1, m.row_num())
    np.testing.assert_array_equal(hg.vcycle(b).cpu().numpy(), hc.vcycle(b).cpu().numpy())


# (16, 24, 32): rows in aligned fours along axis 2 (the four-row float
# kernels); (20, 18, 22): one row per thread
@pytest.mark.parametrize("dims", [(20, 18, 22), (16, 24, 32)])
@pytest.mark.parametrize("form", ["fp64", "f32", "bf16"])
def test_grid_pcg_equals_csr(cuda, form, dims):
    m = cuda.gen_27pt(dims, _k(dims, 7))
    hg, hc = _pair(cuda, m, dims, **FORMS[form])
    b = np.random.default_rng(6).uniform(-1, 1, m.row_num())
    flexible = form != "fp64"
    rg = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=hg, rtol=1e-8, maxit=300, flexible=flexible)
    rc = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=hc, rtol=1e-8, maxit=300, flexible=flexible)
    assert rg.iterations == rc.iterations
    np.testing.assert_array_equal(rg.x.cpu().numpy(), rc.x.cpu().numpy())
    if form == "fp64":
        ref = lo.gen_27pt(dims, _k(dims, 7))
        x = rg.x.cpu().numpy()
        assert np.linalg.norm(b - lo.spmv(ref, x)) <= 1.01e-8 * np.linalg.norm(b)


def test_grid_declared_on_host_matrix(cuda):
    dims = (6, 8, 10)
    ref = lo.gen_27pt(dims, _k(dims))
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    col = cuda.Colouring.from_array(m, _parity(dims), 8)
    h0 = cuda.HierarchyWright(**PARAMS).instantiate(m, finest_colouring=col)
    assert not h0.grid27_active()  # nothing declared
    m.set_grid27(dims)
    h1 = cuda.HierarchyWright(**PARAMS).instantiate(m, finest_colouring=col)
    assert h1.grid27_active()
    b = np.random.default_rng(2).uniform(-1, 1, ref.n)
    np.testing.assert_array_equal(h1.vcycle(b).cpu().numpy(), h0.vcycle(b).cpu().numpy())
    with pytest.raises(cuda.LinealError):
        m.set_grid27((6, 8, 11))


def test_grid_stays_off_without_the_structure(cuda):
    # a 7-point matrix declared as a 27-point grid fails the device check
    dims = (6, 8, 10)
    ref = lo.gen_7pt(dims, _k(dims))
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    m.set_grid27(dims)
    col = cuda.Colouring.from_array(m, _parity(dims), 8)
    h = cuda.HierarchyWright(**PARAMS).instantiate(m, finest_colouring=col)
    assert not h.grid27_active()
    b = np.random.default_rng(4).uniform(-1, 1, ref.n)
    # the CSR path runs instead, the same as without the declaration
    m2 = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    h2 = cuda.HierarchyWright(**PARAMS).instantiate(
        m2, finest_colouring=cuda.Colouring.from_array(m2, _parity(dims), 8))
    np.testing.assert_array_equal(h.vcycle(b).cpu().numpy(), h2.vcycle(b).cpu().numpy())
    # odd edges and a Jones-Plassmann finest colouring keep the CSR path too
    for d, colouring in (((7, 8, 10), "parity"), ((6, 8, 10), "jp")):
        g27 = cuda.gen_27pt(d, _k(d))
        c = (cuda.Colouring.from_array(g27, _parity(d), 8) if colouring == "parity" else None)
        hh = cuda.HierarchyWright(**PARAMS).instantiate(g27, finest_colouring=c)
        assert not hh.grid27_active()


@pytest.mark.parametrize("forward", [1, 0])
def test_standalone_colouring_grid_sweeps(cuda, forward):
    dims = (8, 12, 16)
    m = cuda.gen_27pt(dims, _k(dims, 9))
    plain = cuda.Colouring.from_array(m, _parity(dims), 8)
    grid = cuda.Colouring.from_array(m, _parity(dims), 8)
    assert grid.use_grid27(dims, with_float=True)
    rng = np.random.default_rng(10)
    b = cuda.permute(plain, rng.uniform(-1, 1, m.row_num()))
    x0 = cuda.permute(plain, rng.uniform(-1, 1, m.row_num()))
    xa, xb = x0.clone(), x0.clone()
    cuda.sor_sweep_permuted(plain, b, xa, forward=forward)
    cuda.sor_sweep_permuted(grid, b, xb, forward=forward)
    np.testing.assert_array_equal(xa.cpu().numpy(), xb.cpu().numpy())
    fa, fb = x0.float(), x0.float()
    cuda.sor_sweep_permuted(plain, b.float(), fa, forward=forward)
    cuda.sor_sweep_permuted(grid, b.float(), fb, forward=forward)
    np.testing.assert_array_equal(fa.cpu().numpy(), fb.cpu().numpy())
    # a 7-point matrix's parity colouring does not take the grid kernels
    m7 = cuda.gen_7pt(dims, _k(dims, 9))
    assert not cuda.Colouring.from_array(m7, _parity(dims), 8).use_grid27(dims)


# Grids of more than a hundred thousand rows: the value-staged kernels (one
# tensor copy of a CTA's value planes, FP64 and float, sweeps from zero and
# from a given x) against the CSR kernels, bit for bit, in sweeps, V-cycles
# and solves.
@pytest.mark.parametrize("dims", [(48, 48, 48), (32, 64, 40)])
def test_grid_staged_values_equal_csr(cuda, dims):
    m = cuda.gen_27pt(dims, _k(dims, 12))
    plain = cuda.Colouring.from_array(m, _parity(dims), 8)
    grid = cuda.Colouring.from_array(m, _parity(dims), 8)
    assert grid.use_grid27(dims, with_float=True)
    rng = np.random.default_rng(13)
    b = cuda.permute(plain, rng.uniform(-1, 1, m.row_num())).float()
    x0 = cuda.permute(plain, rng.uniform(-1, 1, m.row_num())).float()
    for forward in (1, 0):
        for dt in (b.dtype, b.double().dtype):
            xa, xb = x0.to(dt), x0.to(dt)
            cuda.sor_sweep_permuted(plain, b.to(dt), xa, forward=forward)
            cuda.sor_sweep_permuted(grid, b.to(dt), xb, forward=forward)
            np.testing.assert_array_equal(xa.cpu().numpy(), xb.cpu().numpy())
    bb = np.random.default_rng(14).uniform(-1, 1, m.row_num())
    h64g, h64c = _pair(cuda, m, dims)
    np.testing.assert_array_equal(h64g.vcycle(bb).cpu().numpy(), h64c.vcycle(bb).cpu().numpy())
    hg, hc = _pair(cuda, m, dims, cycle_f32=True)
    assert hg.grid27_active()
    np.testing.assert_array_equal(hg.vcycle(bb).cpu().numpy(), hc.vcycle(bb).cpu().numpy())
    for refine in (0, 2):
        kw = dict(refine=refine) if refine else dict(flexible=True)
        rg = cuda.pcg(m, bb, precon=cuda.PRECON_AMG, amg=hg, rtol=1e-8, maxit=300, **kw)
        rc = cuda.pcg(m, bb, precon=cuda.PRECON_AMG, amg=hc, rtol=1e-8, maxit=300, **kw)
        assert rg.iterations == rc.iterations
        np.testing.assert_array_equal(rg.x.cpu().numpy(), rc.x.cpu().numpy())


def _red_black(dims):
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    return ((i + j + k) % 2).ravel().astype(np.int32)


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("dims", [(7, 9, 12), (16, 16, 16), (3, 6, 8), (5, 7, 4)])
def test_grid7_vcycle_equals_csr(cuda, form, dims):
    """7-point operators with the red-black colouring (odd n0, n1 allowed;
    (16, 16, 16) runs the four-row bfloat16 kernels)."""
    m = cuda.gen_7pt(dims, _k(dims, 11))
    col = cuda.Colouring.from_array(m, _red_black(dims), 2)
    hg = cuda.HierarchyWright(grid27=True, **PARAMS, **FORMS[form]).instantiate(
        m, finest_colouring=col)
    hc = cuda.HierarchyWright(grid27=False, **PARAMS, **FORMS[form]).instantiate(
        m, finest_colouring=col)
    assert hg.grid27_active() and not hc.grid27_active()
    b = np.random.default_rng(12).uniform(-1, 1, m.row_num())
    np.testing.assert_array_equal(hg.vcycle(b).cpu().numpy(), hc.vcycle(b).cpu().numpy())


@pytest.mark.parametrize("form", ["fp64", "f32", "bf16"])
def test_grid7_pcg_equals_csr(cuda, form):
    dims = (17, 20, 24)
    m = cuda.gen_7pt(dims, np.exp(3.0 * np.random.default_rng(2).standard_normal(
        int(np.prod(dims)))))
    col = cuda.Colouring.from_array(m, _red_black(dims), 2)
    kw = FORMS[form]
    hg = cuda.HierarchyWright(grid27=True, **PARAMS, **kw).instantiate(m, finest_colouring=col)
    hc = cuda.HierarchyWright(grid27=False, **PARAMS, **kw).instantiate(m, finest_colouring=col)
    b = np.random.default_rng(6).uniform(-1, 1, m.row_num())
    flexible = form != "fp64"
    rg = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=hg, rtol=1e-10, maxit=500, flexible=flexible)
    rc = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=hc, rtol=1e-10, maxit=500, flexible=flexible)
    assert rg.iterations == rc.iterations
    np.testing.assert_array_equal(rg.x.cpu().numpy(), rc.x.cpu().numpy())


# A red-black sweep's second colour also writes its rows' residuals (the
# V-cycle's residual pass then covers the first colour only): at sizes with
# the value-staged float kernels and every cycle form, against the CSR path
# (one residual pass over all rows), bit for bit.
@pytest.mark.parametrize("dims", [(48, 48, 48), (33, 40, 26)])
def test_grid7_sweep_residual_equals_csr(cuda, dims):
    m = cuda.gen_7pt(dims, np.exp(3.0 * np.random.default_rng(21).standard_normal(
        int(np.prod(dims)))))
    col = cuda.Colouring.from_array(m, _red_black(dims), 2)
    bb = np.random.default_rng(22).uniform(-1, 1, m.row_num())
    for form in ("fp64", "f32", "f32_coarse"):
        kw = FORMS[form]
        hg = cuda.HierarchyWright(grid27=True, **PARAMS, **kw).instantiate(
            m, finest_colouring=col)
        hc = cuda.HierarchyWright(grid27=False, **PARAMS, **kw).instantiate(
            m, finest_colouring=col)
        assert hg.grid27_active() and not hc.grid27_active()
        np.testing.assert_array_equal(hg.vcycle(bb).cpu().numpy(), hc.vcycle(bb).cpu().numpy())
        solves = [dict()] if form == "fp64" else [dict(flexible=True), dict(refine=2),
                                                   dict(refine=2, flexible=True)]
        for skw in solves:
            rg = cuda.pcg(m, bb, precon=cuda.PRECON_AMG, amg=hg, rtol=1e-10, maxit=500, **skw)
            rc = cuda.pcg(m, bb, precon=cuda.PRECON_AMG, amg=hc, rtol=1e-10, maxit=500, **skw)
            assert rg.iterations == rc.iterations
            np.testing.assert_array_equal(rg.x.cpu().numpy(), rc.x.cpu().numpy())


def test_grid7_stays_off_without_the_structure(cuda):
    dims = (6, 8, 10)
    # odd n2, a 27-point matrix declared as 7-point, a parity (8-colour)
    # colouring of a 7-point matrix: the CSR path stays
    m = cuda.gen_7pt((6, 8, 9), _k((6, 8, 9)))
    h = cuda.HierarchyWright(**PARAMS).instantiate(
        m, finest_colouring=cuda.Colouring.from_array(m, _red_black((6, 8, 9)), 2))
    assert not h.grid27_active()
    ref = lo.gen_27pt(dims, _k(dims))
    m27 = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    m27.set_grid7(dims)
    h = cuda.HierarchyWright(**PARAMS).instantiate(
        m27, finest_colouring=cuda.Colouring.from_array(m27, _parity(dims), 8))
    assert not h.grid27_active()
    m7 = cuda.gen_7pt(dims, _k(dims))
    h = cuda.HierarchyWright(**PARAMS).instantiate(
        m7, finest_colouring=cuda.Colouring.from_array(m7, _parity(dims), 8))
    assert not h.grid27_active()
