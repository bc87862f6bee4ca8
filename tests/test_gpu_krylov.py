"""GPU Krylov solvers against the reference's bound tables and the oracle's
iteration counts."""

import os

import numpy as np
import pytest

import oracle as lo
from lineal_gb300 import io as lio

pytestmark = pytest.mark.gpu


def _stencil_system(cuda):
    dims = (4, 9, 7)
    mat = lo.material_diagonal_lines(dims, 4)
    ref = lo.Stencil(dims, mat=mat, coeffs=(0, 1, 2, 3), sol_start=1, sol_end=0)
    a, _ = ref.to_csr()
    st = cuda.StencilMatrix.lookup(dims, (1, 1, 1), (0, 1, 2, 3), mat, 1.0, 0.0)
    csr = cuda.CsrMatrix.from_host(a.rowptr, a.col, a.val)
    return ref, a, st, csr


# bounds of test/shared-stencil.hpp:157-180 (x = 2) and 201-224 (real rhs)
CASES = [
    ("cg", "pcg", dict(), 129, 1e-12, 1e-13),
    ("bicgstab", "pbicgstab", dict(), 129, 1e-12, 1e-13),
    ("pcg_ssor1", "pcg", dict(precon=2), 129, 1e-13, 1e-13),
    ("pbicgstab_ssor1", "pbicgstab", dict(precon=2), 129, 1e-12, 1e-13),
    ("pcg_amg", "pcg", dict(precon=3), 33, 1e-13, 2e-14),
    ("pbicgstab_amg", "pbicgstab", dict(precon=3), 33, 1e-13, 1e-13),
]


@pytest.mark.parametrize("name,fn,kw,iters,bound_x2,bound_rhs", CASES)
def test_reference_suite_bounds(cuda, name, fn, kw, iters, bound_x2, bound_rhs):
    ref, a, st, csr = _stencil_system(cuda)
    kw = dict(kw)
    if kw.get("precon") == cuda.PRECON_AMG:
        kw["amg"] = cuda.HierarchyWright(min_coarsen_size=32, partition_size=126,
                                         coarse_f32=True).instantiate(csr)
    solve = getattr(cuda, fn)
    mat = csr if kw.get("precon") in (cuda.PRECON_SSOR, cuda.PRECON_AMG) else st
    b2 = lo.spmv(a, np.full(a.n, 2.0))
    res = solve(mat, b2, rtol=0.0, maxit=iters, **kw)
    x = res.x.cpu().numpy()
    assert res.history[-1] <= bound_x2 and np.abs(x - 2).max() <= bound_x2
    b = ref.rhs()
    res = solve(mat, b, rtol=0.0, maxit=iters, **kw)
    x = res.x.cpu().numpy()
    assert res.history[-1] <= bound_rhs and np.abs(lo.spmv(a, x) - b).max() <= bound_rhs


@pytest.mark.parametrize("edge", [24, 64])
def test_jacobi_pcg_poisson_matches_oracle(cuda, edge):
    # the plain-method workload (64^3 Poisson as a lookup stencil with one
    # material, unit cells, b ~ U[-1, 1] seed 0, x0 = 0, Jacobi-PCG to 1e-8)
    # and a smaller copy
    dims = (edge,) * 3
    n = int(np.prod(dims))
    mat = np.ones(n, dtype=np.uint8)
    coeffs = (0.0, 1.0, 0.0, 0.0)
    b = np.random.default_rng(0).uniform(-1, 1, n)
    st = cuda.StencilMatrix.lookup(cuda.BoxInfo(dims, dims), None, coeffs, mat, 0.0, 0.0)
    res = cuda.pcg(st, b, precon=cuda.PRECON_JACOBI, rtol=1e-8, maxit=1000)
    ref = lo.Stencil(dims, mat=mat, coeffs=coeffs, sol_start=0, sol_end=0)
    a, _ = ref.to_csr()
    x, it, hist = lo.pcg(a, b, precon=lo.PRECON_JACOBI, rtol=1e-8, maxit=1000)
    assert res.rel_residual <= 1e-8
    assert abs(res.iterations - it) <= max(1, 0.05 * it)
    np.testing.assert_allclose(res.history[: min(10, it)], hist[: min(10, it)], rtol=1e-10)
    xr = res.x.cpu().numpy()
    assert np.linalg.norm(b - lo.spmv(a, xr)) <= 1.01e-8 * np.linalg.norm(b)


def _lognormal_27pt(dims, sigma, seed):
    n = int(np.prod(dims))
    k = np.exp(sigma * np.random.default_rng(seed).standard_normal(n))
    return lo.gen_27pt(dims, k), k


@pytest.mark.parametrize("cycle_f32", [False, True])
def test_amg_pcg_27pt_matches_oracle(cuda, cycle_f32):
    dims = (20, 20, 20)
    ref, k = _lognormal_27pt(dims, 1.5, 1)
    b = np.random.default_rng(0).uniform(-1, 1, ref.n)
    m = cuda.gen_27pt(dims, k)
    params = dict(min_coarsen_size=200, partition_size=1000)
    h = cuda.HierarchyWright(cycle_f32=cycle_f32, **params).instantiate(m)
    res = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=1e-8, maxit=300)
    oh = lo.Amg(ref, smoother_parts=0, **params)
    x, it, hist = lo.pcg(ref, b, precon=lo.PRECON_AMG, amg=oh, rtol=1e-8, maxit=300)
    assert res.rel_residual <= 1e-8
    xr = res.x.cpu().numpy()
    # FP64-verified residual
    assert np.linalg.norm(b - lo.spmv(ref, xr)) <= 1.1e-8 * np.linalg.norm(b)
    assert abs(res.iterations - it) <= max(1, int(0.05 * it + 0.999))
    if not cycle_f32:
        np.testing.assert_allclose(res.history[:5], hist[:5], rtol=1e-9)


def test_amg_bicgstab_ufz(cuda, golden_dir):
    rowptr, col, val, _ = lio.read_smf(os.path.join(golden_dir, "UFZ_CT_02_LHS.smf"))
    b = lio.read_dvf(os.path.join(golden_dir, "UFZ_CT_02_RHS.dvf"))
    m = cuda.CsrMatrix.from_host(rowptr, col, val, symmetric=False)
    h = cuda.HierarchyWright(min_coarsen_size=32, partition_size=64).instantiate(m)
    res = cuda.pbicgstab(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=1e-10, maxit=300)
    assert res.rel_residual <= 1e-10
    ref = lo.Csr(rowptr, col, val, symmetric=False)
    x = res.x.cpu().numpy()
    assert np.linalg.norm(b - lo.spmv(ref, x)) <= 1e-9 * np.linalg.norm(b)


def test_breakdown_reported_as_status(cuda):
    # a singular (all-zero off-diagonal, zero-diagonal replaced) system whose
    # right-hand side is zero stops immediately; a NaN right-hand side is a
    # non-finite status, not a trap
    ref, a, st, csr = _stencil_system(cuda)
    b = np.full(a.n, np.nan)
    with pytest.raises(cuda.LinealError) as e:
        cuda.pcg(csr, b, rtol=1e-8, maxit=5)
    assert e.value.status in (4, 5)


def test_flexible_cg_precision_form(cuda):
    """Precision form: flexible CG over the float V-cycle reaches 1e-10 on a
    high-contrast 7-point problem (lognormal sigma = 3), verified in FP64 on
    the oracle, within a few iterations of the plain FP64 AMG-PCG; on a
    linear (FP64) preconditioner flexible CG follows plain CG."""
    dims = (24, 24, 24)
    n = int(np.prod(dims))
    k = np.exp(3.0 * np.random.default_rng(2).standard_normal(n))
    ref = lo.gen_7pt(dims, k)
    b = np.random.default_rng(0).uniform(-1, 1, n)
    m = cuda.gen_7pt(dims, k)
    params = dict(min_coarsen_size=200, partition_size=1000)
    h64 = cuda.HierarchyWright(**params).instantiate(m)
    h32 = cuda.HierarchyWright(cycle_f32=True, **params).instantiate(m)
    plain = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h64, rtol=1e-10, maxit=500)
    flex64 = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h64, rtol=1e-10, maxit=500,
                      flexible=True)
    flex32 = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h32, rtol=1e-10, maxit=500,
                      flexible=True)
    for res in (plain, flex64, flex32):
        assert res.rel_residual <= 1e-10
        xr = res.x.cpu().numpy()
        assert np.linalg.norm(b - lo.spmv(ref, xr)) <= 1.2e-10 * np.linalg.norm(b)
    assert abs(flex64.iterations - plain.iterations) <= 2
    assert flex32.iterations <= plain.iterations + max(2, plain.iterations // 10)
    x64 = plain.x.cpu().numpy()
    assert np.linalg.norm(flex32.x.cpu().numpy() - x64) <= 1e-7 * np.linalg.norm(x64)


def test_precision_form_five_levels_matches_oracle(cuda):
    """The precision-form operator family (7 points, lognormal sigma = 3,
    seed 2) on a 56^3 grid whose hierarchy has at least five levels, as the
    256^3 workload's does: level sizes equal the oracle's; the FP64 solve's
    iterations are the oracle's; flexible CG and the refinement over the
    float cycle reach 1e-10 verified in FP64 with the oracle's product,
    within a few iterations of the oracle, close to its solution."""
    dims = (56, 56, 56)
    n = int(np.prod(dims))
    k = np.exp(3.0 * np.random.default_rng(2).standard_normal(n))
    ref = lo.gen_7pt(dims, k)
    b = np.random.default_rng(0).uniform(-1, 1, n)
    m = cuda.gen_7pt(dims, k)
    i, j, kk = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    rb = ((i + j + kk) % 2).ravel().astype(np.int32)
    col = cuda.Colouring.from_array(m, rb, 2)
    params = dict(min_coarsen_size=200, partition_size=4096)
    h64 = cuda.HierarchyWright(**params).instantiate(m, finest_colouring=col)
    h32 = cuda.HierarchyWright(cycle_f32=True, **params).instantiate(m, finest_colouring=col)
    oh = lo.Amg(ref, finest_colours=rb, ncolours=2, smoother_parts=0, **params)
    rows, _ = h64.sizes()
    assert len(rows) >= 5
    assert rows == [oh.level_size(l) for l in range(oh.nlevels)]
    xo, it, hist = lo.pcg(ref, b, precon=lo.PRECON_AMG, amg=oh, rtol=1e-10, maxit=600)
    plain = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h64, rtol=1e-10, maxit=600)
    assert abs(plain.iterations - it) <= max(1, int(0.05 * it + 0.999))
    np.testing.assert_allclose(plain.history[:5], hist[:5], rtol=1e-9)
    # (solve, iteration slack): restarted refinement pays for its restarts
    for res, slack in ((plain, 2),
                       (cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h32, rtol=1e-10, maxit=600,
                                 flexible=True), max(5, (15 * it) // 100)),
                       (cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h32, rtol=1e-10, maxit=600,
                                 refine=2), max(5, (15 * it) // 100)),
                       (cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h32, rtol=1e-10, maxit=600,
                                 refine=1), max(8, (30 * it) // 100))):
        xr = res.x.cpu().numpy()
        assert np.linalg.norm(b - lo.spmv(ref, xr)) <= 1.2e-10 * np.linalg.norm(b)
        assert res.iterations <= it + slack
        assert np.linalg.norm(xr - xo) <= 1e-6 * np.linalg.norm(xo)


@pytest.mark.parametrize("dims,npts", [((20, 20, 20), 27), ((24, 24, 24), 7)])
def test_bf16_cycle_precision_form(cuda, dims, npts):
    """Precision form with bfloat16 level values (diagonal row scales): flexible
    CG over the bf16 float cycle reaches 1e-10, verified in FP64 on the
    oracle, in at most a few more iterations than the float-valued cycle."""
    n = int(np.prod(dims))
    k = np.exp(1.5 * np.random.default_rng(3).standard_normal(n))
    ref = (lo.gen_27pt if npts == 27 else lo.gen_7pt)(dims, k)
    m = (cuda.gen_27pt if npts == 27 else cuda.gen_7pt)(dims, k)
    b = np.random.default_rng(0).uniform(-1, 1, n)
    params = dict(min_coarsen_size=200, partition_size=1000)
    h32 = cuda.HierarchyWright(cycle_f32=True, **params).instantiate(m)
    h16 = cuda.HierarchyWright(cycle_f32=True, cycle_bf16=True, **params).instantiate(m)
    f32 = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h32, rtol=1e-10, maxit=500, flexible=True)
    f16 = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h16, rtol=1e-10, maxit=500, flexible=True)
    assert f16.rel_residual <= 1e-10
    xr = f16.x.cpu().numpy()
    assert np.linalg.norm(b - lo.spmv(ref, xr)) <= 1.2e-10 * np.linalg.norm(b)
    assert f16.iterations <= f32.iterations + max(3, f32.iterations // 5)
    # the bf16 cycle is a nearby preconditioner: one application differs from
    # the float cycle's by about the bfloat16 precision
    z32 = h32.vcycle(b).cpu().numpy()
    z16 = h16.vcycle(b).cpu().numpy()
    assert np.linalg.norm(z16 - z32) <= 0.05 * np.linalg.norm(z32)
