"""The precision form's float-vector CG under an FP64 solution and residual
(lgx_solve_params.refine): 1 = iterative refinement (restarted inner
solves), 2 = reliable updates (one unbroken float recurrence with FP64
residual replacement).  The FP64-verified residual reaches the tolerance,
the iteration counts stay close to the FP64 PCG's (reliable updates: within
two), graph replay equals the eager run bit for bit, and the option refuses
what it cannot run."""

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu

PARAMS = dict(min_coarsen_size=64, partition_size=512)


def _parity(dims):
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    return ((i % 2) * 4 + (j % 2) * 2 + (k % 2)).ravel().astype(np.int32)


def _red_black(dims):
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    return ((i + j + k) % 2).ravel().astype(np.int32)


def _case27(dims, seed=1, sigma=1.5):
    k = np.exp(sigma * np.random.default_rng(seed).standard_normal(int(np.prod(dims))))
    return k, lo.gen_27pt(dims, k)


@pytest.mark.parametrize("dims,grid", [((20, 18, 22), True), ((20, 18, 22), False),
                                       ((17, 19, 13), True)])
@pytest.mark.parametrize("rtol", [1e-8, 1e-10])
@pytest.mark.parametrize("mode", [1, 2])
def test_refined_reaches_fp64_tolerance(cuda, dims, grid, rtol, mode):
    k, ref = _case27(dims)
    m = cuda.gen_27pt(dims, k)
    col = cuda.Colouring.from_array(m, _parity(dims), 8) if dims[2] % 2 == 0 else None
    h64 = cuda.HierarchyWright(grid27=grid, **PARAMS).instantiate(m, finest_colouring=col)
    h32 = cuda.HierarchyWright(grid27=grid, cycle_f32=True, **PARAMS).instantiate(
        m, finest_colouring=col)
    b = np.random.default_rng(0).uniform(-1, 1, ref.n)
    r64 = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h64, rtol=rtol, maxit=400)
    rr = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h32, rtol=rtol, maxit=400, refine=mode)
    x = rr.x.cpu().numpy()
    # the stopping test is the FP64 residual: verified with the oracle's product
    true_rel = np.linalg.norm(b - lo.spmv(ref, x)) / np.linalg.norm(b)
    assert rr.rel_residual <= rtol and true_rel <= 1.01 * rtol
    assert abs(true_rel - rr.rel_residual) <= 1e-3 * rtol + 1e-16
    # restarts cost a few iterations against the FP64 recurrence; reliable
    # updates keep it
    if mode == 1:
        assert rr.iterations <= r64.iterations + max(5, int(0.15 * r64.iterations))
    else:
        assert abs(rr.iterations - r64.iterations) <= 2
    # the last history entry is the FP64 residual
    assert rr.history[-1] == pytest.approx(rr.rel_residual * np.linalg.norm(b), rel=1e-12)
    # error against the FP64 solution: both within the tolerance's reach
    x64 = r64.x.cpu().numpy()
    assert np.linalg.norm(x - x64) <= 1e3 * rtol * np.linalg.norm(x64)


@pytest.mark.parametrize("mode", [1, 2])
def test_refined_graph_replay_equals_eager(cuda, mode):
    dims = (16, 16, 16)
    k, ref = _case27(dims, 2)
    m = cuda.gen_27pt(dims, k)
    col = cuda.Colouring.from_array(m, _parity(dims), 8)
    h = cuda.HierarchyWright(cycle_f32=True, **PARAMS).instantiate(m, finest_colouring=col)
    b = np.random.default_rng(3).uniform(-1, 1, ref.n)
    g = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=1e-9, refine=mode, use_graphs=True)
    e = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=1e-9, refine=mode, use_graphs=False)
    assert g.iterations == e.iterations
    np.testing.assert_array_equal(g.x.cpu().numpy(), e.x.cpu().numpy())
    np.testing.assert_array_equal(g.history, e.history)


@pytest.mark.parametrize("mode,flexible", [(1, False), (2, False), (2, True)])
def test_refined_seven_point_high_contrast(cuda, mode, flexible):
    # the precision-form operator family: 7 points, lognormal sigma = 3
    dims = (24, 24, 24)
    kk = np.exp(3.0 * np.random.default_rng(2).standard_normal(int(np.prod(dims))))
    ref = lo.gen_7pt(dims, kk)
    m = cuda.gen_7pt(dims, kk)
    col = cuda.Colouring.from_array(m, _red_black(dims), 2)
    h = cuda.HierarchyWright(cycle_f32=True, **PARAMS).instantiate(m, finest_colouring=col)
    b = np.random.default_rng(0).uniform(-1, 1, ref.n)
    rr = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=1e-10, maxit=500, refine=mode,
                  flexible=flexible)
    x = rr.x.cpu().numpy()
    assert np.linalg.norm(b - lo.spmv(ref, x)) <= 1.01e-10 * np.linalg.norm(b)
    xr, it, _ = lo.pcg(ref, b, precon=lo.PRECON_AMG,
                       amg=lo.Amg(ref, finest_colours=_red_black(dims), ncolours=2,
                                  smoother_parts=0, **PARAMS), rtol=1e-10, maxit=500)
    # each refinement step restarts the Krylov recurrence: a few more
    # iterations than the unbroken FP64 recurrence; reliable updates keep it
    # (the float recurrence on this high-contrast operator with the
    # flexible beta)
    assert rr.iterations <= it + (max(5, int(0.15 * it)) if mode == 1 or not flexible else 2)
    assert np.linalg.norm(x - xr) <= 1e-6 * np.linalg.norm(xr)


def test_refined_refusals(cuda):
    dims = (8, 8, 8)
    k, ref = _case27(dims)
    m = cuda.gen_27pt(dims, k)
    b = np.ones(ref.n)
    h64 = cuda.HierarchyWright(**PARAMS).instantiate(m)
    with pytest.raises(cuda.LinealError) as e:
        cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h64, refine=True)
    assert "cycle_f32" in str(e.value)
    with pytest.raises(cuda.LinealError):
        cuda.pcg(m, b, precon=cuda.PRECON_JACOBI, refine=True)
    h32 = cuda.HierarchyWright(cycle_f32=True, **PARAMS).instantiate(m)
    with pytest.raises(cuda.LinealError):
        cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h32, refine=True, inner_rtol=0.0)
    with pytest.raises(cuda.LinealError):
        cuda.pbicgstab(m, b, precon=cuda.PRECON_AMG, amg=h32, refine=True)
    with pytest.raises(cuda.LinealError):
        cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h32, refine=3)
    with pytest.raises(cuda.LinealError):
        cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h64, refine=2)
