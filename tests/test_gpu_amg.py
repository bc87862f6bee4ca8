"""GPU parity of the AMG setup (bit-exact integer/bit data and level
matrices) and of the V-cycle against the oracle."""

import os

import numpy as np
import pytest

import oracle as lo
from lineal_gb300 import io as lio

pytestmark = pytest.mark.gpu


def _case(dims=(14, 15, 16), seed=1, sigma=1.5, npts=27):
    n = int(np.prod(dims))
    k = np.exp(sigma * np.random.default_rng(seed).standard_normal(n))
    return (lo.gen_27pt if npts == 27 else lo.gen_7pt)(dims, k)


def _dev(cuda, ref, storage=0):
    return cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=ref.symmetric,
                                    storage=storage)


def _ufz(golden_dir):
    rowptr, col, val, _ = lio.read_smf(os.path.join(golden_dir, "UFZ_CT_02_LHS.smf"))
    return lo.Csr(rowptr, col, val, symmetric=False)


@pytest.mark.parametrize("which", ["27pt", "7pt", "ufz"])
def test_strength_bitexact(cuda, golden_dir, which):
    ref = _ufz(golden_dir) if which == "ufz" else _case(npts=27 if which == "27pt" else 7)
    m = _dev(cuda, ref)
    dep, inf, iso = cuda.amg_strength(m)
    rdep, rinf, riso = lo.amg_strength(ref)
    np.testing.assert_array_equal(dep.cpu().numpy(), rdep)
    np.testing.assert_array_equal(inf.cpu().numpy(), rinf)
    np.testing.assert_array_equal(iso.cpu().numpy(), riso)


@pytest.fixture(params=["warp", "cta"])
def agg_kernel(request, monkeypatch):
    """Both aggregation kernels: one warp per partition with its state in
    global memory, one CTA per partition with its state in shared memory."""
    monkeypatch.setenv("LGX_AGG_KERNEL", request.param)
    return request.param


@pytest.mark.parametrize("nparts", [1, 7, 64])
@pytest.mark.parametrize("aggressive", [False, True])
def test_aggregation_bitexact(cuda, nparts, aggressive, agg_kernel):
    ref = _case()
    m = _dev(cuda, ref)
    dep, inf, iso = cuda.amg_strength(m)
    nc, agg = cuda.amg_aggregate(m, dep, inf, iso, 6, 9, nparts, aggressive)
    rdep, rinf, riso = lo.amg_strength(ref)
    rnc, ragg, _, _, _ = lo.amg_aggregate(ref, rdep, rinf, riso, 6, 9, nparts, aggressive)
    assert nc == rnc
    np.testing.assert_array_equal(agg, ragg)


@pytest.mark.parametrize("dims,npts,nparts", [((30, 28, 26), 27, 3), ((40, 36, 30), 7, 5)])
def test_aggregation_coarse_level_bitexact(cuda, agg_kernel, dims, npts, nparts):
    """A coarse level (the Galerkin product of the first aggregation: dense,
    irregular rows) split into few large partitions, the case the CTA
    kernel serves; plain and aggressive thresholds."""
    ref = _case(dims, npts=npts)
    oh = lo.Amg(ref, min_coarsen_size=100, partition_size=4096, smoother_parts=0)
    c = oh.level_csr(1)
    m = _dev(cuda, c)
    for aggressive in (False, True):
        dep, inf, iso = cuda.amg_strength(m)
        nc, agg = cuda.amg_aggregate(m, dep, inf, iso, 6, 9, nparts, aggressive)
        rdep, rinf, riso = lo.amg_strength(c)
        rnc, ragg, _, _, _ = lo.amg_aggregate(c, rdep, rinf, riso, 6, 9, nparts, aggressive)
        assert nc == rnc
        np.testing.assert_array_equal(agg, ragg)


def test_aggregation_ufz_bitexact(cuda, golden_dir, agg_kernel):
    ref = _ufz(golden_dir)
    m = _dev(cuda, ref)
    dep, inf, iso = cuda.amg_strength(m)
    nc, agg = cuda.amg_aggregate(m, dep, inf, iso, 6, 9, 4)
    rdep, rinf, riso = lo.amg_strength(ref)
    rnc, ragg, _, _, _ = lo.amg_aggregate(ref, rdep, rinf, riso, 6, 9, 4)
    assert nc == rnc
    np.testing.assert_array_equal(agg, ragg)


@pytest.mark.parametrize("case", ["front", "ids"])
def test_aggregation_beyond_shared_capacity(cuda, agg_kernel, monkeypatch, case):
    """Partitions that outgrow the CTA kernel's capacities -- a front or
    connected set longer than the list capacity (lowered to 64 entries;
    27-point rows and aggregates of up to 9 vertices reach ~100),
    more than 65533 aggregates in one partition (70k vertices, aggregates of
    one) -- are redone in global memory: the result is the oracle's for
    every kernel choice."""
    if case == "front":
        monkeypatch.setenv("LGX_AGG_CTA_CAP", "64")
        ref, lo_size, hi_size = _case(), 6, 9
    else:
        ref, lo_size, hi_size = _case((40, 42, 42), npts=7), 1, 1
    m = _dev(cuda, ref)
    dep, inf, iso = cuda.amg_strength(m)
    nc, agg = cuda.amg_aggregate(m, dep, inf, iso, lo_size, hi_size, 1)
    rdep, rinf, riso = lo.amg_strength(ref)
    rnc, ragg, _, _, _ = lo.amg_aggregate(ref, rdep, rinf, riso, lo_size, hi_size, 1)
    assert nc == rnc
    np.testing.assert_array_equal(agg, ragg)
    if case == "ids":
        assert nc > 65533


PARAMS = dict(min_coarsen_size=64, partition_size=512, max_partitions=1 << 30)


@pytest.mark.parametrize("coarse_f32", [False, True])
def test_hierarchy_bitexact(cuda, coarse_f32, agg_kernel):
    ref = _case()
    m = _dev(cuda, ref)
    h = cuda.HierarchyWright(coarse_f32=coarse_f32, **PARAMS).instantiate(m)
    oh = lo.Amg(ref, coarse_f32=int(coarse_f32), smoother_parts=0, **PARAMS)
    rows, _ = h.sizes()
    assert len(rows) == oh.nlevels >= 3
    for l in range(oh.nlevels):
        rowptr, col, val, agg = h.level(l)
        rl = oh.level_csr(l)
        np.testing.assert_array_equal(rowptr, rl.rowptr)
        np.testing.assert_array_equal(col, rl.col)
        np.testing.assert_array_equal(val, rl.val)
        if agg is not None:
            np.testing.assert_array_equal(agg, oh.level_agg(l))


def test_hierarchy_bitexact_large_aggregates(cuda):
    """Aggregates of 24 to 48 rows: coarse rows gather up to 48 * 27 fine
    entries, beyond the 512 the warp-per-row Galerkin product stages, so
    those rows take the thread-per-row product while the smaller ones stay
    on the warp kernel; every level equals the oracle's bit for bit."""
    ref = _case((18, 20, 22))
    m = _dev(cuda, ref)
    params = dict(PARAMS, min_aggregate_size=24, max_aggregate_size=48)
    h = cuda.HierarchyWright(**params).instantiate(m)
    oh = lo.Amg(ref, smoother_parts=0, **params)
    rows, _ = h.sizes()
    assert len(rows) == oh.nlevels >= 2
    for l in range(oh.nlevels):
        rowptr, col, val, agg = h.level(l)
        rl = oh.level_csr(l)
        np.testing.assert_array_equal(rowptr, rl.rowptr)
        np.testing.assert_array_equal(col, rl.col)
        np.testing.assert_array_equal(val, rl.val)
    # the first coarse level holds rows gathered from more than 512 entries
    rowptr0 = oh.level_csr(0).rowptr
    agg0 = oh.level_agg(0)
    lens = np.diff(rowptr0)
    sizes = np.zeros(rows[1], dtype=np.int64)
    np.add.at(sizes, agg0[agg0 < rows[1]], lens[agg0 < rows[1]])
    assert sizes.max() > 512 and sizes.min() <= 512


@pytest.mark.parametrize("coarse_f32", [False, True])
def test_vcycle_matches_oracle(cuda, coarse_f32):
    ref = _case()
    m = _dev(cuda, ref)
    h = cuda.HierarchyWright(coarse_f32=coarse_f32, **PARAMS).instantiate(m)
    oh = lo.Amg(ref, coarse_f32=int(coarse_f32), smoother_parts=0, **PARAMS)
    b = np.random.default_rng(3).uniform(-1, 1, ref.n)
    got = h.vcycle(b).cpu().numpy()
    want = oh.vcycle(b)
    # same colour orders and level matrices; the coarsest solve is a dense
    # inverse on the GPU and a Cholesky substitution in the oracle
    assert np.abs(got - want).max() <= 1e-11 * np.abs(want).max()


def test_vcycle_float_cycle(cuda):
    ref = _case()
    m = _dev(cuda, ref)
    h = cuda.HierarchyWright(cycle_f32=True, **PARAMS).instantiate(m)
    oh = lo.Amg(ref, smoother_parts=0, **PARAMS)
    b = np.random.default_rng(3).uniform(-1, 1, ref.n)
    got = h.vcycle(b).cpu().numpy()
    want = oh.vcycle(b)
    assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max()


def test_finest_parity_colouring(cuda):
    dims = (12, 12, 12)
    ref = _case(dims)
    m = _dev(cuda, ref)
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    colours = ((i % 2) * 4 + (j % 2) * 2 + (k % 2)).ravel().astype(np.int32)
    col = cuda.Colouring.from_array(m, colours, 8)
    h = cuda.HierarchyWright(**PARAMS).instantiate(m, finest_colouring=col)
    b = np.random.default_rng(1).uniform(-1, 1, ref.n)
    x = h.vcycle(b).cpu().numpy()
    # one V-cycle reduces the residual of the error equation
    r = b - lo.spmv(ref, x)
    assert np.linalg.norm(r) < 0.5 * np.linalg.norm(b)


def _convdiff():
    # upwind convection-diffusion: nonsymmetric values and coarse operators
    return lo.gen_convdiff((14, 13, 12), (8.0, -5.0, 3.0))


def test_vcycle_nonsymmetric_lu_coarse_matches_oracle(cuda):
    """Nonsymmetric hierarchy (coarsest solved like LuSolver: unpivoted
    elimination) against the oracle's LU."""
    ref = _convdiff()
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=False)
    h = cuda.HierarchyWright(**PARAMS).instantiate(m)
    oh = lo.Amg(ref, smoother_parts=0, **PARAMS)
    b = np.random.default_rng(4).uniform(-1, 1, ref.n)
    got = h.vcycle(b).cpu().numpy()
    want = oh.vcycle(b)
    assert np.abs(got - want).max() <= 1e-11 * np.abs(want).max()


def test_bicgstab_amg_nonsymmetric_matches_oracle(cuda):
    """BiCGStab + AMG with the LU coarse solve (test/aux/iterative.hpp:175-181
    runs this combination)."""
    ref = _convdiff()
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=False)
    h = cuda.HierarchyWright(**PARAMS).instantiate(m)
    oh = lo.Amg(ref, smoother_parts=0, **PARAMS)
    b = np.random.default_rng(5).uniform(-1, 1, ref.n)
    res = cuda.pbicgstab(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=1e-8, maxit=300)
    _, it, _ = lo.pbicgstab(ref, b, precon=lo.PRECON_AMG, amg=oh, rtol=1e-8, maxit=300)
    assert abs(res.iterations - it) <= max(1, int(0.05 * it + 0.999))
    x = res.x.cpu().numpy()
    assert np.linalg.norm(b - lo.spmv(ref, x)) <= 1.01e-8 * np.linalg.norm(b)
