"""GPU parity of the operators against the oracle (bit-exact where the
summation order is the reference's scalar order)."""

import os

import numpy as np
import pytest

import oracle as lo
from lineal_gb300 import io as lio

pytestmark = pytest.mark.gpu


def _ufz(golden_dir):
    rowptr, col, val, _ = lio.read_smf(os.path.join(golden_dir, "UFZ_CT_02_LHS.smf"))
    b = lio.read_dvf(os.path.join(golden_dir, "UFZ_CT_02_RHS.dvf"))
    return lo.Csr(rowptr, col, val, symmetric=False), b


def test_csr_spmv_ufz_bitexact(cuda, golden_dir):
    a, b = _ufz(golden_dir)
    m = cuda.CsrMatrix.from_host(a.rowptr, a.col, a.val, symmetric=False)
    assert m.info()[1:3] == (a.n, a.nnz)
    for seed in range(3):
        x = np.random.default_rng(seed).uniform(-1, 1, a.n)
        y = cuda.spmv(m, x).cpu().numpy()
        np.testing.assert_array_equal(y, lo.spmv(a, x))
    r, nrm = cuda.residual(m, b, x)
    ref = lo.residual(a, b, x)
    np.testing.assert_array_equal(r.cpu().numpy(), ref)
    assert abs(nrm - ref @ ref) <= 1e-14 * (ref @ ref)


@pytest.mark.parametrize("dims", [(5, 6, 7), (16, 9, 33), (1, 1, 1), (40, 3, 2)])
@pytest.mark.parametrize("npts", [27, 7])
def test_generator_bitexact(cuda, dims, npts):
    n = int(np.prod(dims))
    k = np.exp(1.5 * np.random.default_rng(1).standard_normal(n))
    gen = cuda.gen_27pt if npts == 27 else cuda.gen_7pt
    m = gen(dims, k)
    ref = (lo.gen_27pt if npts == 27 else lo.gen_7pt)(dims, k)
    rowptr, col, val = m.download()
    np.testing.assert_array_equal(rowptr, ref.rowptr)
    np.testing.assert_array_equal(col, ref.col)
    np.testing.assert_array_equal(val, ref.val)
    x = np.random.default_rng(5).uniform(-1, 1, n)
    np.testing.assert_array_equal(cuda.spmv(m, x).cpu().numpy(), lo.spmv(ref, x))


def test_generator_f32_storage(cuda):
    dims = (12, 10, 9)
    n = int(np.prod(dims))
    k = np.exp(np.random.default_rng(3).standard_normal(n))
    m32 = cuda.gen_27pt(dims, k, storage=cuda.F32)
    ref = lo.gen_27pt(dims, k)
    x = np.random.default_rng(4).uniform(-1, 1, n)
    v32 = ref.val.astype(np.float32).astype(np.float64)
    ref32 = lo.Csr(ref.rowptr, ref.col, v32)
    # double accumulation over float-stored values
    np.testing.assert_array_equal(cuda.spmv(m32, x).cpu().numpy(), lo.spmv(ref32, x))
    y = cuda.spmv_f32(m32, x.astype(np.float32)).cpu().numpy().astype(np.float64)
    exact = lo.spmv(ref32, x.astype(np.float32).astype(np.float64))
    assert np.abs(y - exact).max() <= 1e-5 * np.abs(exact).max()


def _lookup_case(dims, seed):
    rng = np.random.default_rng(seed)
    mat = rng.integers(0, 4, int(np.prod(dims))).astype(np.uint8)
    return mat


@pytest.mark.parametrize("dims", [(4, 9, 7), (17, 13, 19), (1, 5, 3), (33, 1, 40)])
@pytest.mark.parametrize("zero_to_one", [True, False])
def test_stencil_lookup_bitexact(cuda, dims, zero_to_one):
    mat = _lookup_case(dims, 11)
    q = lo.axis_quotients(dims, (1.3, 0.7, 2.1))
    coeffs = (0.0, 1.0, 2.0, 3.0)
    ref = lo.Stencil(dims, q=q, mat=mat, coeffs=coeffs, sol_start=1.0, sol_end=0.5,
                     zero_to_one=zero_to_one)
    m = cuda.StencilMatrix.lookup(cuda.BoxInfo(dims, (1.3, 0.7, 2.1)), None, coeffs, mat, 1.0,
                                  0.5, zero_to_one)
    x = np.random.default_rng(2).uniform(-1, 1, ref.n)
    np.testing.assert_array_equal(cuda.spmv(m, x).cpu().numpy(), ref.spmv(x))
    np.testing.assert_array_equal(m.diagonal().cpu().numpy(), ref.diagonal())
    np.testing.assert_array_equal(m.rhs().cpu().numpy(), ref.rhs())
    csr, cmap = m.to_csr(with_compress_map=True)
    rcsr, rcmap = ref.to_csr()
    rowptr, col, val = csr.download()
    np.testing.assert_array_equal(rowptr, rcsr.rowptr)
    np.testing.assert_array_equal(col, rcsr.col)
    np.testing.assert_array_equal(val, rcsr.val)
    np.testing.assert_array_equal(cmap.cpu().numpy(), rcmap)


@pytest.mark.parametrize("dims", [(4, 9, 7), (21, 8, 30)])
def test_stencil_value_bitexact(cuda, dims):
    n = int(np.prod(dims))
    k = np.exp(np.random.default_rng(9).standard_normal(n))
    k[::7] = 0.0  # zero conductivities exercise the harmonic-mean guard
    q = lo.axis_quotients(dims, dims)
    ref = lo.Stencil(dims, q=q, k=k, sol_start=1.0, sol_end=0.0)
    m = cuda.StencilMatrix.value(cuda.BoxInfo(dims, dims), None, k, 1.0, 0.0)
    x = np.random.default_rng(8).uniform(-1, 1, n)
    np.testing.assert_array_equal(cuda.spmv(m, x).cpu().numpy(), ref.spmv(x))
    np.testing.assert_array_equal(m.rhs().cpu().numpy(), ref.rhs())
    b = ref.rhs()
    r, nrm = cuda.residual(m, b, x)
    rr = b - ref.spmv(x)
    np.testing.assert_array_equal(r.cpu().numpy(), rr)
    assert abs(nrm - rr @ rr) <= 1e-13 * (rr @ rr)


# with engine 1, even axis-2 lengths run the plane-marching kernel (x planes
# staged by TMA); the cases cover partial tiles on both plane axes, single
# planes, tiny grids and several slabs per column of tiles (the 1600 x 64
# planes); odd lengths fall back to the thread-per-cell kernel
PLANE_DIMS = [(6, 9, 130), (1, 17, 66), (2, 1, 2), (12, 1600, 64), (70, 3, 64), (3, 8, 192),
              (5, 7, 9)]


@pytest.fixture(params=[0, 1], ids=["cells", "planes"])
def stencil_engine(cuda, request):
    before = cuda.stencil_engine()
    cuda.stencil_engine(request.param)
    yield request.param
    cuda.stencil_engine(before)


@pytest.mark.parametrize("dims", PLANE_DIMS)
@pytest.mark.parametrize("valuator", ["lookup", "value"])
def test_stencil_engines_bitexact(cuda, stencil_engine, dims, valuator):
    n = int(np.prod(dims))
    q = lo.axis_quotients(dims, (1.1, 0.9, 1.7))
    if valuator == "lookup":
        mat = _lookup_case(dims, 13)
        coeffs = (0.5, 1.0, 2.0, 3.0)
        ref = lo.Stencil(dims, q=q, mat=mat, coeffs=coeffs, sol_start=1.0, sol_end=0.25)
        m = cuda.StencilMatrix.lookup(dims, q, coeffs, mat, 1.0, 0.25)
    else:
        k = np.exp(np.random.default_rng(10).standard_normal(n))
        ref = lo.Stencil(dims, q=q, k=k, sol_start=1.0, sol_end=0.0)
        m = cuda.StencilMatrix.value(dims, q, k, 1.0, 0.0)
    x = np.random.default_rng(11).uniform(-1, 1, n)
    np.testing.assert_array_equal(cuda.spmv(m, x).cpu().numpy(), ref.spmv(x))
    b = np.random.default_rng(12).uniform(-1, 1, n)
    r, nrm = cuda.residual(m, b, x)
    rr = b - ref.spmv(x)
    np.testing.assert_array_equal(r.cpu().numpy(), rr)
    assert abs(nrm - rr @ rr) <= 1e-13 * (rr @ rr)


def test_stencil_engine_rejects_unknown(cuda):
    with pytest.raises(cuda.LinealError):
        cuda.stencil_engine(2)


def test_reductions(cuda):
    rng = np.random.default_rng(0)
    for n in (1, 255, 256 * 8 + 3, 1 << 20):
        a = rng.uniform(-1, 1, n)
        b = rng.uniform(-1, 1, n)
        assert abs(cuda.dot(a, b) - np.dot(a, b)) <= 1e-12 * max(1.0, np.abs(a * b).sum())
        assert cuda.max_norm(a) == np.abs(a).max()
        d1 = cuda.dot(a, b)
        assert cuda.dot(a, b) == d1  # deterministic


def test_empty_and_tiny(cuda):
    m = cuda.CsrMatrix.from_host(np.array([0, 1]), np.array([0]), np.array([4.0]))
    np.testing.assert_array_equal(cuda.spmv(m, [2.0]).cpu().numpy(), [8.0])
    e = cuda.CsrMatrix.from_host(np.array([0]), np.array([], dtype=np.int32), np.array([]))
    assert e.row_num() == 0
    assert cuda.spmv(e, np.zeros(0)).numel() == 0


def test_invalid_csr_rejected(cuda):
    # missing diagonal / unsorted columns are reported, not computed
    with pytest.raises(cuda.LinealError):
        cuda.CsrMatrix.from_host(np.array([0, 1, 2]), np.array([1, 0]), np.array([1.0, 1.0]))
    with pytest.raises(cuda.LinealError):
        cuda.CsrMatrix.from_host(np.array([0, 2]), np.array([0, 0]), np.array([1.0, 1.0]))


def _diagonal_lines(dims):
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    return ((j + k) % 4).ravel().astype(np.uint8)


@pytest.mark.parametrize("zero_to_one", [True, False])
def test_effective_diffusion_matches_oracle(cuda, zero_to_one):
    """EffDiffCalc on the reference suite's system (test/shared-stencil.hpp:
    69-104, 225-238): the cross-section mean of the coefficients
    (materials.hpp:236-250), on the stencil (ZeroToOne) or on the
    compressed CSR system (ZeroToZero, compress map)."""
    dims, coeffs, lengths = (4, 9, 7), (0.0, 1.0, 2.0, 3.0), (4.0, 9.0, 7.0)
    q = lo.axis_quotients(dims, lengths)
    mat = _diagonal_lines(dims)
    st = cuda.StencilMatrix.lookup(cuda.BoxInfo(dims, lengths), None, coeffs, mat, 1.0, 0.0,
                                   zero_to_one)
    ref = lo.Stencil(dims, q=q, mat=mat, coeffs=coeffs, sol_start=1.0, sol_end=0.0,
                     zero_to_one=zero_to_one)
    if zero_to_one:
        res = cuda.pcg(st, st.rhs(), precon=cuda.PRECON_JACOBI, rtol=1e-14, maxit=2000)
        cmap = None
    else:
        csr, cmap = st.to_csr(with_compress_map=True)
        rhs = st.rhs()[cmap >= 0]
        res = cuda.pcg(csr, rhs, precon=cuda.PRECON_JACOBI, rtol=1e-14, maxit=2000)
    eff, area = st.effective_diffusion(lengths, res.x, compress_map=cmap)
    j, k = np.meshgrid(np.arange(9), np.arange(7), indexing="ij")
    assert area == 1.0
    assert abs(eff - np.mean(np.asarray(coeffs)[(j + k) % 4])) <= 1e-12
    want, want_area = ref.effective_diffusion(
        lengths, res.x.cpu().numpy(), None if cmap is None else cmap.cpu().numpy())
    assert area == want_area and abs(eff - want) <= 1e-13 * abs(want)
    # a "none" material leaves the area part
    eff0, area0 = st.effective_diffusion(lengths, res.x, compress_map=cmap, none_mask=1)
    assert area0 == pytest.approx(1.0 - np.mean((j + k) % 4 == 0))


def test_stencil_values_bitexact(cuda, stencil_engine):
    dims = (6, 7, 10)
    n = int(np.prod(dims))
    rng = np.random.default_rng(22)
    ks = [np.exp(rng.standard_normal(n)) for _ in range(3)]
    q = lo.axis_quotients(dims, (1.5, 0.7, 2.0))
    ref = lo.Stencil(dims, q=q, k_axes=ks, sol_start=1.0, sol_end=0.25)
    m = cuda.StencilMatrix.values(cuda.BoxInfo(dims, (1.5, 0.7, 2.0)), None, ks, 1.0, 0.25)
    x = rng.uniform(-1, 1, n)
    np.testing.assert_array_equal(cuda.spmv(m, x).cpu().numpy(), ref.spmv(x))
    np.testing.assert_array_equal(m.diagonal().cpu().numpy(), ref.diagonal())
    np.testing.assert_array_equal(m.rhs().cpu().numpy(), ref.rhs())
    csr, _ = m.to_csr(with_compress_map=True)
    rcsr, _ = ref.to_csr()
    rowptr, col, val = csr.download()
    np.testing.assert_array_equal(rowptr, rcsr.rowptr)
    np.testing.assert_array_equal(col, rcsr.col)
    np.testing.assert_array_equal(val, rcsr.val)
    with pytest.raises(cuda.LinealError):
        m.effective_diffusion((6.0, 7.0, 10.0), x)


def test_stencil_henry_bitexact(cuda, stencil_engine):
    dims = (6, 7, 10)
    mat = _lookup_case(dims, 25)
    coeffs = (0.5, 1.0, 2.0, 3.0)
    lengths = (6.0, 3.5, 10.0)
    q = lo.axis_quotients(dims, lengths)
    ref = lo.Stencil(dims, q=q, mat=mat, coeffs=coeffs, sol_start=1.0, sol_end=0.0, henry=0.3,
                     gaseous_mask=0b0110)
    m = cuda.StencilMatrix.lookup_henry(cuda.BoxInfo(dims, lengths), None, coeffs, mat, 0.3,
                                        0b0110, 1.0, 0.0)
    x = np.random.default_rng(26).uniform(-1, 1, ref.n)
    np.testing.assert_array_equal(cuda.spmv(m, x).cpu().numpy(), ref.spmv(x))
    np.testing.assert_array_equal(m.diagonal().cpu().numpy(), ref.diagonal())
    np.testing.assert_array_equal(m.rhs().cpu().numpy(), ref.rhs())
    eff, area = m.effective_diffusion(lengths, x, none_mask=0b1000)
    want, want_area = ref.effective_diffusion(lengths, x, none_mask=0b1000)
    assert area == want_area and abs(eff - want) <= 1e-13 * abs(want)
