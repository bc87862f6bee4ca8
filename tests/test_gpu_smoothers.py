"""GPU parity of the smoothers and the colouring.

The multicolour SOR sweep equals the reference SOR run in the row order
"sorted by (colour, index)" (oracle lo_sor_sweep_ordered), bit for bit.
"""

import os

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu


def _case(dims=(9, 10, 11), seed=1, npts=27):
    n = int(np.prod(dims))
    k = np.exp(1.5 * np.random.default_rng(seed).standard_normal(n))
    ref = (lo.gen_27pt if npts == 27 else lo.gen_7pt)(dims, k)
    return ref, k


@pytest.mark.parametrize("relax", [1.0, 0.8])
def test_jacobi_bitexact(cuda, relax):
    ref, _ = _case()
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    rng = np.random.default_rng(3)
    b = rng.uniform(-1, 1, ref.n)
    x = rng.uniform(-1, 1, ref.n)
    np.testing.assert_array_equal(cuda.jacobi_sweep(m, b, x, relax).cpu().numpy(),
                                  lo.jacobi_sweep(ref, b, x, relax))
    np.testing.assert_array_equal(cuda.jacobi_sweep(m, b, None, relax).cpu().numpy(),
                                  lo.jacobi_sweep(ref, b, None, relax))


def test_stencil_jacobi_from_zero(cuda):
    dims = (6, 7, 8)
    mat = np.random.default_rng(4).integers(0, 4, int(np.prod(dims))).astype(np.uint8)
    ref = lo.Stencil(dims, mat=mat)
    a, _ = ref.to_csr()
    m = cuda.StencilMatrix.lookup(dims, (1, 1, 1), (0, 1, 2, 3), mat)
    b = np.random.default_rng(5).uniform(-1, 1, ref.n)
    np.testing.assert_array_equal(cuda.jacobi_sweep(m, b, None, 0.7).cpu().numpy(),
                                  lo.jacobi_sweep(a, b, None, 0.7))


@pytest.mark.parametrize("npts", [27, 7])
def test_jp_colouring_matches_oracle(cuda, npts):
    ref, _ = _case(npts=npts)
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    c = cuda.Colouring.jp(m, seed=123)
    colours, nc = c.export()
    rc, rnc = lo.colour_jp(ref, 123)
    np.testing.assert_array_equal(colours.cpu().numpy(), rc)
    assert nc == rnc


@pytest.mark.parametrize("relax", [0.9, 1.0])
@pytest.mark.parametrize("forward", [True, False])
@pytest.mark.parametrize("ultra", [False, True])
@pytest.mark.parametrize("with_input", [False, True])
def test_multicolour_sor_bitexact(cuda, forward, ultra, with_input, relax):
    ref, _ = _case()
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    col = cuda.Colouring.jp(m, seed=7)
    colours, nc = col.export()
    order = lo.colour_order(colours.cpu().numpy(), nc)
    rng = np.random.default_rng(11)
    b = rng.uniform(-1, 1, ref.n)
    x_in = rng.uniform(-1, 1, ref.n) if with_input else None
    got = cuda.sor_sweep(m, col, b, x_in, relax=relax, forward=forward, ultra=ultra)
    want = lo.sor_sweep(ref, b, x_in=x_in, relax=relax, forward=forward, ultra=ultra,
                        order=order)
    np.testing.assert_array_equal(got.cpu().numpy(), want)


def test_parity_colouring_of_grid(cuda):
    # the analytic 8-colouring of a 27-point grid: colour = (i%2) + 2(j%2) + 4(k%2)
    dims = (8, 6, 10)
    ref, _ = _case(dims)
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    colours = ((i % 2) * 4 + (j % 2) * 2 + (k % 2)).ravel().astype(np.int32)
    col = cuda.Colouring.from_array(m, colours, 8)
    order = lo.colour_order(colours, 8)
    b = np.random.default_rng(2).uniform(-1, 1, ref.n)
    got = cuda.sor_sweep(m, col, b, None, relax=1.0, forward=True)
    np.testing.assert_array_equal(got.cpu().numpy(),
                                  lo.sor_sweep(ref, b, relax=1.0, forward=True, order=order))


def test_invalid_colouring_rejected(cuda):
    ref, _ = _case((4, 4, 4))
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    with pytest.raises(cuda.LinealError):
        cuda.Colouring.from_array(m, np.zeros(ref.n, dtype=np.int32), 1)


def test_sor_python_reference_problem_converges(cuda, golden_dir):
    # the sor.py system, solved by repeated multicolour SOR sweeps
    g = np.load(os.path.join(golden_dir, "sor_python_reference.npz"))
    s = lo.Stencil(g["dims"], mat=g["materials"], coeffs=g["coeffs"])
    a, _ = s.to_csr()
    m = cuda.CsrMatrix.from_host(a.rowptr, a.col, a.val)
    col = cuda.Colouring.jp(m)
    x = np.zeros(a.n)
    for _ in range(400):
        x = cuda.sor_sweep(m, col, g["rhs"], x).cpu().numpy()
    np.testing.assert_allclose(x, g["x_true"], rtol=1e-8)
