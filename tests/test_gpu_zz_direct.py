"""The standalone direct solver (lgx_direct_*: CholeskySolver and LuSolver,
direct/cholesky/solver.hpp:22-67, direct/lu/solver.hpp:21-66) against the
reference's Cholesky golden solve and the UFZ_CT_02 system, the banded
Cholesky beyond the dense limit, its refusals, and the C++ concept layer's
CholeskySolver/LuSolver program."""

import os
import subprocess

import numpy as np
import pytest

import oracle as lo
from lineal_gb300 import io as lio

pytestmark = pytest.mark.gpu


def _dev(cuda, a, symmetric):
    return cuda.CsrMatrix.from_host(a.rowptr, a.col, a.val, symmetric=symmetric)


def test_cholesky_golden_solve(cuda, golden_dir):
    c = np.load(os.path.join(golden_dir, "cholesky_python_reference.npz"))
    lhs = c["lhs"]
    rows, cols = np.nonzero(lhs)
    rowptr = np.zeros(lhs.shape[0] + 1, dtype=np.int64)
    np.add.at(rowptr, rows + 1, 1)
    a = lo.Csr(np.cumsum(rowptr), cols.astype(np.int32), lhs[rows, cols])
    d = cuda.DirectSolver(_dev(cuda, a, True))
    x = d.solve(c["rhs"]).cpu().numpy()
    # test/python-reference/cholesky.py's solution; an explicit inverse
    # carries about cond(A) * eps (cond 441)
    np.testing.assert_allclose(x, c["sol"], rtol=0, atol=1e-12 * np.abs(c["sol"]).max())


@pytest.mark.parametrize("lu", [True, False])
def test_ufz_system(cuda, golden_dir, lu):
    rowptr, col, val, _ = lio.read_smf(os.path.join(golden_dir, "UFZ_CT_02_LHS.smf"))
    b = lio.read_dvf(os.path.join(golden_dir, "UFZ_CT_02_RHS.dvf"))
    a = lo.Csr(rowptr, col, val, symmetric=False)
    d = cuda.DirectSolver(_dev(cuda, a, False), lu=lu)
    x = d.solve(b).cpu().numpy()
    assert np.linalg.norm(b - lo.spmv(a, x)) <= 1e-12 * np.linalg.norm(b)
    # against the oracle's unpivoted LU (lu/decomposition.hpp)
    ref = lo.lu_solve(lo.lu_factor(a), b)
    np.testing.assert_allclose(x, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def _tridiagonal(n, lower, diag, upper):
    rowptr, col, val = [0], [], []
    for i in range(n):
        for j, v in ((i - 1, lower), (i, diag), (i + 1, upper)):
            if 0 <= j < n:
                col.append(j)
                val.append(v)
        rowptr.append(len(col))
    return lo.Csr(np.array(rowptr, np.int64), np.array(col, np.int32), np.array(val))


def test_refusals(cuda):
    indefinite = _dev(cuda, _tridiagonal(8, -1.0, 0.5, -1.0), True)
    with pytest.raises(cuda.LinealError, match="non-positive pivot"):
        cuda.DirectSolver(indefinite, lu=False)
    lu = cuda.DirectSolver(indefinite, lu=True)
    x = lu.solve(np.ones(8)).cpu().numpy()
    a = _tridiagonal(8, -1.0, 0.5, -1.0)
    assert np.linalg.norm(1.0 - lo.spmv(a, x)) <= 1e-12 * np.sqrt(8)
    zero_pivot = _dev(cuda, _tridiagonal(6, 1.0, 0.0, 1.0), False)
    with pytest.raises(cuda.LinealError, match="zero, non-finite or tiny pivot"):
        cuda.DirectSolver(zero_pivot, lu=True)
    big = cuda.gen_7pt((32, 32, 9), np.ones(32 * 32 * 9))
    with pytest.raises(cuda.LinealError, match="at most"):
        cuda.DirectSolver(big, lu=True)
    d = cuda.DirectSolver(_dev(cuda, _tridiagonal(4, -1.0, 2.0, -1.0), True))
    with pytest.raises(ValueError):
        d.solve(np.ones(5))


def test_cpp_direct_solvers(cuda):
    from lineal_gb300 import build

    exe = build.build_cpp_demo(name="direct_demo")
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "direct_demo ok" in out.stdout


@pytest.mark.parametrize("dims,npts", [((30, 30, 12), 7), ((24, 24, 16), 27), ((96, 10, 10), 7)])
def test_banded_cholesky_beyond_dense_limit(cuda, dims, npts):
    """More rows than the dense limit: the Cholesky factor in the band of the
    lower envelope (natural order; bandwidth n1 n2 for 7 points, n1 n2 +
    n2 + 1 for 27), then a forward and a backward substitution.  Solutions
    of A x = A x_true agree with x_true to the conditioning's reach and the
    FP64 residual is small; the factor is reused across solves."""
    n = int(np.prod(dims))
    assert n > cuda.DIRECT_MAX_ROWS
    k = np.exp(np.random.default_rng(8).standard_normal(n))
    ref = (lo.gen_27pt if npts == 27 else lo.gen_7pt)(dims, k)
    m = (cuda.gen_27pt if npts == 27 else cuda.gen_7pt)(dims, k)
    d = cuda.DirectSolver(m)
    rng = np.random.default_rng(9)
    for _ in range(2):
        xt = rng.uniform(-1, 1, n)
        b = lo.spmv(ref, xt)
        x = d.solve(b).cpu().numpy()
        assert np.linalg.norm(b - lo.spmv(ref, x)) <= 1e-12 * np.linalg.norm(b)
        assert np.linalg.norm(x - xt) <= 1e-9 * np.linalg.norm(xt)


def test_banded_cholesky_refuses_indefinite(cuda):
    dims = (30, 30, 12)
    n = int(np.prod(dims))
    ref = lo.gen_7pt(dims, np.ones(n))
    val = ref.val.copy()
    # one negative diagonal entry deep inside the matrix
    row = n // 2
    for e in range(ref.rowptr[row], ref.rowptr[row + 1]):
        if ref.col[e] == row:
            val[e] = -1.0
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, val, symmetric=True)
    with pytest.raises(cuda.LinealError, match="non-positive pivot"):
        cuda.DirectSolver(m)
