"""The CSR row engine across its configurations: every configuration gives
the oracle's results bit for bit on a ragged grid matrix (many tiles, odd row
counts), on matrices whose 32-row windows exceed a warp stage (CTA-tile
fallback) and whose rows exceed a CTA stage (unstaged rows), and through the
permuted-order SOR entry points in FP64 and float."""

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu

CONFIGS = list(range(8))


@pytest.fixture
def engine(cuda):
    saved = cuda.row_engine()
    yield cuda
    cuda.row_engine(saved)


def _grid(dims=(37, 41, 43), seed=2):
    n = int(np.prod(dims))
    k = np.exp(1.5 * np.random.default_rng(seed).standard_normal(n))
    return lo.gen_27pt(dims, k)


def _long_rows(n=9000, seed=9):
    """Symmetric-pattern matrix with a band of dense rows: rows 100..163 hold
    1500 entries each (any 32-row window there exceeds a warp stage), row 2000
    holds all 9000 columns (more than a CTA stage holds)."""
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(n):
        if 100 <= i < 164:
            cols = np.sort(rng.choice(n, 1500, replace=False))
        elif i == 2000:
            cols = np.arange(n)
        else:
            cols = np.sort(rng.choice(n, 6, replace=False))
        cols = np.union1d(cols, [i]).astype(np.int32)
        rows.append(cols)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    rowptr[1:] = np.cumsum([len(c) for c in rows])
    col = np.concatenate(rows)
    val = rng.uniform(-1, 1, len(col))
    val[np.concatenate([np.flatnonzero(c == i) + rowptr[i] for i, c in enumerate(rows)])] = 50.0
    return lo.Csr(rowptr, col, val, symmetric=False)


@pytest.mark.parametrize("config", CONFIGS)
def test_spmv_residual_grid(engine, config):
    engine.row_engine(config)
    ref = _grid()
    m = engine.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    rng = np.random.default_rng(config)
    x = rng.uniform(-1, 1, ref.n)
    b = rng.uniform(-1, 1, ref.n)
    np.testing.assert_array_equal(engine.spmv(m, x).cpu().numpy(), lo.spmv(ref, x))
    r, nrm = engine.residual(m, b, x)
    want = lo.residual(ref, b, x)
    np.testing.assert_array_equal(r.cpu().numpy(), want)
    assert abs(nrm - want @ want) <= 1e-13 * (want @ want)


@pytest.mark.parametrize("config", CONFIGS)
def test_long_rows(engine, config):
    engine.row_engine(config)
    ref = _long_rows()
    m = engine.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=False)
    x = np.random.default_rng(1).uniform(-1, 1, ref.n)
    b = np.random.default_rng(2).uniform(-1, 1, ref.n)
    np.testing.assert_array_equal(engine.spmv(m, x).cpu().numpy(), lo.spmv(ref, x))
    r, _ = engine.residual(m, b, x)
    np.testing.assert_array_equal(r.cpu().numpy(), lo.residual(ref, b, x))
    np.testing.assert_array_equal(engine.jacobi_sweep(m, b, x, 0.7).cpu().numpy(),
                                  lo.jacobi_sweep(ref, b, x, 0.7))


@pytest.mark.parametrize("config", [1, 3, 5])
@pytest.mark.parametrize("forward", [True, False])
def test_sor_permuted_matches_natural_and_oracle(engine, config, forward):
    engine.row_engine(config)
    ref = _grid((21, 19, 23))
    m = engine.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    col = engine.Colouring.jp(m, seed=5)
    colours, nc = col.export()
    order = lo.colour_order(colours.cpu().numpy(), nc)
    rng = np.random.default_rng(7)
    b = rng.uniform(-1, 1, ref.n)
    x = rng.uniform(-1, 1, ref.n)
    natural = engine.sor_sweep(m, col, b, x, relax=0.9, forward=forward)
    xp = engine.permute(col, x)
    engine.sor_sweep_permuted(col, engine.permute(col, b), xp, relax=0.9, forward=forward)
    np.testing.assert_array_equal(engine.unpermute(col, xp).cpu().numpy(),
                                  natural.cpu().numpy())
    # float smoother: bit-exact with the oracle's float sweep
    import torch

    xp32 = engine.permute(col, x).float()
    bp32 = engine.permute(col, b).float()
    engine.sor_sweep_permuted(col, bp32, xp32, relax=0.9, forward=forward)
    got32 = engine.unpermute(col, xp32.double()).cpu().numpy()
    want32 = lo.sor_sweep_f32(ref, b.astype(np.float32), order, x_in=x.astype(np.float32),
                              relax=0.9, forward=forward)
    np.testing.assert_array_equal(got32, want32.astype(np.float64))
    assert torch.isfinite(xp32).all()


def test_row_engine_rejects_unknown_configuration(cuda):
    with pytest.raises(cuda.LinealError):
        cuda.row_engine(8)


@pytest.mark.parametrize("relax", [1.0, 0.7])
def test_sor_division_through_reciprocals(engine, relax):
    """The FP64 sweep divides through a table of correctly rounded
    reciprocals; two million rows of a 7-point matrix with diagonals spread
    over 2^-30..2^30 and right-hand sides over 2^-300..2^300 (some beyond
    2^400, which take the direct division) give the oracle's quotients."""
    dims = (128, 128, 128)
    n = int(np.prod(dims))
    rng = np.random.default_rng(21)
    k = np.exp(rng.uniform(-20.0, 20.0, n))
    ref = lo.gen_7pt(dims, k)
    m = engine.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    colours = ((np.arange(n) % 128) + (np.arange(n) // 128) % 128 + np.arange(n) // 16384) % 2
    col = engine.Colouring.from_array(m, colours.astype(np.int32), 2)
    order = lo.colour_order(colours.astype(np.int32), 2)
    b = rng.uniform(-1, 1, n) * np.exp2(rng.uniform(-300, 300, n))
    b[::1000] *= 2.0 ** 500
    x = rng.uniform(-1, 1, n)
    got = engine.sor_sweep(m, col, b, x, relax=relax).cpu().numpy()
    want = lo.sor_sweep(ref, b, x_in=x, relax=relax, order=order)
    np.testing.assert_array_equal(got, want)
