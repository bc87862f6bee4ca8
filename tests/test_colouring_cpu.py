"""The host smallest-last colouring (lgx_colour_smallest_last; no device
work, so it runs without a GPU) against the oracle's restatement of the same
procedure, bit for bit, and the properties that make it a smoother
colouring: proper on the symmetric pattern, fewer colours than
Jones-Plassmann on coarse AMG levels."""

import numpy as np
import pytest

import lineal_gb300 as g
import oracle as lo


def _proper(a, colour):
    rows = np.repeat(np.arange(a.n), np.diff(a.rowptr))
    off = a.col != rows
    return not np.any(colour[rows[off]] == colour[a.col[off]])


@pytest.mark.parametrize("case", ["27pt", "7pt", "ufz", "coarse"])
def test_library_equals_oracle(case, golden_dir):
    import os

    from lineal_gb300 import io as lio

    if case == "ufz":
        rowptr, col, val, _ = lio.read_smf(os.path.join(golden_dir, "UFZ_CT_02_LHS.smf"))
        a = lo.Csr(rowptr, col, val, symmetric=False)
    elif case == "coarse":
        k = np.exp(1.5 * np.random.default_rng(1).standard_normal(24 ** 3))
        h = lo.Amg(lo.gen_27pt((24, 24, 24), k), min_coarsen_size=50, partition_size=512,
                   smoother_parts=0)
        a = h.level_csr(1)
    else:
        dims = (9, 10, 11)
        k = np.exp(np.random.default_rng(2).standard_normal(990))
        a = (lo.gen_27pt if case == "27pt" else lo.gen_7pt)(dims, k)
    got, nc = g.colour_smallest_last(a.rowptr, a.col)
    want, wnc = lo.colour_smallest_last(a)
    np.testing.assert_array_equal(got, want)
    assert nc == wnc == got.max() + 1
    assert _proper(a, got)
    if case == "7pt":
        assert nc == 2  # a bipartite grid graph
    if case == "coarse":
        _, jp = lo.colour_jp(a, 0x5EED)
        assert nc < jp


def test_edge_cases():
    c, nc = g.colour_smallest_last(np.zeros(1, np.int64), np.zeros(0, np.int32))
    assert len(c) == 0 and nc == 0
    # diagonal only: one colour
    c, nc = g.colour_smallest_last(np.arange(4, dtype=np.int64), np.arange(3, dtype=np.int32))
    assert nc == 1 and not c.any()
    with pytest.raises(g.LinealError):
        g.colour_smallest_last(np.array([0, 1], np.int64), np.array([5], np.int32))
    with pytest.raises(g.LinealError):
        g.colour_smallest_last(np.array([0, 2, 1], np.int64), np.array([0, 1], np.int32))


def test_oracle_amg_with_smallest_last_coarse_levels():
    """The oracle's AMG-PCG with smallest-last colourings on the coarse
    levels: fewer colours per coarse sweep than Jones-Plassmann, iteration
    count within one of it (32^3 27-point, lognormal sigma 1.5)."""
    n = 32 ** 3
    a = lo.gen_27pt((32, 32, 32), np.exp(1.5 * np.random.default_rng(1).standard_normal(n)))
    b = np.random.default_rng(0).uniform(-1, 1, n)
    its, colours = [], []
    for sl in (0, 1):
        h = lo.Amg(a, min_coarsen_size=2000, smoother_parts=0, coarse_smallest_last=sl)
        m = h.level_csr(1)
        colours.append(lo.colour_smallest_last(m)[1] if sl else lo.colour_jp(m, 0x5EED + 1)[1])
        order = h.level_order(1)
        assert order is not None and sorted(order.tolist()) == list(range(m.n))
        _, it, hist = lo.pcg(a, b, precon=lo.PRECON_AMG, amg=h, rtol=1e-8, maxit=200)
        assert hist[-1] <= 1e-8 * hist[0]
        its.append(it)
    assert colours[1] < colours[0]
    assert abs(its[1] - its[0]) <= 1


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_structurally_nonsymmetric_pattern_colours_a_plus_at(seed):
    """A pattern with (i, j) stored but not (j, i): both colourings work on
    the pattern of A + A^T, agree bit for bit and are proper for every edge
    in either direction (the multicolour sweep reads both)."""
    rng = np.random.default_rng(seed)
    n = 300
    rows = []
    for i in range(n):
        cols = {i}
        cols.update(int(c) for c in rng.integers(0, n, rng.integers(0, 6)))
        rows.append(sorted(cols))
    rowptr = np.zeros(n + 1, np.int64)
    rowptr[1:] = np.cumsum([len(r) for r in rows])
    col = np.concatenate([np.asarray(r, np.int32) for r in rows])
    a = lo.Csr(rowptr, col, np.ones(len(col)), symmetric=False)
    got, nc = g.colour_smallest_last(rowptr, col)
    want, wnc = lo.colour_smallest_last(a)
    np.testing.assert_array_equal(got, want)
    assert nc == wnc
    r = np.repeat(np.arange(n), np.diff(rowptr))
    off = col != r
    assert not np.any(got[r[off]] == got[col[off]])
    # the pattern really is nonsymmetric
    pairs = set(zip(r[off].tolist(), col[off].tolist()))
    assert any((j, i) not in pairs for i, j in pairs)
