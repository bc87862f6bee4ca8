"""The index arithmetic of the grid finest-level kernels (lineal_gb300/csrc/
lgx_grid.cu), restated here and checked against the oracle's grid matrices
in the colour order the multicolour smoother uses (rows sorted by colour,
then by index):

* 27 points, parity colouring c = 4(i&1) + 2(j&1) + (k&1) with even edges:
  the neighbour of row r at offset (dz, dy, dx) sits at r + delta[c][e];
* 7 points, red-black colouring c = (i+j+k)&1 with an even n2: with
  q = r - cB, s = (c+i+j)&1, the neighbours sit at (1-c)B + q -+ n1 h2,
  (1-c)B + q -+ h2, (1-c)B + q - 1 + s and (1-c)B + q + s.
"""

import numpy as np
import pytest

import oracle as lo


def _colour_order(colours):
    """new index of every row when rows are sorted by (colour, index)"""
    order = np.lexsort((np.arange(len(colours)), colours))
    new = np.empty_like(order)
    new[order] = np.arange(len(order))
    return new


def _delta27(n1, n2, block):
    h1, h2 = n1 // 2, n2 // 2
    d = np.zeros((8, 27), dtype=np.int64)
    for c in range(8):
        pi, pj, pk = c >> 2, (c >> 1) & 1, c & 1
        for e in range(27):
            dz, dy, dx = e // 9 - 1, (e // 3) % 3 - 1, e % 3 - 1
            c2 = ((pi + dz) & 1) * 4 + ((pj + dy) & 1) * 2 + ((pk + dx) & 1)
            fz, fy, fx = (pi + dz) // 2, (pj + dy) // 2, (pk + dx) // 2
            d[c, e] = (c2 - c) * block + (fz * h1 + fy) * h2 + fx
    return d


@pytest.mark.parametrize("dims", [(2, 2, 2), (4, 6, 8), (6, 2, 4)])
def test_parity_27pt_neighbours_are_row_plus_delta(dims):
    n0, n1, n2 = dims
    n = n0 * n1 * n2
    a = lo.gen_27pt(dims, np.ones(n))
    i, j, k = np.unravel_index(np.arange(n), dims)
    colour = 4 * (i & 1) + 2 * (j & 1) + (k & 1)
    new = _colour_order(colour)
    delta = _delta27(n1, n2, n // 8)
    for r in range(n):
        cols = a.col[a.rowptr[r]:a.rowptr[r + 1]]
        assert len(cols) == np.prod([1 + (x > 0) + (x < d - 1) for x, d in zip(
            (i[r], j[r], k[r]), dims)])
        for cc in cols:
            dz, dy, dx = i[cc] - i[r], j[cc] - j[r], k[cc] - k[r]
            e = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)
            assert new[cc] == new[r] + delta[colour[r], e]


@pytest.mark.parametrize("dims", [(1, 1, 2), (3, 5, 4), (5, 7, 4), (4, 3, 6)])
def test_red_black_7pt_neighbours(dims):
    n0, n1, n2 = dims
    n = n0 * n1 * n2
    a = lo.gen_7pt(dims, np.ones(n))
    i, j, k = np.unravel_index(np.arange(n), dims)
    colour = (i + j + k) & 1
    new = _colour_order(colour)
    block, h2 = n // 2, n2 // 2
    assert np.count_nonzero(colour == 0) == block
    for r in range(n):
        c = colour[r]
        q = new[r] - c * block
        s = (c + i[r] + j[r]) & 1
        assert q // h2 == i[r] * n1 + j[r] and k[r] == 2 * (q % h2) + s
        other = (1 - c) * block + q
        want = {(-1, 0, 0): other - n1 * h2, (1, 0, 0): other + n1 * h2,
                (0, -1, 0): other - h2, (0, 1, 0): other + h2,
                (0, 0, -1): other - 1 + s, (0, 0, 1): other + s, (0, 0, 0): new[r]}
        cols = a.col[a.rowptr[r]:a.rowptr[r + 1]]
        for cc in cols:
            off = (int(i[cc] - i[r]), int(j[cc] - j[r]), int(k[cc] - k[r]))
            assert new[cc] == want[off]


def _unvisited27(c):
    """g27_unvisited<27>: offsets whose neighbours lie in colours after c"""
    m = 0
    for e in range(27):
        if e == 13:
            continue
        dz, dy, dx = e // 9 - 1, (e // 3) % 3 - 1, e % 3 - 1
        if c ^ (4 * (dz != 0) + 2 * (dy != 0) + (dx != 0)) > c:
            m |= 1 << e
    return m


def _unvisited7(c):
    """g27_unvisited<7>: every off-diagonal offset for colour 0, none for 1"""
    return sum(1 << e for e in range(7) if e != 3 and 1 - c > c)


@pytest.mark.parametrize("dims", [(2, 2, 2), (4, 6, 8), (6, 4, 10)])
def test_unvisited_masks_match_row_order_27pt(dims):
    """A forward sweep from zero reads a neighbour as 0 when its row sits at
    or past the first row of the launch's colour; the grid kernels test the
    per-colour offset mask instead.  Both agree on every in-grid entry."""
    n = int(np.prod(dims))
    a = lo.gen_27pt(dims, np.ones(n))
    i, j, k = np.unravel_index(np.arange(n), dims)
    colour = 4 * (i & 1) + 2 * (j & 1) + (k & 1)
    new = _colour_order(colour)
    block = n // 8
    for r in range(n):
        c = int(colour[r])
        m = _unvisited27(c)
        for cc in a.col[a.rowptr[r]:a.rowptr[r + 1]]:
            if cc == r:
                continue
            e = (i[cc] - i[r] + 1) * 9 + (j[cc] - j[r] + 1) * 3 + (k[cc] - k[r] + 1)
            assert bool((m >> e) & 1) == (new[cc] >= c * block)


@pytest.mark.parametrize("dims", [(3, 5, 4), (4, 3, 6), (2, 2, 2)])
def test_unvisited_masks_match_row_order_7pt(dims):
    n = int(np.prod(dims))
    a = lo.gen_7pt(dims, np.ones(n))
    i, j, k = np.unravel_index(np.arange(n), dims)
    colour = (i + j + k) & 1
    new = _colour_order(colour)
    block = n // 2
    offsets = [(-1, 0, 0), (0, -1, 0), (0, 0, -1), (0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 0)]
    for r in range(n):
        c = int(colour[r])
        m = _unvisited7(c)
        for cc in a.col[a.rowptr[r]:a.rowptr[r + 1]]:
            if cc == r:
                continue
            e = offsets.index((int(i[cc] - i[r]), int(j[cc] - j[r]), int(k[cc] - k[r])))
            assert bool((m >> e) & 1) == (new[cc] >= c * block)
