"""Pins the CPU restatement (oracle/) against the reference's own golden data.

* test/python-reference/sor.py: matrix and all 128 SOR iterates
  (tests/golden/sor_python_reference.npz, generated by make_golden.py).
* test/python-reference/cholesky.py: factor and solves.
* test/data/UFZ_CT_02_{LHS.smf,RHS.dvf}: a real CSR system.
* the residual/error bound tables of test/shared-stencil.hpp:157-180 and
  201-224 (4x9x7 grid, diagonal_lines materials, coefficients 0..3).
"""

import os

import numpy as np
import pytest

import oracle as lo
from lineal_gb300 import io as lio


@pytest.fixture(scope="module")
def sor_golden(golden_dir):
    return np.load(os.path.join(golden_dir, "sor_python_reference.npz"))


def test_partition_blocks():
    # contiguous parts covering [0, n), sizes differing by at most one
    for n, p in [(10, 3), (252, 2), (7, 7), (1000, 64)]:
        b = [lo.lib().lo_part_begin(n, p, k) for k in range(p + 1)]
        sizes = np.diff(b)
        assert b[0] == 0 and b[-1] == n
        assert sizes.max() - sizes.min() <= 1


def test_sor_python_reference_matrix(sor_golden):
    g = sor_golden
    q = lo.axis_quotients(g["dims"], g["lengths"])
    mat = lo.material_flow_cylinder_gap(g["dims"], float(g["radius"]))
    assert np.array_equal(mat, g["materials"])
    s = lo.Stencil(g["dims"], q=q, mat=mat, coeffs=g["coeffs"], zero_to_one=True)
    a, _ = s.to_csr()
    # defs/diffusion_matrix.py sums the diagonal in another order: 1 ulp allowed
    np.testing.assert_allclose(a.to_dense(), g["lhs"], rtol=1e-15, atol=0)
    np.testing.assert_array_equal(s.spmv(g["x_true"]), g["lhs"] @ g["x_true"])


def test_sor_python_reference_iterates(sor_golden):
    g = sor_golden
    s = lo.Stencil(g["dims"], q=(1, 1, 1), mat=g["materials"], coeffs=g["coeffs"])
    a, _ = s.to_csr()
    x = np.zeros(a.n)
    for k in range(128):
        x = lo.sor_sweep(a, g["rhs"], x_in=x, relax=float(g["relax"]), nparts=1)
        ref = g["iterates"][k + 1]
        # sor.py evaluates relax/diag * (...) instead of (...)/diag: rounding only
        assert np.abs(x - ref).max() <= 1e-14 * np.abs(ref).max()


def test_cholesky_python_reference(golden_dir):
    c = np.load(os.path.join(golden_dir, "cholesky_python_reference.npz"))
    lhs = c["lhs"]
    n = lhs.shape[0]
    rows, cols = np.nonzero(lhs)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rowptr, rows + 1, 1)
    a = lo.Csr(np.cumsum(rowptr), cols.astype(np.int32), lhs[rows, cols])
    l = lo.cholesky_factor(a)
    np.testing.assert_allclose(l, c["chol"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(lo.cholesky_solve(l, c["rhs"]), c["sol"], rtol=0, atol=1e-13)


def test_ufz_io_roundtrip(golden_dir, tmp_path):
    lhs = os.path.join(golden_dir, "UFZ_CT_02_LHS.smf")
    rhs = os.path.join(golden_dir, "UFZ_CT_02_RHS.dvf")
    rowptr, col, val, ncols = lio.read_smf(lhs)
    assert (len(rowptr) - 1, ncols, len(val)) == (0x21B, 0x21B, 0xD27)  # tensor-io test sizes
    out = tmp_path / "m.smf"
    lio.write_smf(str(out), rowptr, col, val, ncols)
    assert out.read_bytes() == open(lhs, "rb").read()
    b = lio.read_dvf(rhs)
    assert len(b) == 539
    out2 = tmp_path / "v.dvf"
    lio.write_dvf(str(out2), b)
    assert out2.read_bytes() == open(rhs, "rb").read()


def _ufz(golden_dir):
    rowptr, col, val, _ = lio.read_smf(os.path.join(golden_dir, "UFZ_CT_02_LHS.smf"))
    b = lio.read_dvf(os.path.join(golden_dir, "UFZ_CT_02_RHS.dvf"))
    return lo.Csr(rowptr, col, val, symmetric=False), b


def test_ufz_spmv_and_solve(golden_dir):
    a, b = _ufz(golden_dir)
    x = np.linspace(-1, 1, a.n)
    np.testing.assert_allclose(lo.spmv(a, x), a.to_dense() @ x, rtol=1e-13, atol=1e-13)
    amg = lo.Amg(a, min_coarsen_size=32, partition_size=64, max_partitions=8,
                 smoother_parts=0)
    xs, it, hist = lo.pbicgstab(a, b, precon=lo.PRECON_AMG, amg=amg, rtol=1e-10, maxit=200)
    assert hist[-1] <= 1e-10 * hist[0]
    r = lo.residual(a, b, xs)
    assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(b)


def _stencil_system():
    dims = (4, 9, 7)
    mat = lo.material_diagonal_lines(dims, 4)
    s = lo.Stencil(dims, q=(1, 1, 1), mat=mat, coeffs=(0, 1, 2, 3), sol_start=1, sol_end=0)
    a, _ = s.to_csr()
    return s, a


def test_stencil_variants_agree():
    # shared-stencil.hpp:124-131: A*2 through every representation
    dims = (4, 9, 7)
    s, a = _stencil_system()
    mat = lo.material_diagonal_lines(dims, 4)
    sv = lo.Stencil(dims, k=np.array([0, 1, 2, 3.0])[mat], sol_start=1, sol_end=0)
    two = np.full(a.n, 2.0)
    np.testing.assert_array_equal(s.spmv(two), sv.spmv(two))
    np.testing.assert_allclose(s.spmv(two), lo.spmv(a, two), rtol=1e-14, atol=1e-14)
    np.testing.assert_array_equal(s.rhs(), sv.rhs())


# (name, iterations, kwargs, bound x=2, bound rhs); bounds from
# test/shared-stencil.hpp:157-180 and 201-224 (regular variant)
SUITE = [
    ("cg", 129, dict(), 1e-12, 1e-13),
    ("bicgstab", 129, dict(), 1e-12, 1e-13),
    ("pcg_ssor1", 129, dict(precon=lo.PRECON_SSOR, nparts=2), 1e-13, 1e-13),
    ("pbicgstab_ssor1", 129, dict(precon=lo.PRECON_SSOR, nparts=2), 1e-12, 1e-13),
    ("pcg_amg", 33, dict(precon=lo.PRECON_AMG), 1e-13, 2e-14),
    ("pbicgstab_amg", 33, dict(precon=lo.PRECON_AMG), 1e-13, 1e-13),
]


@pytest.mark.parametrize("name,iters,kw,bound_x2,bound_rhs", SUITE)
def test_stencil_suite_bounds(name, iters, kw, bound_x2, bound_rhs):
    s, a = _stencil_system()
    amg = lo.Amg(a, min_coarsen_size=32, partition_size=8, max_partitions=2, coarse_f32=1,
                 smoother_parts=2)
    kw = dict(kw)
    if kw.get("precon") == lo.PRECON_AMG:
        kw["amg"] = amg
    fn = lo.pcg if name.startswith(("cg", "pcg")) else lo.pbicgstab
    b2 = lo.spmv(a, np.full(a.n, 2.0))
    x, it, hist = fn(a, b2, rtol=0.0, maxit=iters, **kw)
    assert hist[-1] <= bound_x2 and np.abs(x - 2).max() <= bound_x2
    b = s.rhs()
    x, it, hist = fn(a, b, rtol=0.0, maxit=iters, **kw)
    assert hist[-1] <= bound_rhs and np.abs(lo.spmv(a, x) - b).max() <= bound_rhs


def test_sor_smoother_bounds():
    # "sor" entries: 129 in-situ sweeps, 2 thread partitions
    s, a = _stencil_system()
    for b, bound in ((lo.spmv(a, np.full(a.n, 2.0)), 1e-8), (s.rhs(), 1e-9)):
        x = np.zeros(a.n)
        for _ in range(129):
            x = lo.sor_sweep(a, b, x_in=x, nparts=2)
        assert np.linalg.norm(lo.spmv(a, x) - b) <= bound


def test_colouring_valid_and_deterministic():
    k = np.exp(np.random.default_rng(7).standard_normal(6 * 7 * 8))
    a = lo.gen_27pt((6, 7, 8), k)
    c1, n1 = lo.colour_jp(a, 11)
    c2, n2 = lo.colour_jp(a, 11)
    assert np.array_equal(c1, c2) and n1 == n2
    for i in range(a.n):
        for e in range(a.rowptr[i], a.rowptr[i + 1]):
            j = a.col[e]
            assert j == i or c1[j] != c1[i]
    order = lo.colour_order(c1, n1)
    assert sorted(order.tolist()) == list(range(a.n))


def test_ordered_sor_identity_order_is_lexicographic():
    s, a = _stencil_system()
    b = s.rhs()
    x0 = np.linspace(0, 1, a.n)
    ident = np.arange(a.n, dtype=np.int32)
    for fwd in (True, False):
        np.testing.assert_array_equal(
            lo.sor_sweep(a, b, x_in=x0, forward=fwd, order=ident),
            lo.sor_sweep(a, b, x_in=x0, forward=fwd, nparts=1))


def test_aggregation_invariants():
    k = np.exp(1.5 * np.random.default_rng(1).standard_normal(12 * 12 * 12))
    a = lo.gen_27pt((12, 12, 12), k)
    dep, inf, iso = lo.amg_strength(a)
    for nparts in (1, 3, 8):
        nc, agg, lp, lst, stats = lo.amg_aggregate(a, dep, inf, iso, 6, 9, nparts)
        assert stats[0] == nc
        sizes = np.diff(lp)
        assert sizes.min() >= 1 and sizes.max() <= 9
        for c in range(nc):
            assert np.all(agg[lst[lp[c]:lp[c + 1]]] == c)
        assert np.all((agg < nc) | (agg == lo.ISOLATED))
        # aggregates never cross partitions
        bounds = [lo.lib().lo_part_begin(a.n, nparts, p) for p in range(nparts + 1)]
        part = np.searchsorted(bounds, np.arange(a.n), side="right") - 1
        for c in range(nc):
            assert len(set(part[lst[lp[c]:lp[c + 1]]])) == 1


def test_galerkin_matches_dense_product():
    k = np.exp(np.random.default_rng(2).standard_normal(8 * 8 * 8))
    a = lo.gen_27pt((8, 8, 8), k)
    dep, inf, iso = lo.amg_strength(a)
    nc, agg, lp, lst, _ = lo.amg_aggregate(a, dep, inf, iso, 6, 9, 2)
    ac = lo.amg_galerkin(a, nc, agg, lp, lst)
    p = np.zeros((a.n, nc))
    for i in range(a.n):
        if agg[i] < nc:
            p[i, agg[i]] = 1.0
    np.testing.assert_allclose(ac.to_dense(), p.T @ a.to_dense() @ p, rtol=1e-13, atol=1e-13)


def test_amg_pcg_27pt_converges():
    dims = (16, 16, 16)
    k = np.exp(1.5 * np.random.default_rng(1).standard_normal(np.prod(dims)))
    a = lo.gen_27pt(dims, k)
    b = np.random.default_rng(0).uniform(-1, 1, a.n)
    amg = lo.Amg(a, min_coarsen_size=100, partition_size=512, smoother_parts=0)
    x, it, hist = lo.pcg(a, b, precon=lo.PRECON_AMG, amg=amg, rtol=1e-8, maxit=200)
    assert hist[-1] <= 1e-8 * hist[0]
    assert it < 60


def test_lu_factor_solves_nonsymmetric():
    """Unpivoted row-wise LU (lu/decomposition.hpp) of a nonsymmetric,
    diagonally dominant sparse matrix against a dense solve; the factors
    reproduce A."""
    rng = np.random.default_rng(7)
    n = 60
    dense = np.where(rng.random((n, n)) < 0.1, rng.uniform(-1, 1, (n, n)), 0.0)
    dense += np.diag(np.abs(dense).sum(axis=1) + 1.0)
    rowptr = np.concatenate([[0], np.cumsum((dense != 0).sum(axis=1))]).astype(np.int64)
    col = np.concatenate([np.flatnonzero(r) for r in dense]).astype(np.int32)
    val = dense[dense != 0]
    a = lo.Csr(rowptr, col, val, symmetric=False)
    lu = lo.lu_factor(a)
    lower = np.tril(lu, -1) + np.eye(n)
    upper = np.triu(lu)
    assert np.abs(lower @ upper - dense).max() <= 1e-13 * np.abs(dense).max()
    b = rng.uniform(-1, 1, n)
    np.testing.assert_allclose(lo.lu_solve(lu, b), np.linalg.solve(dense, b), rtol=1e-12,
                               atol=1e-14)


def test_amg_bicgstab_nonsymmetric_uses_lu():
    """BiCGStab + AMG on an upwind convection-diffusion operator (values and
    coarse operators nonsymmetric): the coarsest level is solved by LU, and
    the solve reaches its tolerance (test/aux/iterative.hpp:175-181 runs
    this combination)."""
    a = lo.gen_convdiff((14, 13, 12), (8.0, -5.0, 3.0))
    dense = np.zeros((a.n, a.n))
    for i in range(a.n):
        dense[i, a.col[a.rowptr[i]:a.rowptr[i + 1]]] = a.val[a.rowptr[i]:a.rowptr[i + 1]]
    assert np.abs(dense - dense.T).max() > 0.1  # nonsymmetric values
    amg = lo.Amg(a, min_coarsen_size=64, partition_size=512)
    b = np.random.default_rng(3).uniform(-1, 1, a.n)
    x, it, hist = lo.pbicgstab(a, b, precon=lo.PRECON_AMG, amg=amg, rtol=1e-8, maxit=300)
    assert hist[-1] <= 1e-8 * hist[0] and it < 60
    assert np.linalg.norm(b - dense @ x) <= 1.01e-8 * np.linalg.norm(b)


def _diagonal_lines(dims):
    # test/aux/materials.hpp:214-232: material (j + k) mod 4, constant along
    # the flow axis
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    return ((j + k) % 4).ravel().astype(np.uint8)


def test_effective_diffusion_diagonal_lines():
    """EffDiffCalc on the reference suite's system (test/shared-stencil.hpp:
    69-104, 225-238): materials constant along the flow axis give the
    cross-section mean of the coefficients (materials.hpp:236-250)."""
    dims, coeffs, lengths = (4, 9, 7), (0.0, 1.0, 2.0, 3.0), (4.0, 9.0, 7.0)
    mat = _diagonal_lines(dims)
    st = lo.Stencil(dims, q=lo.axis_quotients(dims, lengths), mat=mat, coeffs=coeffs,
                    sol_start=1.0, sol_end=0.0)
    a, _ = st.to_csr()
    x, it, hist = lo.pcg(a, st.rhs(), precon=lo.PRECON_JACOBI, rtol=1e-14, maxit=1000)
    eff, area = st.effective_diffusion(lengths, x)
    j, k = np.meshgrid(np.arange(9), np.arange(7), indexing="ij")
    want = np.mean(np.asarray(coeffs)[(j + k) % 4])
    assert area == 1.0
    assert abs(eff - want) <= 1e-12
    # "none" materials leave the area part, not the flux
    eff0, area0 = st.effective_diffusion(lengths, x, none_mask=0b0001)
    assert area0 == pytest.approx(1.0 - np.mean((j + k) % 4 == 0))
    assert eff0 == pytest.approx(eff / area0, rel=1e-13)


def test_values_valuator_matches_explicit_operator():
    """StationaryDiffusionValuesValuator (stationary-diffusion-values.hpp):
    connections hm(k_d(i), k_d(j)) q_d along axis d, axis-0 Dirichlet terms
    2 q_0 k_0(i); with equal axes it is the value valuator bit for bit."""
    dims = (5, 4, 6)
    n = int(np.prod(dims))
    rng = np.random.default_rng(21)
    ks = [np.exp(rng.standard_normal(n)) for _ in range(3)]
    q = lo.axis_quotients(dims, (1.0, 2.0, 0.5))
    st = lo.Stencil(dims, q=q, k_axes=ks, sol_start=1.0, sol_end=0.0)
    same = lo.Stencil(dims, q=q, k_axes=[ks[0]] * 3, sol_start=1.0, sol_end=0.0)
    val = lo.Stencil(dims, q=q, k=ks[0], sol_start=1.0, sol_end=0.0)
    x = rng.uniform(-1, 1, n)
    np.testing.assert_array_equal(same.spmv(x), val.spmv(x))
    strides = (dims[1] * dims[2], dims[2], 1)
    dense = np.zeros((n, n))
    hm = lambda a, b: 2 * a * b / (a + b)  # noqa: E731
    for i in range(n):
        pos = np.unravel_index(i, dims)
        for d in range(3):
            for s in (-1, 1):
                p = list(pos)
                p[d] += s
                if 0 <= p[d] < dims[d]:
                    j = i + s * strides[d]
                    c = hm(ks[d][i], ks[d][j]) * q[d]
                    dense[i, j] -= c
                    dense[i, i] += c
        if pos[0] == 0 or pos[0] == dims[0] - 1:
            dense[i, i] += 2 * q[0] * ks[0][i] * ((pos[0] == 0) + (pos[0] == dims[0] - 1))
    np.testing.assert_allclose(st.spmv(x), dense @ x, rtol=1e-13, atol=1e-13)
    assert not np.allclose(st.spmv(x), val.spmv(x))


def test_henry_lookup_provider():
    """HenryDiffusionLookupProvider (lookup-wright.hpp:38-60): factor
    hm(c_a f_b, c_b f_a) with f = H for gaseous materials; H = 1 gives the
    symmetric provider."""
    dims = (5, 4, 6)
    mat = np.random.default_rng(23).integers(0, 4, int(np.prod(dims))).astype(np.uint8)
    coeffs = (0.5, 1.0, 2.0, 3.0)
    q = lo.axis_quotients(dims, (1.0, 1.2, 0.8))
    sym = lo.Stencil(dims, q=q, mat=mat, coeffs=coeffs)
    h1 = lo.Stencil(dims, q=q, mat=mat, coeffs=coeffs, henry=1.0, gaseous_mask=0b1010)
    np.testing.assert_array_equal(h1.conn, sym.conn)
    h = lo.Stencil(dims, q=q, mat=mat, coeffs=coeffs, henry=0.3, gaseous_mask=0b1010)
    hm = lambda a, b: 2 * a * b / (a + b)  # noqa: E731
    for a in range(4):
        for b in range(4):
            fa = 0.3 if (0b1010 >> a) & 1 else 1.0
            fb = 0.3 if (0b1010 >> b) & 1 else 1.0
            want = hm(coeffs[a] * fb, coeffs[b] * fa) * q[1]
            assert h.conn[16 + a * 4 + b] == pytest.approx(want, rel=1e-15)
    x = np.random.default_rng(24).uniform(-1, 1, len(mat))
    assert not np.allclose(h.spmv(x), sym.spmv(x))


def test_oracle_ctypes_structs_match_the_header(tmp_path):
    """The oracle's ctypes mirrors have lineal_oracle.h's sizes and offsets."""
    import ctypes
    import subprocess

    pairs = {"lo_csr": lo._Csr, "lo_stencil": lo._Stencil, "lo_amg_params": lo._AmgParams,
             "lo_amg_level": lo._AmgLevel, "lo_amg": lo._Amg, "lo_agg_map": lo._AggMap,
             "lo_precon": lo._Precon}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "lineal_oracle.h"',
             "int main(void) {"]
    for cname, py in pairs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "probe")
    here = os.path.dirname(lo.__file__)
    subprocess.run(["gcc", "-std=c11", "-I", here, str(src), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(line.split()[:2]): int(line.split()[2]) for line in out if line}
    for cname, py in pairs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)
