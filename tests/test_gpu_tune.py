"""GPU tests of the row-engine autotuner: it keeps the fastest timed
configuration per matrix, operation and value type, and a tuned matrix
gives the same products, sweeps and V-cycles bit for bit."""

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu

PARAMS = dict(min_coarsen_size=64, partition_size=512, max_partitions=1 << 30)


def _case(dims=(20, 21, 22), seed=5, sigma=1.5):
    n = int(np.prod(dims))
    k = np.exp(sigma * np.random.default_rng(seed).standard_normal(n))
    return lo.gen_27pt(dims, k)


def _check_entry(e, default=None):
    assert e["fastest"] == int(np.argmin(e["ms"]))
    # a hierarchy level keeps its fastest shapes only when the V-cycle agrees
    assert e["config"] in ({e["fastest"]} if default is None else {e["fastest"], default})
    assert all(t > 0 for t in e["ms"])


@pytest.mark.parametrize("storage", [0, 1])
def test_matrix_autotune_keeps_fastest_and_results(cuda, storage):
    ref = _case()
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True, storage=storage)
    x = np.random.default_rng(2).uniform(-1, 1, ref.n)
    before = m.spmv(x).cpu().numpy()
    e = m.autotune(reps=3)
    _check_entry(e)
    assert e["value_bytes"] == (8 if storage == 0 else 4)
    np.testing.assert_array_equal(m.spmv(x).cpu().numpy(), before)
    if storage == 0:
        np.testing.assert_array_equal(before, lo.spmv(ref, x))


@pytest.mark.parametrize("form", ["fp64", "f32", "bf16"])
def test_amg_autotune_leaves_vcycle_bitexact(cuda, form):
    ref = _case()
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    kw = {"fp64": {}, "f32": dict(coarse_f32=True, cycle_f32=True),
          "bf16": dict(coarse_f32=True, cycle_f32=True, cycle_bf16=True)}[form]
    h = cuda.HierarchyWright(**PARAMS, **kw).instantiate(m)
    b = np.random.default_rng(3).uniform(-1, 1, ref.n)
    before = h.vcycle(b).cpu().numpy()
    entries = h.autotune(reps=2)
    L = h.level_num()
    smoothed = L - 1
    vb = {"fp64": 8, "f32": 4, "bf16": 2}[form]
    cycle = [e for e in entries if e["value_bytes"] == vb]
    assert sorted((e["level"], e["op"]) for e in cycle) == sorted(
        (lv, op) for lv in range(smoothed) for op in ("product", "sor"))
    if form != "fp64":
        # the outer Krylov product on the finest level reads FP64 values
        outer = [e for e in entries if e["value_bytes"] == 8]
        assert [(e["level"], e["op"]) for e in outer] == [(0, "product")]
    for e in entries:
        _check_entry(e, default=cuda.row_engine())
    np.testing.assert_array_equal(h.vcycle(b).cpu().numpy(), before)
    h.autotune_reset()
    np.testing.assert_array_equal(h.vcycle(b).cpu().numpy(), before)


def test_amg_pcg_after_autotune(cuda):
    ref = _case()
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    h = cuda.HierarchyWright(**PARAMS).instantiate(m)
    b = np.random.default_rng(4).uniform(-1, 1, ref.n)
    plain = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=1e-8, maxit=300)
    h.autotune(reps=2)
    tuned = cuda.pcg(m, b, precon=cuda.PRECON_AMG, amg=h, rtol=1e-8, maxit=300)
    # products and the V-cycle are unchanged; only the grouping of the
    # recomputed residual's norm may follow the tuned grid
    assert abs(tuned.iterations - plain.iterations) <= 1
    assert tuned.rel_residual <= 1e-8
    x = tuned.x.cpu().numpy()
    assert np.linalg.norm(b - lo.spmv(ref, x)) <= 1.01e-8 * np.linalg.norm(b)


def test_autotune_rejects_bad_reps(cuda):
    ref = _case((6, 6, 6))
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    with pytest.raises(cuda.LinealError):
        m.autotune(reps=0)
    h = cuda.HierarchyWright(**PARAMS).instantiate(m)
    with pytest.raises(cuda.LinealError):
        h.autotune(reps=1001)
