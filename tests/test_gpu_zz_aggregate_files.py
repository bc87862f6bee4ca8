"""Aggregate maps of a GPU hierarchy: both halves (fine -> coarse ids and
the coarse -> fine lists in aggregation order) equal the oracle's, and the
files the GPU hierarchy writes (RefinedAggregator with base_agg_map_path,
aggregation/independent.hpp:264-272) rebuild, through the oracle's
FileAggregator path, the GPU's level matrices bit for bit."""

import numpy as np
import pytest

import oracle as lo
from lineal_gb300 import io as lio

pytestmark = pytest.mark.gpu

PARAMS = dict(min_coarsen_size=64, partition_size=512, max_partitions=1 << 30)


def test_gpu_aggregate_maps_cross_check_the_oracle(cuda, tmp_path):
    dims = (14, 15, 16)
    ref = lo.gen_27pt(dims, np.exp(1.5 * np.random.default_rng(1).standard_normal(
        int(np.prod(dims)))))
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    h = cuda.HierarchyWright(**PARAMS).instantiate(m)
    oh = lo.Amg(ref, smoother_parts=0, **PARAMS)
    maps = h.aggregate_maps()
    assert len(maps) == oh.nlevels - 1 >= 2
    for l, mm in enumerate(maps):
        lio.check_aggregate_map(mm)
        for got, want in zip(mm, oh.level_map(l)):
            np.testing.assert_array_equal(got, want)
    with pytest.raises(IndexError):
        h.aggregate_map(len(maps))
    base = str(tmp_path / "gpu")
    assert h.save_aggregates(base) == [lio.aggs_path(base, k) for k in range(len(maps))]
    # one partition of its own: only the files decide the aggregates
    g = lo.Amg(ref, maps=lio.load_aggregates(base), smoother_parts=0,
               **dict(PARAMS, partition_size=1 << 24, max_partitions=1))
    assert g.nlevels == len(maps) + 1
    for l in range(g.nlevels):
        rowptr, col, val, _ = h.level(l, with_agg=False)
        rl = g.level_csr(l)
        np.testing.assert_array_equal(rowptr, rl.rowptr)
        np.testing.assert_array_equal(col, rl.col)
        np.testing.assert_array_equal(val, rl.val)


def test_gpu_setup_from_given_maps(cuda, tmp_path):
    """lgx_amg_setup_given (FileAggregator, aggregation/independent.hpp:
    279-298): a GPU hierarchy built from the maps of another hierarchy
    equals it, whatever its own partitioning parameters say."""
    dims = (12, 14, 16)
    ref = lo.gen_27pt(dims, np.exp(1.5 * np.random.default_rng(4).standard_normal(
        int(np.prod(dims)))))
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    one_part = dict(PARAMS, partition_size=1 << 24, max_partitions=1)
    b = np.random.default_rng(5).uniform(-1, 1, ref.n)
    # GPU maps through files -> GPU hierarchy
    h = cuda.HierarchyWright(**PARAMS).instantiate(m)
    base = str(tmp_path / "h")
    h.save_aggregates(base)
    g = cuda.HierarchyWright(**one_part).instantiate(m, aggregates=lio.load_aggregates(base))
    assert g.sizes() == h.sizes()
    np.testing.assert_array_equal(g.vcycle(b).cpu().numpy(), h.vcycle(b).cpu().numpy())
    # the oracle's maps (64-vertex partitions) -> GPU level matrices = oracle's
    oh = lo.Amg(ref, smoother_parts=0, **dict(PARAMS, partition_size=64))
    omaps = [oh.level_map(l) for l in range(oh.nlevels - 1)]
    go = cuda.HierarchyWright(**one_part).instantiate(m, aggregates=omaps)
    rows, _ = go.sizes()
    assert len(rows) == oh.nlevels
    for l in range(oh.nlevels):
        rowptr, col, val, _ = go.level(l, with_agg=False)
        rl = oh.level_csr(l)
        np.testing.assert_array_equal(rowptr, rl.rowptr)
        np.testing.assert_array_equal(col, rl.col)
        np.testing.assert_array_equal(val, rl.val)
    # too few maps, or a map for another level, are refused before device work
    with pytest.raises(cuda.LinealError, match="no aggregate map"):
        cuda.HierarchyWright(**PARAMS).instantiate(m, aggregates=omaps[:1])
    with pytest.raises(cuda.LinealError, match="fine size"):
        cuda.HierarchyWright(**PARAMS).instantiate(m, aggregates=omaps[1:])


def test_gpu_setup_log_matches_the_oracle(cuda):
    """Hierarchy.setup_log (lgx_amg_setup_log): lineal's setup log keys, the
    level sizes, the level-0 aggregation statistics of the oracle's
    aggregation with the same partitions, and the stop reason."""
    import ctypes

    dims = (14, 15, 16)
    ref = lo.gen_27pt(dims, np.exp(1.5 * np.random.default_rng(1).standard_normal(
        int(np.prod(dims)))))
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val, symmetric=True)
    h = cuda.HierarchyWright(**PARAMS).instantiate(m)
    log = h.setup_log()["create_hierarchy"]
    rows, nnz = h.sizes()
    assert [e["dimensions"]["rows"] for e in log["levels"]] == rows
    assert [e["non_zeros"] for e in log["levels"]] == nnz
    assert "aggregation_stats" not in log["levels"][-1]
    assert rows[-1] < PARAMS["min_coarsen_size"]
    assert log["stop_coarsening"]["reason"] == "too_small"
    nparts = lo.lib().lo_amg_partitions(ref.n, 0, ctypes.byref(lo.amg_params(**PARAMS)))
    dep, inf, iso = lo.amg_strength(ref)
    nc, _, _, _, stats = lo.amg_aggregate(ref, dep, inf, iso, 6, 9, nparts)
    got = log["levels"][0]["aggregation_stats"]
    assert got["aggregate_num"] == nc == rows[1]
    assert [got[k] for k in ("aggregate_num", "multi_vertex_aggregate_num",
                             "single_vertex_aggregate_num", "merged_aggregate_num",
                             "isolated_aggregate_num")] == [int(v) for v in stats]
    assert not log["levels"][0]["aggressive"] and not log["levels"][0]["given_map"]


def test_cpp_solver_writes_and_reads_maps(cuda, tmp_path):
    """The C++ MultiGridSolver's base_agg_map_path / file_agg_map_path
    (tests/cpp/aggs_solver_demo.cpp); the files it writes are the ones
    lineal_gb300.io reads."""
    import subprocess

    from lineal_gb300 import build

    exe = build.build_cpp_demo(name="aggs_solver_demo")
    base = str(tmp_path / "cpp")
    out = subprocess.run([exe, base], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "aggs_solver_demo ok" in out.stdout
    for m in lio.load_aggregates(base):
        lio.check_aggregate_map(m)
