"""Aggregate-map files (lineal_gb300.io) and hierarchies built from given
aggregate maps, lineal's RefinedAggregator / FileAggregator pair
(linear-solver/multigrid/aggregation/independent.hpp:237-298), on the CPU:
the oracle's maps survive a file round trip, a hierarchy rebuilt from them
equals the one that computed them, and damaged maps or files are refused."""

import os

import numpy as np
import pytest

import oracle as lo
from lineal_gb300 import io as lio

PARAMS = dict(min_coarsen_size=20, partition_size=64, smoother_parts=0)


def _case(dims=(10, 12, 14), seed=0, npts=27):
    k = np.exp(1.5 * np.random.default_rng(seed).standard_normal(int(np.prod(dims))))
    return (lo.gen_27pt if npts == 27 else lo.gen_7pt)(dims, k)


def _maps(h):
    return [lio.AggregateMap(*h.level_map(l)) for l in range(h.nlevels - 1)]


def _assert_maps_equal(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        for u, v in zip(x, y):
            np.testing.assert_array_equal(u, v)


@pytest.mark.parametrize("npts", [27, 7])
def test_file_round_trip_and_rebuild(tmp_path, npts):
    a = _case(npts=npts)
    h = lo.Amg(a, **PARAMS)
    assert h.nlevels >= 3
    maps = _maps(h)
    for m in maps:
        assert lo.agg_map_check(*m)
        lio.check_aggregate_map(m)
    base = str(tmp_path / "level")
    paths = lio.save_aggregates(base, maps)
    assert paths == [f"{base}{k}.aggs" for k in range(len(maps))]
    back = lio.load_aggregates(base)
    _assert_maps_equal(maps, back)
    # FileAggregator: the rebuilt hierarchy equals the one that aggregated
    g = lo.Amg(a, maps=back, **PARAMS)
    assert g.nlevels == h.nlevels
    for l in range(h.nlevels):
        x, y = h.level_csr(l), g.level_csr(l)
        np.testing.assert_array_equal(x.rowptr, y.rowptr)
        np.testing.assert_array_equal(x.col, y.col)
        np.testing.assert_array_equal(x.val, y.val)
    b = np.random.default_rng(1).uniform(-1, 1, a.n)
    np.testing.assert_array_equal(h.vcycle(b), g.vcycle(b))


def test_given_maps_override_the_partitioning():
    # maps computed with 64-vertex partitions, used by a setup whose own
    # aggregation would run in one partition: the maps decide the hierarchy
    a = _case(seed=3)
    h = lo.Amg(a, **PARAMS)
    one = dict(PARAMS, partition_size=1 << 20, max_partitions=1)
    plain = lo.Amg(a, **one)
    assert [plain.level_size(l) for l in range(plain.nlevels)] != \
        [h.level_size(l) for l in range(h.nlevels)] or \
        not np.array_equal(plain.level_agg(0), h.level_agg(0))
    g = lo.Amg(a, maps=_maps(h), **one)
    _assert_maps_equal(_maps(g), _maps(h))


def test_missing_and_mismatched_maps_are_refused():
    a = _case()
    h = lo.Amg(a, **PARAMS)
    maps = _maps(h)
    with pytest.raises(ValueError, match="no aggregate map"):
        lo.Amg(a, maps=maps[:1], **PARAMS)
    # level 1's map given for level 0: wrong fine size
    with pytest.raises(ValueError, match="does not fit"):
        lo.Amg(a, maps=maps[1:] + maps[:1], **PARAMS)


def _damaged(m):
    agg, ptr, lst = (np.array(v) for v in m)
    out = {}
    bad = agg.copy()
    bad[int(lst[0])] = len(ptr) + 5  # id beyond the coarse size
    out["id"] = (bad, ptr, lst)
    swap = lst.copy()
    swap[[0, -1]] = swap[[-1, 0]]  # vertices listed under the wrong aggregate
    out["owner"] = (agg, ptr, swap)
    dup = lst.copy()
    dup[1] = dup[0]
    out["repeat"] = (agg, ptr, dup)
    iso = agg.copy()
    iso[int(lst[0])] = lio.ISOLATED  # an isolated vertex still listed
    out["isolated"] = (iso, ptr, lst)
    return out


def test_damaged_maps_fail_both_checks():
    h = lo.Amg(_case(), **PARAMS)
    m = lio.AggregateMap(*h.level_map(0))
    for name, d in _damaged(m).items():
        assert not lo.agg_map_check(*d), name
        with pytest.raises(ValueError):
            lio.check_aggregate_map(lio.AggregateMap(*d))
        with pytest.raises(ValueError, match="does not fit"):
            lo.Amg(_case(), maps=[d] + _maps(h)[1:], **PARAMS)


def test_damaged_files_are_refused(tmp_path):
    h = lo.Amg(_case(), **PARAMS)
    maps = _maps(h)
    base = str(tmp_path / "m")
    lio.save_aggregates(base, maps)
    raw = open(lio.aggs_path(base, 0), "rb").read()
    open(lio.aggs_path(base, 0), "wb").write(raw[:-4])
    with pytest.raises(ValueError, match="size"):
        lio.read_aggs(lio.aggs_path(base, 0))
    open(lio.aggs_path(base, 0), "wb").write(b"NOTAGGS!" + raw[8:])
    with pytest.raises(ValueError, match="not an aggregate-map"):
        lio.read_aggs(lio.aggs_path(base, 0))
    # levels that do not chain
    lio.save_aggregates(base, [maps[0], maps[0]])
    with pytest.raises(ValueError, match="coarse size"):
        lio.load_aggregates(base)
    with pytest.raises(FileNotFoundError):
        lio.load_aggregates(str(tmp_path / "absent"))
    with pytest.raises(ValueError):
        lio.write_aggs(str(tmp_path / "x.aggs"), lio.AggregateMap(*_damaged(maps[0])["owner"]))
    assert not os.path.exists(str(tmp_path / "x.aggs"))


def test_library_map_check_agrees_with_the_oracle():
    """lgx_agg_map_check, the host-side check lgx_amg_setup_given runs
    before it copies a map to the device, accepts the oracle's maps and
    refuses every damaged one (no device work: it runs without a GPU)."""
    import lineal_gb300 as g

    h = lo.Amg(_case(), **PARAMS)
    for m in _maps(h):
        g.agg_map_check(m)
    m = _maps(h)[0]
    with pytest.raises(g.LinealError, match="fine size"):
        g.agg_map_check(m, len(m.agg) + 1)
    for name, d in _damaged(m).items():
        with pytest.raises(g.LinealError):
            g.agg_map_check(d)
    agg, ptr, lst = (np.array(v) for v in m)
    empty = np.concatenate([ptr[:1], ptr])  # an empty first aggregate
    with pytest.raises(g.LinealError, match="empty"):
        g.agg_map_check((np.where(agg == lio.ISOLATED, agg, agg + 1), empty, lst))
    with pytest.raises(ValueError):
        g.agg_map_check((agg, ptr, lst[:-1]))  # list shorter than its offsets


def _cpp_aggs():
    from lineal_gb300 import build

    return build.build_cpp_demo(name="aggs_io_demo")


def _run(*args):
    import subprocess

    return subprocess.run(list(args), capture_output=True, text=True, timeout=120)


def test_cpp_and_python_files_agree(tmp_path):
    """The C++ layer's write_aggs / read_aggregates and lineal_gb300.io read
    and write the same bytes (host code only, no GPU)."""
    exe = _cpp_aggs()
    base = str(tmp_path / "cpp")
    r = _run(exe, "write", base)
    assert r.returncode == 0, r.stdout + r.stderr
    maps = lio.load_aggregates(base)
    assert len(maps) == 2
    np.testing.assert_array_equal(maps[0].agg, [1, 1, 0, 0, lio.ISOLATED, 2, 2, 0, 1, 2])
    np.testing.assert_array_equal(maps[0].list_ptr, [0, 3, 6, 9])
    np.testing.assert_array_equal(maps[0].list, [3, 2, 7, 8, 0, 1, 9, 5, 6])
    np.testing.assert_array_equal(maps[1].list, [1, 0, 2])
    # Python writes the oracle's maps, C++ reads them back
    h = lo.Amg(_case(), **PARAMS)
    pbase = str(tmp_path / "py")
    lio.save_aggregates(pbase, _maps(h))
    r = _run(exe, "read", pbase)
    assert r.returncode == 0, r.stdout + r.stderr
    want = [f"level {k} n {len(m.agg)} nc {len(m.list_ptr) - 1} sum "
            f"{int(m.agg.astype(np.int64).sum() + 3 * m.list.astype(np.int64).sum())}"
            for k, m in enumerate(_maps(h))]
    assert r.stdout.split("\n")[:-1] == want


def test_cpp_reader_refuses_damaged_files(tmp_path):
    exe = _cpp_aggs()
    h = lo.Amg(_case(), **PARAMS)
    m = _maps(h)[0]
    good = str(tmp_path / "good.aggs")
    lio.write_aggs(good, m)
    raw = open(good, "rb").read()
    cases = {"truncated": raw[:-4], "longer": raw + b"\0", "magic": b"NOTAGGS!" + raw[8:]}
    # a consistent-looking file whose lists put a vertex under another aggregate
    agg, ptr, lst = (np.array(v) for v in m)
    swap = lst.copy()
    swap[[0, -1]] = swap[[-1, 0]]
    body = (b"LGXAGGS1" + np.array([len(agg), len(ptr) - 1], "<u8").tobytes()
            + agg.astype("<u4").tobytes() + ptr.astype("<u8").tobytes()
            + swap.astype("<u4").tobytes())
    cases["owner"] = body
    for name, data in cases.items():
        path = str(tmp_path / f"{name}.aggs")
        open(path, "wb").write(data)
        r = _run(exe, "refuse", path)
        assert r.returncode == 0 and "refused" in r.stdout, (name, r.stdout, r.stderr)
    assert _run(exe, "refuse", good).returncode == 1


def _random_map(rng, n, nc):
    """a consistent map: nc non-empty aggregates, some isolated vertices"""
    agg = np.full(n, lio.ISOLATED, dtype=np.uint32)
    members = rng.permutation(n)[: rng.integers(nc, n + 1)]
    owner = np.concatenate([np.arange(nc), rng.integers(0, nc, len(members) - nc)])
    agg[members] = owner
    order = np.argsort(owner, kind="stable")
    lst = members[order].astype(np.int32)
    ptr = np.concatenate([[0], np.cumsum(np.bincount(owner, minlength=nc))]).astype(np.int64)
    return agg, ptr, lst


def _damage(rng, agg, ptr, lst):
    agg, ptr, lst = agg.copy(), ptr.copy(), lst.copy()
    kind = rng.integers(0, 6)
    if kind == 0 and len(lst):
        agg[lst[rng.integers(len(lst))]] = len(ptr) + rng.integers(0, 3)  # id out of range
    elif kind == 1 and len(lst) > 1:
        i, j = rng.choice(len(lst), 2, replace=False)
        if agg[lst[i]] != agg[lst[j]]:
            lst[i], lst[j] = lst[j], lst[i]  # listed under another aggregate
        else:
            lst[i] = lst[j]  # repeated
    elif kind == 2 and len(lst):
        agg[lst[rng.integers(len(lst))]] = lio.ISOLATED  # listed but isolated
    elif kind == 3 and len(lst):
        lst[rng.integers(len(lst))] = len(agg) + rng.integers(0, 5)  # vertex out of range
    elif kind == 4:
        ptr[0] = 1  # offsets not from 0
    else:
        return agg, ptr, lst, True  # untouched
    return agg, ptr, lst, False


def test_three_checkers_agree_on_random_maps():
    """lgx_agg_map_check (the library's guard before any device copy), the
    oracle's lo_agg_map_check and io.check_aggregate_map accept and refuse
    the same maps: 300 random maps, most of them damaged."""
    import lineal_gb300 as g

    rng = np.random.default_rng(12)
    for _ in range(300):
        n = int(rng.integers(1, 60))
        nc = int(rng.integers(1, n + 1))
        agg, ptr, lst, intact = _damage(rng, *_random_map(rng, n, nc))
        votes = []
        try:
            g.agg_map_check((agg, ptr, lst))
            votes.append(True)
        except (g.LinealError, ValueError):
            votes.append(False)
        votes.append(lo.agg_map_check(agg, ptr, lst) if ptr[-1] <= len(lst) else False)
        try:
            lio.check_aggregate_map(lio.AggregateMap(agg, ptr, lst))
            votes.append(True)
        except ValueError:
            votes.append(False)
        assert votes[0] == votes[1] == votes[2], (votes, n, nc)
        if intact:
            assert votes[0]
