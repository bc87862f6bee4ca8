"""SMF (sparse matrix) and DVF (dense vector) files, lineal's binary formats,
and per-level aggregate-map files.

Layouts (include/lineal/io/tensor.hpp:25-263):

* SMF: u64 rows, u64 columns, u64 non-zeros, u64 row offsets[rows + 1], then
  per non-zero an interleaved (u64 column, f64 value) pair.  The writer
  (SmfWriter, tensor.hpp:153-205) skips entries equal to zero.
* DVF: u64 size, then f64 values.

Aggregate maps: lineal's RefinedAggregator writes the map of level k to
``<base>k.aggs`` and its FileAggregator reads it back instead of aggregating
(linear-solver/multigrid/aggregation/independent.hpp:35-44, 264-272,
293-298); a file holds both halves of BaseMultithreadAggregateMap, the
fine -> coarse ids and the coarse -> fine lists (aggregate-map/
multithread.hpp:299-303, 346-349).  lineal serialises them with its
thesauros containers, whose byte layout is not part of lineal, so the layout
here is this package's own:

* ``.aggs``: 8 magic bytes ``LGXAGGS1``, u64 fine size n, u64 coarse size
  nc, u32 aggregate id per fine vertex (0xFFFFFFFE for an isolated vertex),
  u64 list offsets[nc + 1], u32 fine vertex per list entry.

All integers are little-endian.
"""

from __future__ import annotations

import os
from typing import NamedTuple

import numpy as np

_U64 = np.dtype("<u8")
_F64 = np.dtype("<f8")
_PAIR = np.dtype([("col", "<u8"), ("val", "<f8")])


def read_smf(path: str):
    """Returns (rowptr int64, col int32, val float64, ncols)."""
    with open(path, "rb") as f:
        rows, cols, nnz = np.frombuffer(f.read(24), dtype=_U64)
        rows, cols, nnz = int(rows), int(cols), int(nnz)
        rowptr = np.frombuffer(f.read(8 * (rows + 1)), dtype=_U64).astype(np.int64)
        pairs = np.frombuffer(f.read(16 * nnz), dtype=_PAIR)
    if int(rowptr[-1]) != nnz or len(pairs) != nnz:
        raise ValueError(f"{path}: inconsistent SMF header")
    return rowptr, pairs["col"].astype(np.int32), pairs["val"].astype(np.float64), cols


def write_smf(path: str, rowptr, col, val, ncols: int | None = None) -> None:
    rowptr = np.asarray(rowptr, dtype=np.int64)
    col = np.asarray(col)
    val = np.asarray(val, dtype=np.float64)
    n = len(rowptr) - 1
    keep = val != 0
    counts = np.add.reduceat(keep.astype(np.int64), rowptr[:-1]) if len(val) else np.zeros(n)
    counts = np.where(np.diff(rowptr) > 0, counts, 0)
    new_ptr = np.zeros(n + 1, dtype=np.uint64)
    new_ptr[1:] = np.cumsum(counts)
    pairs = np.empty(int(keep.sum()), dtype=_PAIR)
    pairs["col"] = col[keep]
    pairs["val"] = val[keep]
    with open(path, "wb") as f:
        f.write(np.array([n, n if ncols is None else ncols, len(pairs)], dtype=_U64).tobytes())
        f.write(new_ptr.astype(_U64).tobytes())
        f.write(pairs.tobytes())


def read_dvf(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        (size,) = np.frombuffer(f.read(8), dtype=_U64)
        return np.frombuffer(f.read(8 * int(size)), dtype=_F64).astype(np.float64)


def write_dvf(path: str, vec) -> None:
    vec = np.asarray(vec, dtype=np.float64)
    with open(path, "wb") as f:
        f.write(np.array([len(vec)], dtype=_U64).tobytes())
        f.write(vec.astype(_F64).tobytes())


ISOLATED = 0xFFFFFFFE
_AGGS_MAGIC = b"LGXAGGS1"
_U32 = np.dtype("<u4")


class AggregateMap(NamedTuple):
    """One level's aggregates: ``agg[v]`` is the aggregate of fine vertex v
    (ISOLATED for an isolated vertex); aggregate c holds the fine vertices
    ``list[list_ptr[c]:list_ptr[c + 1]]`` in the order aggregation added them."""

    agg: np.ndarray       # uint32[n]
    list_ptr: np.ndarray  # int64[nc + 1]
    list: np.ndarray      # int32[list_ptr[nc]]

    @property
    def fine_size(self) -> int:
        return len(self.agg)

    @property
    def coarse_size(self) -> int:
        return len(self.list_ptr) - 1


def check_aggregate_map(m: AggregateMap) -> None:
    """Raises ValueError unless the two halves agree: every id below the
    coarse size or ISOLATED, every aggregated vertex in exactly the list of
    its aggregate, no empty aggregate."""
    agg = np.asarray(m.agg, dtype=np.uint32)
    ptr = np.asarray(m.list_ptr, dtype=np.int64)
    lst = np.asarray(m.list, dtype=np.int64)
    n, nc = len(agg), len(ptr) - 1
    if nc < 0 or ptr[0] != 0:
        raise ValueError("aggregate map: list offsets must start at 0")
    if np.any(np.diff(ptr) < 1):
        raise ValueError("aggregate map: empty or decreasing aggregate lists")
    aggregated = agg != ISOLATED
    if np.any(agg[aggregated] >= nc):
        raise ValueError("aggregate map: aggregate id beyond the coarse size")
    if int(ptr[-1]) != len(lst) or len(lst) != int(aggregated.sum()):
        raise ValueError("aggregate map: lists do not cover the aggregated vertices")
    if len(lst) and (lst.min() < 0 or lst.max() >= n or len(np.unique(lst)) != len(lst)):
        raise ValueError("aggregate map: list entry out of range or repeated")
    owner = np.repeat(np.arange(nc, dtype=np.int64), np.diff(ptr))
    if np.any(agg[lst].astype(np.int64) != owner):
        raise ValueError("aggregate map: a listed vertex belongs to another aggregate")


def write_aggs(path: str, m: AggregateMap) -> None:
    check_aggregate_map(m)
    with open(path, "wb") as f:
        f.write(_AGGS_MAGIC)
        f.write(np.array([m.fine_size, m.coarse_size], dtype=_U64).tobytes())
        f.write(np.asarray(m.agg).astype(_U32).tobytes())
        f.write(np.asarray(m.list_ptr).astype(_U64).tobytes())
        f.write(np.asarray(m.list).astype(_U32).tobytes())


def read_aggs(path: str) -> AggregateMap:
    with open(path, "rb") as f:
        if f.read(8) != _AGGS_MAGIC:
            raise ValueError(f"{path}: not an aggregate-map file")
        n, nc = (int(v) for v in np.frombuffer(f.read(16), dtype=_U64))
        agg = np.frombuffer(f.read(4 * n), dtype=_U32).astype(np.uint32)
        ptr = np.frombuffer(f.read(8 * (nc + 1)), dtype=_U64).astype(np.int64)
        if len(agg) != n or len(ptr) != nc + 1:
            raise ValueError(f"{path}: truncated aggregate-map file")
        total = int(ptr[-1])
        lst = np.frombuffer(f.read(4 * total), dtype=_U32).astype(np.int32)
        if len(lst) != total or f.read(1):
            raise ValueError(f"{path}: aggregate-map file size does not match its header")
    m = AggregateMap(agg, ptr, lst)
    check_aggregate_map(m)
    return m


def aggs_path(base: str, level: int) -> str:
    """``<base><level>.aggs`` (independent.hpp:35-44, one process)"""
    return f"{base}{level}.aggs"


def save_aggregates(base: str, maps) -> list[str]:
    """Writes maps[k] to aggs_path(base, k); returns the paths."""
    paths = []
    for k, m in enumerate(maps):
        paths.append(aggs_path(base, k))
        write_aggs(paths[-1], AggregateMap(*m))
    return paths


def load_aggregates(base: str) -> list[AggregateMap]:
    """Reads aggs_path(base, 0), aggs_path(base, 1), ... up to the first
    missing level; consecutive levels must chain (coarse size of level k =
    fine size of level k + 1)."""
    maps = []
    while os.path.exists(aggs_path(base, len(maps))):
        maps.append(read_aggs(aggs_path(base, len(maps))))
        if len(maps) > 1 and maps[-2].coarse_size != maps[-1].fine_size:
            raise ValueError(f"{aggs_path(base, len(maps) - 1)}: fine size does not match the "
                             "coarse size of the level above")
    if not maps:
        raise FileNotFoundError(aggs_path(base, 0))
    return maps
