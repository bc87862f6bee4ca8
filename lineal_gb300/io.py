"""SMF (sparse matrix) and DVF (dense vector) files, lineal's binary formats.

Layouts (include/lineal/io/tensor.hpp:25-263):

* SMF: u64 rows, u64 columns, u64 non-zeros, u64 row offsets[rows + 1], then
  per non-zero an interleaved (u64 column, f64 value) pair.  The writer
  (SmfWriter, tensor.hpp:153-205) skips entries equal to zero.
* DVF: u64 size, then f64 values.

All integers are little-endian.
"""

from __future__ import annotations

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
