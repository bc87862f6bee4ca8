"""Python front end of lineal_gb300 (ctypes over the C ABI in include/lineal_gb300.h).

The names follow lineal's C++ API (KurtBoehm/lineal): ``CsrMatrix`` and the
stencil matrices (``AdjacentStencilMatrix`` with lookup/value valuators),
``ConjugateGradientsSolver`` / ``BiCgStabSolver`` (linear-solver/
conjugate-gradients/solver.hpp, linear-solver/bicgstab/solver.hpp),
``JacobiSolver`` / ``SorSolver`` / ``SsorSolver`` (linear-solver/
iterative-stationary/) and ``MultiGridSolver`` over a ``HierarchyWright``
(linear-solver/multigrid/).  Vectors are CUDA tensors from PyTorch, which is
used only for device memory and streams; every computation runs in the
library's own sm_103a kernels.

There is no CPU fallback: importing this module without the compiled library
raises ``LinealLibraryMissing``.
"""

from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

__all__ = [
    "LinealError", "LinealLibraryMissing", "lib", "CsrMatrix", "StencilMatrix", "Colouring",
    "HierarchyWright", "Hierarchy", "pcg", "pbicgstab", "spmv", "residual", "jacobi_sweep",
    "sor_sweep", "sor_sweep_permuted", "permute", "unpermute", "gen_27pt", "gen_7pt",
    "amg_strength", "amg_aggregate", "dot", "norm2sq", "max_norm", "sampled_outer",
    "diffusion7_grad", "residual_compensated", "batch_convdiff_bicgstab", "pcg_multi",
    "row_engine", "stencil_engine", "PRECON_NONE",
    "PRECON_JACOBI", "PRECON_SSOR", "PRECON_AMG",
]

PRECON_NONE, PRECON_JACOBI, PRECON_SSOR, PRECON_AMG = 0, 1, 2, 3
KIND_CSR, KIND_STENCIL_LOOKUP, KIND_STENCIL_VALUE = 0, 1, 2
F64, F32 = 0, 1
ISOLATED = 0xFFFFFFFE


class LinealError(RuntimeError):
    """A lineal_gb300 call returned a non-OK status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"lineal_gb300 status {status}: {message}")
        self.status = status


class LinealLibraryMissing(ImportError):
    pass


_lib = None


TUNE_CONFIGS = 8  # LGX_TUNE_CONFIGS


class _TuneEntry(C.Structure):
    _fields_ = [("level", C.c_int32), ("op", C.c_int32), ("value_bytes", C.c_int32),
                ("config", C.c_int32), ("fastest", C.c_int32),
                ("ms", C.c_float * TUNE_CONFIGS)]

    def as_dict(self):
        return {"level": self.level, "op": ("product", "sor")[self.op],
                "value_bytes": self.value_bytes, "config": self.config,
                "fastest": self.fastest,
                "ms": [float(t) for t in self.ms]}


class _AmgLevelLog(C.Structure):
    _fields_ = [(f, C.c_int64) for f in (
        "rows", "columns", "nnz", "aggregate_num", "multi_vertex_aggregate_num",
        "single_vertex_aggregate_num", "merged_aggregate_num", "isolated_aggregate_num")] + [
        ("aggressive", C.c_int32), ("given_map", C.c_int32)]


STOP_REASONS = {1: "too_small", 2: "too_many_levels", 3: "too_small_rate", 4: "level_cap"}


class _AmgParams(C.Structure):
    _fields_ = [
        ("min_aggregate_size", C.c_int32),
        ("max_aggregate_size", C.c_int32),
        ("partition_size", C.c_int64),
        ("partition_growth", C.c_double),
        ("min_partitions", C.c_int64),
        ("max_partitions", C.c_int64),
        ("strong_threshold", C.c_double),
        ("aggressive_threshold", C.c_double),
        ("max_level_num", C.c_int64),
        ("min_coarsen_size", C.c_int64),
        ("min_coarsen_factor", C.c_double),
        ("coarse_f32", C.c_int),
        ("cycle_f32", C.c_int),
        ("relax", C.c_double),
        ("smoother_relax", C.c_double),
        ("smoother_ultra", C.c_int),
        ("colour_seed", C.c_uint64),
        ("cycle_bf16", C.c_int),
        ("grid27", C.c_int),
        ("coarse_smallest_last", C.c_int),
    ]


class _SolveParams(C.Structure):
    _fields_ = [
        ("precon", C.c_int),
        ("relax", C.c_double),
        ("ultra", C.c_int),
        ("colouring", C.c_void_p),
        ("amg", C.c_void_p),
        ("rtol", C.c_double),
        ("maxit", C.c_int64),
        ("rere_period", C.c_int64),
        ("use_graphs", C.c_int),
        ("flexible", C.c_int),
        ("refine", C.c_int),
        ("inner_rtol", C.c_double),
    ]


def library_path() -> str:
    return _build.LIB


def lib():
    """Loads liblineal_gb300.so (building it first when sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        raise LinealLibraryMissing(
            f"{path} is missing: run lineal_gb300.build.build() (nvcc, sm_103a) first")
    L = C.CDLL(path)
    _signatures(L)
    _lib = L
    return L


def _signatures(L):
    V, P, I64, I32, D = C.c_void_p, C.POINTER, C.c_int64, C.c_int32, C.c_double
    L.lgx_status_string.restype = C.c_char_p
    L.lgx_status_string.argtypes = [C.c_int]
    L.lgx_last_error.restype = C.c_char_p
    L.lgx_version.restype = C.c_char_p
    L.lgx_row_engine_get.restype = C.c_int
    L.lgx_row_engine_get.argtypes = []
    L.lgx_row_engine_set.restype = C.c_int
    L.lgx_row_engine_set.argtypes = [C.c_int]
    L.lgx_stencil_engine_get.restype = C.c_int
    L.lgx_stencil_engine_get.argtypes = []
    L.lgx_stencil_engine_set.restype = C.c_int
    L.lgx_stencil_engine_set.argtypes = [C.c_int]
    L.lgx_amg_grid27.restype = C.c_int
    L.lgx_amg_grid27.argtypes = [C.c_void_p]
    L.lgx_kernel_launches.restype = C.c_uint64
    L.lgx_kernel_launches.argtypes = []
    sigs = {
        "lgx_csr_create": [I64, I64, V, V, V, C.c_int, C.c_int, V, P(V)],
        "lgx_csr_create_host": [I64, I64, V, V, V, C.c_int, C.c_int, P(V)],
        "lgx_csr_download": [V, V, V, V, V],
        "lgx_stencil_create_lookup": [V, V, V, V, D, D, C.c_int, V, P(V)],
        "lgx_stencil_create_value": [V, V, V, D, D, C.c_int, V, P(V)],
        "lgx_stencil_create_lookup_henry": [V, V, V, C.c_uint8, D, V, D, D, C.c_int, V, P(V)],
        "lgx_stencil_create_values": [V, V, V, V, V, D, D, C.c_int, V, P(V)],
        "lgx_matrix_destroy": [V],
        "lgx_matrix_info": [V, P(C.c_int), P(I64), P(I64), P(C.c_int)],
        "lgx_spmv": [V, V, V, V],
        "lgx_spmv_f32": [V, V, V, V],
        "lgx_residual": [V, V, V, V, V, V],
        "lgx_diagonal": [V, V, V],
        "lgx_stencil_rhs": [V, V, V],
        "lgx_stencil_effective_diffusion": [V, V, C.c_uint8, V, V, V, P(D), P(D)],
        "lgx_stencil_to_csr": [V, V, V, P(V)],
        "lgx_gen_27pt": [V, V, C.c_int, V, P(V)],
        "lgx_gen_7pt": [V, V, C.c_int, V, P(V)],
        "lgx_csr_set_grid27": [V, V],
        "lgx_csr_set_grid7": [V, V],
        "lgx_dot": [I64, V, V, V, V],
        "lgx_dot_static": [I64, V, V, V, V],
        "lgx_norm2sq": [I64, V, V, V],
        "lgx_max_norm": [I64, V, V, V],
        "lgx_axpy": [I64, D, V, V, V],
        "lgx_jacobi_sweep": [V, D, V, V, V, V],
        "lgx_colouring_create_jp": [V, C.c_uint64, V, P(V)],
        "lgx_colouring_create": [V, V, I32, V, P(V)],
        "lgx_colouring_destroy": [V],
        "lgx_colouring_grid27": [V, V, C.c_int, V, P(C.c_int)],
        "lgx_colouring_export": [V, V, P(I32), V],
        "lgx_sor_sweep": [V, V, D, C.c_int, C.c_int, V, V, V, V],
        "lgx_colouring_permute": [V, V, V, V],
        "lgx_colouring_unpermute": [V, V, V, V],
        "lgx_sor_sweep_permuted": [V, D, C.c_int, C.c_int, V, V, V],
        "lgx_sor_sweep_permuted_f32": [V, C.c_float, C.c_int, C.c_int, V, V, V],
        "lgx_amg_setup": [V, P(_AmgParams), V, V, P(V)],
        "lgx_amg_destroy": [V],
        "lgx_direct_create": [V, C.c_int, V, P(V)],
        "lgx_lincomb": [I64, D, V, D, V, V, V],
        "lgx_fill": [I64, D, V, V],
        "lgx_direct_solve": [V, V, V, V],
        "lgx_direct_destroy": [V],
        "lgx_amg_info": [V, P(I64), V, V, I64],
        "lgx_amg_level_download": [V, I64, V, V, V, V, V],
        "lgx_amg_level_lists": [V, I64, V, V, V, V],
        "lgx_amg_setup_log": [V, P(_AmgLevelLog), I64, P(I64), P(C.c_int32)],
        "lgx_colour_smallest_last": [I64, V, V, V, P(C.c_int32)],
        "lgx_amg_setup_given": [V, P(_AmgParams), V, P(_AggMap), I64, V, P(V)],
        "lgx_agg_map_check": [P(_AggMap), I64],
        "lgx_amg_vcycle": [V, V, V, V],
        "lgx_matrix_autotune": [V, C.c_int, P(_TuneEntry), V],
        "lgx_amg_autotune": [V, C.c_int, P(_TuneEntry), C.c_int, P(C.c_int), V],
        "lgx_amg_autotune_reset": [V],
        "lgx_amg_strength": [V, D, V, V, V, V],
        "lgx_amg_aggregate": [V, V, V, V, I32, I32, I64, C.c_int, V, P(I64), V],
        "lgx_batch_convdiff_bicgstab": [C.c_int32, V, V, V, D, I64, I64, D, V, V, V, V],
        "lgx_sampled_outer": [V, D, V, V, V, V],
        "lgx_residual_compensated": [V, V, V, V, V],
        "lgx_diffusion7_grad": [V, V, V, V, V, V],
        "lgx_pcg": [V, V, V, P(_SolveParams), V, P(I64), P(D), V],
        "lgx_pcg_multi": [V, V, C.c_int32, V, V, D, I64, C.c_int, V, V, V],
        "lgx_pbicgstab": [V, V, V, P(_SolveParams), V, P(I64), P(D), V],
    }
    for name, args in sigs.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.lgx_amg_default_params.argtypes = [P(_AmgParams)]
    L.lgx_amg_default_params.restype = None
    L.lgx_solve_default_params.argtypes = [P(_SolveParams)]
    L.lgx_solve_default_params.restype = None


def _check(status: int):
    if status != 0:
        raise LinealError(status, lib().lgx_last_error().decode())


def _torch():
    import torch
    return torch


def _stream():
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t) -> C.c_void_p:
    if t is None:
        return C.c_void_p(0)
    if isinstance(t, np.ndarray):
        return t.ctypes.data_as(C.c_void_p)
    return C.c_void_p(t.data_ptr())


def _dvec(t, dtype=None):
    """Contiguous CUDA tensor of the requested dtype."""
    torch = _torch()
    dtype = dtype or torch.float64
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(np.ascontiguousarray(t))
    return t.to(device="cuda", dtype=dtype).contiguous()


def _empty(n: int, dtype=None):
    torch = _torch()
    return torch.empty(max(int(n), 0), dtype=dtype or torch.float64, device="cuda")


# ---------------------------------------------------------------------------
# Matrices
# ---------------------------------------------------------------------------
class _Matrix:
    def __init__(self, handle: C.c_void_p):
        self._h = handle

    @property
    def handle(self):
        return self._h

    def info(self):
        kind, n, nnz, sym = C.c_int(), C.c_int64(), C.c_int64(), C.c_int()
        _check(lib().lgx_matrix_info(self._h, C.byref(kind), C.byref(n), C.byref(nnz),
                                     C.byref(sym)))
        return kind.value, n.value, nnz.value, bool(sym.value)

    @property
    def kind(self) -> int:
        return self.info()[0]

    def row_num(self) -> int:
        return self.info()[1]

    def column_num(self) -> int:
        return self.info()[1]

    def non_zero_num(self) -> int:
        return self.info()[2]

    def is_symmetric(self) -> bool:
        return self.info()[3]

    def __mul__(self, x):
        return spmv(self, x)

    def spmv(self, x, out=None):
        return spmv(self, x, out)

    def set_grid27(self, dims):
        """Declares this CSR matrix a 27-point operator on the grid `dims`
        (as gen_27pt's matrices are)."""
        d = np.ascontiguousarray(dims, dtype=np.int64)
        _check(lib().lgx_csr_set_grid27(self._h, _ptr(d)))

    def set_grid7(self, dims):
        """Declares this CSR matrix a 7-point operator on the grid `dims`
        (as gen_7pt's matrices are)."""
        d = np.ascontiguousarray(dims, dtype=np.int64)
        _check(lib().lgx_csr_set_grid7(self._h, _ptr(d)))

    def autotune(self, reps: int = 5) -> dict:
        """Times every row-engine configuration on this CSR matrix's FP64
        SpMV and keeps the fastest for it; returns the timings."""
        e = _TuneEntry()
        _check(lib().lgx_matrix_autotune(self._h, int(reps), C.byref(e), _stream()))
        return e.as_dict()

    def diagonal(self):
        d = _empty(self.row_num())
        _check(lib().lgx_diagonal(self._h, _ptr(d), _stream()))
        return d

    def close(self):
        if self._h:
            lib().lgx_matrix_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CsrMatrix(_Matrix):
    """CsrMatrix (tensor/dynamic/csr/shared.hpp): sorted columns, stored diagonal."""

    @classmethod
    def from_host(cls, rowptr, col, val, symmetric=True, storage=F64) -> "CsrMatrix":
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        col = np.ascontiguousarray(col, dtype=np.int32)
        val = np.ascontiguousarray(val, dtype=np.float64)
        n = len(rowptr) - 1
        h = C.c_void_p()
        _check(lib().lgx_csr_create_host(n, int(rowptr[-1]), _ptr(rowptr), _ptr(col), _ptr(val),
                                         int(symmetric), storage, C.byref(h)))
        return cls(h)

    @classmethod
    def from_device(cls, rowptr, col, val, symmetric=True, storage=F64) -> "CsrMatrix":
        torch = _torch()
        rowptr = _dvec(rowptr, torch.int64)
        col = _dvec(col, torch.int32)
        val = _dvec(val, torch.float64)
        h = C.c_void_p()
        _check(lib().lgx_csr_create(rowptr.numel() - 1, col.numel(), _ptr(rowptr), _ptr(col),
                                    _ptr(val), int(symmetric), storage, _stream(), C.byref(h)))
        return cls(h)

    def download(self):
        _, n, nnz, _ = self.info()
        rowptr = np.empty(n + 1, dtype=np.int64)
        col = np.empty(nnz, dtype=np.int32)
        val = np.empty(nnz, dtype=np.float64)
        _check(lib().lgx_csr_download(self._h, _ptr(rowptr), _ptr(col), _ptr(val), _stream()))
        return rowptr, col, val


class _BoxInfo(C.Structure):
    _fields_ = [("cells", C.c_int64 * 3), ("lengths", C.c_double * 3)]


class BoxInfo:
    """BoxInfo (discretization/box-equidistant.hpp:57-110): cell counts and
    axis lengths of an equidistant box; axis_quotients() are the stencil
    valuators' geometric factors q_d = prod_{e != d} h_e / h_d, h = L / N."""

    def __init__(self, cells, lengths):
        self.cells = tuple(int(c) for c in cells)
        self.lengths = tuple(float(v) for v in lengths)
        if len(self.cells) != 3 or len(self.lengths) != 3:
            raise ValueError("BoxInfo needs three cell counts and three axis lengths")

    def axis_quotients(self) -> np.ndarray:
        box = _BoxInfo((C.c_int64 * 3)(*self.cells), (C.c_double * 3)(*self.lengths))
        q = np.zeros(3)
        _check(lib().lgx_box_axis_quotients(C.byref(box), _ptr(q)))
        return q


def _box_q(dims, q):
    """(dims, q) from a BoxInfo given as dims (q then must be None), else as given"""
    if isinstance(dims, BoxInfo):
        if q is not None:
            raise ValueError("give either a BoxInfo or dims with q, not both")
        return dims.cells, dims.axis_quotients()
    if q is None:
        raise ValueError("q (axis quotients) is required unless dims is a BoxInfo")
    return dims, q


class StencilMatrix(_Matrix):
    """AdjacentStencilMatrix over a stationary-diffusion valuator (7-point,
    Dirichlet on the faces of axis 0)."""

    @classmethod
    def lookup(cls, dims, q, coeffs, materials, sol_start=1.0, sol_end=0.0,
               zero_to_one=True) -> "StencilMatrix":
        """Lookup valuator; dims may be a BoxInfo (then q=None)."""
        torch = _torch()
        dims, q = _box_q(dims, q)
        d = np.ascontiguousarray(dims, dtype=np.int64)
        qq = np.ascontiguousarray(q, dtype=np.float64)
        cc = np.ascontiguousarray(coeffs, dtype=np.float64)
        mat = _dvec(materials, torch.uint8)
        h = C.c_void_p()
        _check(lib().lgx_stencil_create_lookup(_ptr(d), _ptr(qq), _ptr(cc), _ptr(mat), sol_start,
                                               sol_end, int(zero_to_one), _stream(), C.byref(h)))
        return cls(h)

    @classmethod
    def value(cls, dims, q, k, sol_start=1.0, sol_end=0.0, zero_to_one=True) -> "StencilMatrix":
        """Value valuator; dims may be a BoxInfo (then q=None)."""
        dims, q = _box_q(dims, q)
        d = np.ascontiguousarray(dims, dtype=np.int64)
        qq = np.ascontiguousarray(q, dtype=np.float64)
        kk = _dvec(k)
        h = C.c_void_p()
        _check(lib().lgx_stencil_create_value(_ptr(d), _ptr(qq), _ptr(kk), sol_start, sol_end,
                                              int(zero_to_one), _stream(), C.byref(h)))
        return cls(h)

    @classmethod
    def lookup_henry(cls, dims, q, coeffs, materials, henry, gaseous_mask, sol_start=1.0,
                     sol_end=0.0, zero_to_one=True) -> "StencilMatrix":
        """Lookup valuator with the Henry-law diffusion factors; dims may be a
        BoxInfo (then q=None)."""
        torch = _torch()
        dims, q = _box_q(dims, q)
        d = np.ascontiguousarray(dims, dtype=np.int64)
        qq = np.ascontiguousarray(q, dtype=np.float64)
        cc = np.ascontiguousarray(coeffs, dtype=np.float64)
        mat = _dvec(materials, torch.uint8)
        h = C.c_void_p()
        _check(lib().lgx_stencil_create_lookup_henry(
            _ptr(d), _ptr(qq), _ptr(cc), int(gaseous_mask), float(henry), _ptr(mat), sol_start,
            sol_end, int(zero_to_one), _stream(), C.byref(h)))
        return cls(h)

    @classmethod
    def values(cls, dims, q, k_axes, sol_start=1.0, sol_end=0.0,
               zero_to_one=True) -> "StencilMatrix":
        """StationaryDiffusionValuesValuator: one conductivity array per axis;
        dims may be a BoxInfo (then q=None)."""
        dims, q = _box_q(dims, q)
        d = np.ascontiguousarray(dims, dtype=np.int64)
        qq = np.ascontiguousarray(q, dtype=np.float64)
        k0, k1, k2 = (_dvec(v) for v in k_axes)
        h = C.c_void_p()
        _check(lib().lgx_stencil_create_values(_ptr(d), _ptr(qq), _ptr(k0), _ptr(k1), _ptr(k2),
                                               sol_start, sol_end, int(zero_to_one), _stream(),
                                               C.byref(h)))
        return cls(h)

    def rhs(self):
        b = _empty(self.row_num())
        _check(lib().lgx_stencil_rhs(self._h, _ptr(b), _stream()))
        return b

    def effective_diffusion(self, lengths, sol, compress_map=None, none_mask=0):
        """EffDiffCalc: (effective diffusivity, area part) of the solution
        `sol` (with `compress_map` for a compressed system)."""
        torch = _torch()
        le = np.ascontiguousarray(lengths, dtype=np.float64)
        x = _dvec(sol)
        cm = _dvec(compress_map, torch.int64) if compress_map is not None else None
        eff, ap = C.c_double(), C.c_double()
        _check(lib().lgx_stencil_effective_diffusion(self._h, _ptr(le), int(none_mask), _ptr(x),
                                                     _ptr(cm), _stream(), C.byref(eff),
                                                     C.byref(ap)))
        return eff.value, ap.value

    def to_csr(self, with_compress_map=False):
        torch = _torch()
        cmap = _empty(self.row_num(), torch.int64) if with_compress_map else None
        h = C.c_void_p()
        _check(lib().lgx_stencil_to_csr(self._h, _ptr(cmap), _stream(), C.byref(h)))
        m = CsrMatrix(h)
        return (m, cmap) if with_compress_map else m


def gen_27pt(dims, k, storage=F64) -> CsrMatrix:
    d = np.ascontiguousarray(dims, dtype=np.int64)
    kk = _dvec(k)
    h = C.c_void_p()
    _check(lib().lgx_gen_27pt(_ptr(d), _ptr(kk), storage, _stream(), C.byref(h)))
    return CsrMatrix(h)


def gen_7pt(dims, k, storage=F64) -> CsrMatrix:
    d = np.ascontiguousarray(dims, dtype=np.int64)
    kk = _dvec(k)
    h = C.c_void_p()
    _check(lib().lgx_gen_7pt(_ptr(d), _ptr(kk), storage, _stream(), C.byref(h)))
    return CsrMatrix(h)


# ---------------------------------------------------------------------------
# Kernels
# ---------------------------------------------------------------------------
def spmv(a: _Matrix, x, out=None):
    x = _dvec(x)
    y = out if out is not None else _empty(a.row_num())
    _check(lib().lgx_spmv(a.handle, _ptr(x), _ptr(y), _stream()))
    return y


def spmv_f32(a: _Matrix, x, out=None):
    torch = _torch()
    x = _dvec(x, torch.float32)
    y = out if out is not None else _empty(a.row_num(), torch.float32)
    _check(lib().lgx_spmv_f32(a.handle, _ptr(x), _ptr(y), _stream()))
    return y


def residual(a: _Matrix, b, x, with_norm=True):
    b, x = _dvec(b), _dvec(x)
    r = _empty(a.row_num())
    nrm = _empty(1) if with_norm else None
    _check(lib().lgx_residual(a.handle, _ptr(b), _ptr(x), _ptr(r), _ptr(nrm), _stream()))
    return (r, float(nrm.item())) if with_norm else r


def dot(a, b) -> float:
    a, b = _dvec(a), _dvec(b)
    out = _empty(1)
    _check(lib().lgx_dot(a.numel(), _ptr(a), _ptr(b), _ptr(out), _stream()))
    return float(out.item())


def norm2sq(a) -> float:
    a = _dvec(a)
    out = _empty(1)
    _check(lib().lgx_norm2sq(a.numel(), _ptr(a), _ptr(out), _stream()))
    return float(out.item())


def max_norm(a) -> float:
    a = _dvec(a)
    out = _empty(1)
    _check(lib().lgx_max_norm(a.numel(), _ptr(a), _ptr(out), _stream()))
    return float(out.item())


def lincomb(alpha: float, x, beta: float = 0.0, y=None, out=None):
    """alpha x + beta y (y None: alpha x) with each product and the sum
    rounded on its own, the bits of lineal's add / subtract / scale
    expressions (component-wise/vector-expression.hpp:67-91)."""
    x = _dvec(x)
    if y is not None:
        y = _dvec(y)
        if y.numel() != x.numel():
            raise ValueError("x and y differ in size")
    out = out if out is not None else _empty(x.numel())
    _check(lib().lgx_lincomb(x.numel(), float(alpha), _ptr(x), float(beta), _ptr(y), _ptr(out),
                             _stream()))
    return out


def fill(n: int, value: float, out=None):
    out = out if out is not None else _empty(n)
    _check(lib().lgx_fill(out.numel(), float(value), _ptr(out), _stream()))
    return out


def jacobi_sweep(a: _Matrix, b, x_in=None, relax=1.0):
    b = _dvec(b)
    xi = None if x_in is None else _dvec(x_in)
    out = _empty(a.row_num())
    _check(lib().lgx_jacobi_sweep(a.handle, relax, _ptr(xi), _ptr(out), _ptr(b), _stream()))
    return out


class Colouring:
    """Graph colouring driving the multicolour SOR sweeps."""

    def __init__(self, handle: C.c_void_p, n: int):
        self._h = handle
        self.n = n

    @classmethod
    def jp(cls, a: CsrMatrix, seed: int = 0x5EED) -> "Colouring":
        h = C.c_void_p()
        _check(lib().lgx_colouring_create_jp(a.handle, seed, _stream(), C.byref(h)))
        return cls(h, a.row_num())

    @classmethod
    def red_black(cls, a: "StencilMatrix") -> "Colouring":
        """Red-black colouring of a stencil matrix: its SOR sweeps run
        matrix-free in natural order."""
        h = C.c_void_p()
        _check(lib().lgx_colouring_create_red_black(a.handle, _stream(), C.byref(h)))
        return cls(h, a.row_num())

    @classmethod
    def from_array(cls, a: CsrMatrix, colours, ncolours: int | None = None) -> "Colouring":
        torch = _torch()
        c = _dvec(colours, torch.int32)
        nc = int(c.max().item()) + 1 if ncolours is None else ncolours
        h = C.c_void_p()
        _check(lib().lgx_colouring_create(a.handle, _ptr(c), nc, _stream(), C.byref(h)))
        return cls(h, a.row_num())

    def export(self):
        torch = _torch()
        out = _empty(self.n, torch.int32)
        nc = C.c_int32()
        _check(lib().lgx_colouring_export(self._h, _ptr(out), C.byref(nc), _stream()))
        return out, nc.value

    def use_grid27(self, dims, with_float: bool = True) -> bool:
        """Sweeps through the 27-point grid kernels when this is the parity
        colouring of a 27-point operator on `dims`; returns whether they
        were attached (bit-identical results either way)."""
        d = np.ascontiguousarray(dims, dtype=np.int64)
        att = C.c_int()
        _check(lib().lgx_colouring_grid27(self._h, _ptr(d), int(with_float), _stream(),
                                          C.byref(att)))
        return bool(att.value)

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().lgx_colouring_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def colour_smallest_last(rowptr, col):
    """Smallest-last greedy colouring of a host CSR pattern
    (lgx_colour_smallest_last, host code): (colour int32[n], ncolours); give
    the colours to ``Colouring.from_array`` for a multicolour smoother."""
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    n = len(rowptr) - 1
    colour = np.empty(max(n, 1), dtype=np.int32)
    nc = C.c_int32()
    _check(lib().lgx_colour_smallest_last(n, _ptr(rowptr), _ptr(col), _ptr(colour),
                                          C.byref(nc)))
    return colour[:n], nc.value


def stencil_engine(engine: int | None = None) -> int:
    """Selects (when given) and returns the stencil kernel: 0 thread per
    cell, 1 plane march with TMA-staged x planes."""
    if engine is not None:
        _check(lib().lgx_stencil_engine_set(int(engine)))
    return int(lib().lgx_stencil_engine_get())


def row_engine(config: int | None = None) -> int:
    """Returns the CSR row-kernel configuration; sets it first when given."""
    if config is not None:
        _check(lib().lgx_row_engine_set(int(config)))
    return int(lib().lgx_row_engine_get())


def permute(colouring: Colouring, v):
    """v in the colouring's row order (out[r] = v[perm[r]])."""
    v = _dvec(v)
    out = _empty(v.numel())
    _check(lib().lgx_colouring_permute(colouring.handle, _ptr(v), _ptr(out), _stream()))
    return out


def unpermute(colouring: Colouring, v):
    """Inverse of permute (out[perm[r]] = v[r])."""
    v = _dvec(v)
    out = _empty(v.numel())
    _check(lib().lgx_colouring_unpermute(colouring.handle, _ptr(v), _ptr(out), _stream()))
    return out


def sor_sweep_permuted(colouring: Colouring, b_perm, x_perm, relax=1.0, forward=True,
                       ultra=False):
    """One multicolour SOR sweep in the colouring's row order, in place on
    x_perm (float64 vectors: FP64 arithmetic; float32 vectors: the float
    smoother of the precision form)."""
    torch = _torch()
    if x_perm.dtype == torch.float32:
        b_perm = _dvec(b_perm, torch.float32)
        _check(lib().lgx_sor_sweep_permuted_f32(colouring.handle, float(relax), int(forward),
                                                int(ultra), _ptr(x_perm), _ptr(b_perm),
                                                _stream()))
    else:
        b_perm = _dvec(b_perm)
        _check(lib().lgx_sor_sweep_permuted(colouring.handle, float(relax), int(forward),
                                            int(ultra), _ptr(x_perm), _ptr(b_perm), _stream()))
    return x_perm


def sor_sweep(a: CsrMatrix, colouring: Colouring, b, x_in=None, relax=1.0, forward=True,
              ultra=False, out=None):
    b = _dvec(b)
    xi = None if x_in is None else _dvec(x_in)
    y = out if out is not None else _empty(a.row_num())
    _check(lib().lgx_sor_sweep(a.handle, colouring.handle, relax, int(forward), int(ultra),
                               _ptr(xi), _ptr(y), _ptr(b), _stream()))
    return y


# ---------------------------------------------------------------------------
# AMG
# ---------------------------------------------------------------------------
@dataclass
class HierarchyWright:
    """HierarchyWrightParams + AggregationParams + DuneDependencyCriterion
    (hierarchy/wright.hpp:46-55, aggregation/params.hpp:13-20,
    dependency/criterion.hpp:103-118)."""

    max_level_num: int = 16
    min_coarsen_size: int = 2000
    min_coarsen_factor: float = 1.2
    strong_threshold: float = 1.0 / 3.0
    aggressive_threshold: float = 1.0 / 3.0
    min_aggregate_size: int = 6
    max_aggregate_size: int = 9
    partition_size: int = 4096
    partition_growth: float = 4.0
    min_partitions: int = 8
    max_partitions: int = 1 << 30
    coarse_f32: bool = False
    cycle_f32: bool = False
    relax: float = 1.0
    smoother_relax: float = 1.0
    smoother_ultra: bool = False
    colour_seed: int = 0x5EED
    cycle_bf16: bool = False
    grid27: bool = True
    coarse_smallest_last: bool = False

    def params(self) -> _AmgParams:
        p = _AmgParams()
        lib().lgx_amg_default_params(C.byref(p))
        for f in self.__dataclass_fields__:
            v = getattr(self, f)
            setattr(p, f, int(v) if isinstance(v, bool) else v)
        return p

    def instantiate(self, a: CsrMatrix, finest_colouring: Colouring | None = None,
                    aggregates=None) -> "Hierarchy":
        """The hierarchy of ``a``.  With ``aggregates`` (per level an
        ``io.AggregateMap`` or an (agg, list_ptr, list) triple, e.g. from
        ``io.load_aggregates``) level k takes aggregates[k] instead of
        computing its aggregation, as lineal's FileAggregator does
        (aggregation/independent.hpp:279-298)."""
        p = self.params()
        h = C.c_void_p()
        col = finest_colouring.handle if finest_colouring else None
        if aggregates is None:
            _check(lib().lgx_amg_setup(a.handle, C.byref(p), col, _stream(), C.byref(h)))
        else:
            maps, _keep = _agg_maps(aggregates)
            _check(lib().lgx_amg_setup_given(a.handle, C.byref(p), col, maps, len(_keep) // 3,
                                             _stream(), C.byref(h)))
        return Hierarchy(h, a)


class _AggMap(C.Structure):
    _fields_ = [("n", C.c_int64), ("ncoarse", C.c_int64), ("agg", C.c_void_p),
                ("list_ptr", C.c_void_p), ("list", C.c_void_p)]


def agg_map_check(m, n: int | None = None) -> None:
    """The host-side checks of a given aggregate map (lgx_agg_map_check) for
    a level of n rows (default: the map's own fine size); raises LinealError."""
    maps, _keep = _agg_maps([m])
    _check(lib().lgx_agg_map_check(maps, maps[0].n if n is None else int(n)))


def _agg_maps(aggregates):
    """host lgx_agg_map array for lgx_amg_setup_given, plus the arrays it
    points into (kept alive by the caller)"""
    keep = []
    maps = (_AggMap * max(len(aggregates), 1))()
    for k, (agg, list_ptr, lst) in enumerate(aggregates):
        agg = np.ascontiguousarray(agg, dtype=np.uint32)
        list_ptr = np.ascontiguousarray(list_ptr, dtype=np.int64)
        lst = np.ascontiguousarray(lst, dtype=np.int32)
        if list_ptr.ndim != 1 or len(list_ptr) < 1:
            raise ValueError(f"aggregate map {k}: list_ptr needs ncoarse + 1 entries")
        if int(list_ptr[-1]) > len(lst):
            raise ValueError(f"aggregate map {k}: list shorter than its offsets say")
        keep += [agg, list_ptr, lst]
        maps[k] = _AggMap(len(agg), len(list_ptr) - 1, agg.ctypes.data, list_ptr.ctypes.data,
                          lst.ctypes.data)
    if not keep:
        raise ValueError("no aggregate maps given")
    return maps, keep


class Hierarchy:
    def __init__(self, handle, matrix):
        self._h = handle
        self._a = matrix  # the finest matrix must outlive the hierarchy

    @property
    def handle(self):
        return self._h

    def level_num(self) -> int:
        return len(self.sizes()[0])

    def sizes(self):
        L = C.c_int64()
        rows = np.zeros(32, dtype=np.int64)
        nnz = np.zeros(32, dtype=np.int64)
        _check(lib().lgx_amg_info(self._h, C.byref(L), _ptr(rows), _ptr(nnz), 32))
        return rows[: L.value].tolist(), nnz[: L.value].tolist()

    def level(self, l: int, with_agg: bool = True):
        rows, nnz = self.sizes()
        n, m = rows[l], nnz[l]
        rowptr = np.empty(n + 1, dtype=np.int64)
        col = np.empty(m, dtype=np.int32)
        val = np.empty(m, dtype=np.float64)
        agg = np.empty(n, dtype=np.uint32) if with_agg and l + 1 < len(rows) else None
        _check(lib().lgx_amg_level_download(self._h, l, _ptr(rowptr), _ptr(col), _ptr(val),
                                            _ptr(agg), _stream()))
        return rowptr, col, val, agg

    def setup_log(self) -> dict:
        """The hierarchy setup in the shape of lineal's JSON log
        (hierarchy/wright.hpp:26-31, 120-143, 210-225; aggregation/stats.hpp:
        16-32): per level its dimensions, non-zeros, aggregation statistics
        and aggressive mode, and why coarsening stopped."""
        cap = 32
        levels = (_AmgLevelLog * cap)()
        n, reason = C.c_int64(), C.c_int32()
        _check(lib().lgx_amg_setup_log(self._h, levels, cap, C.byref(n), C.byref(reason)))
        out = []
        for l in range(min(n.value, cap)):
            e = levels[l]
            entry = {"dimensions": {"rows": e.rows, "columns": e.columns}, "non_zeros": e.nnz}
            if l + 1 < n.value:
                entry["aggressive"] = bool(e.aggressive)
                entry["given_map"] = bool(e.given_map)
                entry["aggregation_stats"] = {
                    k: getattr(e, k) for k in (
                        "aggregate_num", "multi_vertex_aggregate_num",
                        "single_vertex_aggregate_num", "merged_aggregate_num",
                        "isolated_aggregate_num")}
            out.append(entry)
        return {"create_hierarchy": {"levels": out, "stop_coarsening": {
            "reason": STOP_REASONS.get(reason.value, "unknown")}}}

    def aggregate_map(self, l: int):
        """Level l's aggregates as an ``io.AggregateMap``: the fine -> coarse
        ids and the coarse -> fine lists in the order aggregation added the
        vertices (natural ordering)."""
        from . import io as _io

        rows, _ = self.sizes()
        if not 0 <= l < len(rows) - 1:
            raise IndexError(f"level {l} has no aggregate map")
        agg = np.empty(rows[l], dtype=np.uint32)
        _check(lib().lgx_amg_level_download(self._h, l, None, None, None, _ptr(agg), _stream()))
        list_ptr = np.empty(rows[l + 1] + 1, dtype=np.int64)
        total = C.c_int64()
        _check(lib().lgx_amg_level_lists(self._h, l, _ptr(list_ptr), None, C.byref(total),
                                         _stream()))
        lst = np.empty(max(total.value, 1), dtype=np.int32)
        _check(lib().lgx_amg_level_lists(self._h, l, None, _ptr(lst), None, _stream()))
        return _io.AggregateMap(agg, list_ptr, lst[: total.value])

    def aggregate_maps(self) -> list:
        return [self.aggregate_map(l) for l in range(self.level_num() - 1)]

    def save_aggregates(self, base: str) -> list:
        """Writes every level's aggregate map to ``<base><level>.aggs``, as
        lineal's RefinedAggregator does with ``base_agg_map_path``
        (aggregation/independent.hpp:264-272); returns the paths."""
        from . import io as _io

        return _io.save_aggregates(base, self.aggregate_maps())

    def vcycle(self, b, out=None):
        b = _dvec(b)
        x = out if out is not None else _empty(b.numel())
        _check(lib().lgx_amg_vcycle(self._h, _ptr(b), _ptr(x), _stream()))
        return x

    def autotune(self, reps: int = 5) -> list:
        """Times every row-engine configuration on each smoothed level's
        residual and SOR sweep (and, for FP32 cycles, the finest FP64
        product) and keeps the fastest per level; returns the timings."""
        n = C.c_int()
        cap = 2 * self.level_num() + 1  # residual and sweep per level, finest product
        entries = (_TuneEntry * cap)()
        _check(lib().lgx_amg_autotune(self._h, int(reps), entries, cap, C.byref(n), _stream()))
        return [entries[i].as_dict() for i in range(min(n.value, cap))]

    def autotune_reset(self):
        _check(lib().lgx_amg_autotune_reset(self._h))

    def grid27_active(self) -> bool:
        """Whether the finest level runs the 27-point grid kernels."""
        return bool(lib().lgx_amg_grid27(self._h))

    def close(self):
        if self._h:
            lib().lgx_amg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DirectSolver:
    """FP64 direct solver: lineal's CholeskySolver (positive pivots) or
    LuSolver (nonzero pivots, no pivoting), direct/cholesky/solver.hpp:22-67,
    direct/lu/solver.hpp:21-66.  ``lu=None`` picks Cholesky for a matrix
    created symmetric.  Up to DIRECT_MAX_ROWS rows the inverse is formed
    once and each solve is one dense product; beyond, Cholesky factors in
    the band of the matrix's lower envelope and solves by substitution (LU
    refuses)."""

    def __init__(self, a: CsrMatrix, lu: bool | None = None):
        if lu is None:
            lu = not a.info()[3]
        h = C.c_void_p()
        _check(lib().lgx_direct_create(a.handle, DIRECT_LU if lu else DIRECT_CHOLESKY, _stream(),
                                       C.byref(h)))
        self._h = h
        self._a = a
        self._n = a.row_num()

    def solve(self, b, out=None):
        b = _dvec(b)
        if b.numel() != self._n:
            raise ValueError(f"right-hand side has {b.numel()} entries, the matrix {self._n} rows")
        x = out if out is not None else _empty(self._n)
        _check(lib().lgx_direct_solve(self._h, _ptr(b), _ptr(x), _stream()))
        return x

    def close(self):
        if self._h:
            lib().lgx_direct_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


DIRECT_MAX_ROWS = 8192
DIRECT_CHOLESKY, DIRECT_LU = 0, 1


def amg_strength(a: CsrMatrix, theta: float = 1.0 / 3.0):
    torch = _torch()
    _, n, nnz, _ = a.info()
    dep = _empty(nnz, torch.uint8)
    inf = _empty(nnz, torch.uint8)
    iso = _empty(n, torch.uint8)
    _check(lib().lgx_amg_strength(a.handle, theta, _ptr(dep), _ptr(inf), _ptr(iso), _stream()))
    return dep, inf, iso


def amg_aggregate(a: CsrMatrix, dep, inf, iso, min_size=6, max_size=9, nparts=1,
                  aggressive=False):
    torch = _torch()
    agg = _empty(a.row_num(), torch.int32)
    nc = C.c_int64()
    _check(lib().lgx_amg_aggregate(a.handle, _ptr(dep), _ptr(inf), _ptr(iso), min_size, max_size,
                                   nparts, int(aggressive), _ptr(agg), C.byref(nc), _stream()))
    return nc.value, agg.cpu().numpy().view(np.uint32)


# ---------------------------------------------------------------------------
# Krylov solvers
# ---------------------------------------------------------------------------
@dataclass
class SolveResult:
    x: object
    iterations: int
    rel_residual: float
    history: np.ndarray = field(repr=False)


def _solve(fn, a: _Matrix, b, x0=None, precon=PRECON_NONE, relax=1.0, ultra=False,
           colouring: Colouring | None = None, amg: Hierarchy | None = None, rtol=1e-8,
           maxit=1000, rere_period=8, use_graphs=True, flexible=False, refine=False,
           inner_rtol=1e-4) -> SolveResult:
    b = _dvec(b)
    x = _dvec(x0) if x0 is not None else _empty(b.numel()).zero_()
    if x0 is not None:
        x = x.clone()
    p = _SolveParams()
    lib().lgx_solve_default_params(C.byref(p))
    p.precon = precon
    p.relax = relax
    p.ultra = int(ultra)
    p.colouring = colouring.handle if colouring else None
    p.amg = amg.handle if amg else None
    p.rtol = rtol
    p.maxit = maxit
    p.rere_period = rere_period
    p.use_graphs = int(use_graphs)
    p.flexible = int(flexible)
    p.refine = int(refine)
    p.inner_rtol = inner_rtol
    it = C.c_int64()
    rel = C.c_double()
    hist = np.zeros(maxit + 1)
    _check(fn(a.handle, _ptr(b), _ptr(x), C.byref(p), _stream(), C.byref(it), C.byref(rel),
              _ptr(hist)))
    return SolveResult(x, it.value, rel.value, hist[: it.value + 1])


class _ConvDiffSystem(C.Structure):
    _fields_ = [("dims", C.c_int64 * 3), ("v", C.c_double * 3)]


@dataclass
class BatchResult:
    x: object
    iterations: np.ndarray
    rel_residual: np.ndarray
    status: np.ndarray


def batch_convdiff_bicgstab(systems, b, x0=None, rtol=1e-8, maxit=1000, rere_period=8,
                            relax=1.0) -> BatchResult:
    """Jacobi-BiCGStab on many convection-diffusion systems in one persistent
    launch; systems = [(dims, v), ...], b the concatenated right-hand sides."""
    ns = len(systems)
    arr = (_ConvDiffSystem * max(ns, 1))()
    for i, (dims, v) in enumerate(systems):
        arr[i].dims[:] = [int(d) for d in dims]
        arr[i].v[:] = [float(c) for c in v]
    b = _dvec(b)
    x = _dvec(x0).clone() if x0 is not None else _empty(b.numel()).zero_()
    it = np.zeros(max(ns, 1), dtype=np.int64)
    rel = np.zeros(max(ns, 1))
    st = np.zeros(max(ns, 1), dtype=np.int32)
    _check(lib().lgx_batch_convdiff_bicgstab(ns, arr, _ptr(b), _ptr(x), float(rtol), int(maxit),
                                             int(rere_period), float(relax), _stream(),
                                             _ptr(it), _ptr(rel), _ptr(st)))
    return BatchResult(x, it[:ns], rel[:ns], st[:ns])


def sampled_outer(a: CsrMatrix, u, v, alpha=1.0):
    """alpha * u[row(e)] * v[col(e)] for every stored entry e of a (nnz
    values in storage order)."""
    u, v = _dvec(u), _dvec(v)
    out = _empty(a.non_zero_num())
    _check(lib().lgx_sampled_outer(a.handle, float(alpha), _ptr(u), _ptr(v), _ptr(out),
                                   _stream()))
    return out


def residual_compensated(a: CsrMatrix, b, x):
    """b - A x with compensated (twice-FP64-accurate) row sums."""
    b, x = _dvec(b), _dvec(x)
    r = _empty(a.row_num())
    _check(lib().lgx_residual_compensated(a.handle, _ptr(b), _ptr(x), _ptr(r), _stream()))
    return r


def diffusion7_grad(dims, k, lam, x):
    """dL/dtheta of the 7-point operator of gen_7pt with k = exp(theta), from
    the adjoint lam and the solution x."""
    d = np.ascontiguousarray(dims, dtype=np.int64)
    k, lam, x = _dvec(k), _dvec(lam), _dvec(x)
    out = _empty(k.numel())
    _check(lib().lgx_diffusion7_grad(_ptr(d), _ptr(k), _ptr(lam), _ptr(x), _ptr(out),
                                     _stream()))
    return out


def pcg(a: _Matrix, b, **kw) -> SolveResult:
    """Preconditioned CG (ConjugateGradientsSolver); flexible=True selects the
    flexible-CG beta for the float V-cycle of the precision form; refine=True
    (AMG hierarchy with cycle_f32) runs FP64 iterative refinement over a
    float-vector PCG with compensated dots and FP64 scalars, each inner
    solve to inner_rtol."""
    return _solve(lib().lgx_pcg, a, b, **kw)


def pcg_multi(a: CsrMatrix, amg: Hierarchy, b, x0=None, rtol=1e-8, maxit=1000,
              use_graphs=True):
    """Blocked AMG-PCG on up to 32 right-hand sides (columns of the n x k
    array b); returns (X, iterations per column, relative residual per
    column).  use_graphs replays a CUDA-graph recording of the iteration."""
    torch = _torch()
    b = _dvec(b)
    if b.dim() == 1:
        b = b.reshape(-1, 1)
    n, k = b.shape
    b = b.contiguous()
    x = (_dvec(x0).reshape(n, k).clone() if x0 is not None
         else torch.zeros((n, k), dtype=torch.float64, device="cuda"))
    it = np.zeros(k, dtype=np.int64)
    rel = np.zeros(k)
    _check(lib().lgx_pcg_multi(a.handle, amg.handle, int(k), _ptr(b), _ptr(x), float(rtol),
                               int(maxit), int(use_graphs), _stream(), _ptr(it), _ptr(rel)))
    return x, it, rel


def pbicgstab(a: _Matrix, b, **kw) -> SolveResult:
    """Preconditioned BiCGStab (BiCgStabSolver)."""
    return _solve(lib().lgx_pbicgstab, a, b, **kw)


def kernel_launches() -> int:
    """Kernels launched by the library since it was loaded."""
    return int(lib().lgx_kernel_launches())


def version() -> str:
    return lib().lgx_version().decode()
