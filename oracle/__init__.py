"""ctypes front end of the CPU restatement of lineal's solve path.

TEST INFRASTRUCTURE ONLY: this package is the oracle that the CUDA path is
checked against (tests/, ``__graft_entry__.smoke``) and the CPU baseline that
``bench.py`` times.  The product package ``lineal_gb300`` never imports it.

The C sources (``lo_*.c``) restate the reference algorithms; each function
there cites the lineal file:line it follows.  ``build()`` compiles them with
the committed Makefile into ``oracle/_build/liblineal_oracle.so``.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liblineal_oracle.so")
_lib = None

UNAGGREGATED = 0xFFFFFFFF
ISOLATED = 0xFFFFFFFE


def build(force: bool = False) -> str:
    """Compile the restatement (make -C oracle)."""
    if force or not os.path.exists(_LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(_LIB_PATH)
    for f in os.listdir(_HERE):
        if f.endswith((".c", ".h")) or f == "Makefile":
            if os.path.getmtime(os.path.join(_HERE, f)) > t:
                return True
    return False


class _Csr(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("ncols", C.c_int64),
        ("rowptr", C.POINTER(C.c_int64)),
        ("col", C.POINTER(C.c_int32)),
        ("val", C.POINTER(C.c_double)),
        ("symmetric", C.c_int),
        ("is_f32", C.c_int),
    ]


class _Stencil(C.Structure):
    _fields_ = [
        ("dims", C.c_int64 * 3),
        ("q", C.c_double * 3),
        ("k", C.POINTER(C.c_double)),
        ("mat", C.POINTER(C.c_uint8)),
        ("coeffs", C.c_double * 4),
        ("conn", C.c_double * 48),
        ("sol_start", C.c_double),
        ("sol_end", C.c_double),
        ("zero_to_one", C.c_int),
        ("k1", C.POINTER(C.c_double)),
        ("k2", C.POINTER(C.c_double)),
        ("henry", C.c_int),
        ("henry_constant", C.c_double),
        ("gaseous_mask", C.c_int),
    ]


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
        ("relax", C.c_double),
        ("smoother_relax", C.c_double),
        ("smoother_ultra", C.c_int),
        ("smoother_parts", C.c_int64),
        ("colour_seed", C.c_uint64),
        ("coarse_smallest_last", C.c_int),
    ]


class _AmgLevel(C.Structure):
    _fields_ = [
        ("a", _Csr),
        ("agg", C.POINTER(C.c_uint32)),
        ("list_ptr", C.POINTER(C.c_int64)),
        ("list", C.POINTER(C.c_int32)),
        ("order", C.POINTER(C.c_int32)),
        ("colour", C.POINTER(C.c_int32)),
        ("colour_ptr", C.POINTER(C.c_int64)),
        ("ncolours", C.c_int32),
        ("b", C.POINTER(C.c_double)),
        ("x", C.POINTER(C.c_double)),
        ("r", C.POINTER(C.c_double)),
    ]


class _Amg(C.Structure):
    _fields_ = [
        ("nlevels", C.c_int64),
        ("lv", _AmgLevel * 32),
        ("chol", C.POINTER(C.c_double)),
        ("p", _AmgParams),
    ]


class _AggMap(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("ncoarse", C.c_int64),
        ("agg", C.c_void_p),
        ("list_ptr", C.c_void_p),
        ("list", C.c_void_p),
    ]


LO_ERR_NO_MAP, LO_ERR_BAD_MAP = -2, -3


class _Precon(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("relax", C.c_double),
        ("ultra", C.c_int),
        ("nparts", C.c_int64),
        ("amg", C.POINTER(_Amg)),
    ]


PRECON_NONE, PRECON_JACOBI, PRECON_SSOR, PRECON_AMG = 0, 1, 2, 3


def set_threads(n: int) -> None:
    """Thread count of the restatement's OpenMP loops from now on."""
    lib().lo_set_threads(int(n))


def max_threads() -> int:
    return int(lib().lo_max_threads())


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
        _setup_signatures(_lib)
    return _lib


def _setup_signatures(L):
    P = C.POINTER
    L.lo_csr_free.argtypes = [P(_Csr)]
    L.lo_set_threads.restype = None
    L.lo_set_threads.argtypes = [C.c_int]
    L.lo_max_threads.restype = C.c_int
    L.lo_max_threads.argtypes = []
    L.lo_part_begin.restype = C.c_int64
    L.lo_part_begin.argtypes = [C.c_int64, C.c_int64, C.c_int64]
    L.lo_harmonic_mean.restype = C.c_double
    L.lo_harmonic_mean.argtypes = [C.c_double, C.c_double]
    L.lo_stencil_init.argtypes = [P(_Stencil)]
    L.lo_stencil_spmv.argtypes = [P(_Stencil), C.c_void_p, C.c_void_p]
    L.lo_stencil_diagonal.argtypes = [P(_Stencil), C.c_void_p]
    L.lo_stencil_rhs.argtypes = [P(_Stencil), C.c_void_p]
    L.lo_stencil_to_csr.argtypes = [P(_Stencil), P(_Csr), C.c_void_p]
    L.lo_gen_27pt.argtypes = [C.c_void_p, C.c_void_p, P(_Csr)]
    L.lo_gen_7pt.argtypes = [C.c_void_p, C.c_void_p, P(_Csr)]
    L.lo_gen_convdiff.argtypes = [C.c_void_p, C.c_void_p, P(_Csr)]
    L.lo_material_diagonal_lines.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
    L.lo_material_flow_cylinder_gap.argtypes = [C.c_void_p, C.c_double, C.c_void_p]
    L.lo_axis_quotients.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.lo_csr_spmv.argtypes = [P(_Csr), C.c_void_p, C.c_void_p]
    L.lo_csr_residual.argtypes = [P(_Csr), C.c_void_p, C.c_void_p, C.c_void_p]
    L.lo_jacobi_sweep.argtypes = [P(_Csr), C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    L.lo_sor_sweep.argtypes = [P(_Csr), C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_int, C.c_int, C.c_int64]
    L.lo_sor_sweep_ordered.argtypes = [P(_Csr), C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_int, C.c_int, C.c_void_p]
    L.lo_colour_smallest_last.restype = C.c_int32
    L.lo_colour_smallest_last.argtypes = [P(_Csr), C.c_void_p]
    L.lo_colour_jp.restype = C.c_int32
    L.lo_colour_jp.argtypes = [P(_Csr), C.c_uint64, C.c_void_p]
    L.lo_colour_order.argtypes = [C.c_int64, C.c_void_p, C.c_int32, C.c_void_p]
    L.lo_cholesky_factor.restype = C.c_int
    L.lo_cholesky_factor.argtypes = [P(_Csr), C.c_void_p]
    L.lo_cholesky_solve.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    L.lo_effective_diffusion.restype = C.c_double
    L.lo_effective_diffusion.argtypes = [P(_Stencil), C.c_void_p, C.c_uint8, C.c_void_p,
                                         C.c_void_p, P(C.c_double)]
    L.lo_lu_factor.restype = C.c_int
    L.lo_lu_factor.argtypes = [P(_Csr), C.c_void_p]
    L.lo_lu_solve.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    L.lo_amg_default_params.argtypes = [P(_AmgParams)]
    L.lo_amg_partitions.restype = C.c_int64
    L.lo_amg_partitions.argtypes = [C.c_int64, C.c_int64, P(_AmgParams)]
    L.lo_amg_strength.argtypes = [P(_Csr), C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    L.lo_amg_aggregate.restype = C.c_int64
    L.lo_amg_aggregate.argtypes = [P(_Csr), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                   C.c_int32, C.c_int64, C.c_int, C.c_void_p,
                                   P(P(C.c_int64)), P(P(C.c_int32)), C.c_void_p]
    L.lo_amg_galerkin.argtypes = [P(_Csr), C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_int, P(_Csr)]
    L.lo_amg_setup.restype = C.c_int
    L.lo_amg_setup.argtypes = [P(_Csr), P(_AmgParams), P(_Amg)]
    L.lo_amg_free.argtypes = [P(_Amg)]
    L.lo_agg_map_check.restype = C.c_int
    L.lo_agg_map_check.argtypes = [P(_AggMap)]
    L.lo_amg_setup_coloured.restype = C.c_int
    L.lo_amg_setup_coloured.argtypes = [P(_Csr), P(_AmgParams), C.c_void_p, C.c_int32, P(_Amg)]
    L.lo_amg_setup_given.restype = C.c_int
    L.lo_amg_setup_given.argtypes = [P(_Csr), P(_AmgParams), P(_AggMap), C.c_int64, P(_Amg)]
    L.lo_amg_vcycle.argtypes = [P(_Amg), C.c_void_p, C.c_void_p]
    L.lo_pcg.restype = C.c_int64
    L.lo_pcg.argtypes = [P(_Csr), C.c_void_p, C.c_void_p, P(_Precon), C.c_double, C.c_int64,
                         C.c_int64, C.c_void_p]
    L.lo_pbicgstab.restype = C.c_int64
    L.lo_pbicgstab.argtypes = [P(_Csr), C.c_void_p, C.c_void_p, P(_Precon), C.c_double,
                               C.c_int64, C.c_int64, C.c_void_p]
    L.free = C.CDLL(None).free
    L.free.argtypes = [C.c_void_p]


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class Csr:
    """Host CSR with sorted columns and a stored diagonal (numpy arrays)."""

    rowptr: np.ndarray  # int64, n+1
    col: np.ndarray     # int32, nnz
    val: np.ndarray     # float64, nnz
    symmetric: bool = True
    is_f32: bool = False

    @property
    def n(self) -> int:
        return len(self.rowptr) - 1

    @property
    def nnz(self) -> int:
        return int(self.rowptr[-1])

    def _c(self) -> _Csr:
        self.rowptr = np.ascontiguousarray(self.rowptr, dtype=np.int64)
        self.col = np.ascontiguousarray(self.col, dtype=np.int32)
        self.val = np.ascontiguousarray(self.val, dtype=np.float64)
        c = _Csr()
        c.n = self.n
        c.ncols = self.n
        c.rowptr = self.rowptr.ctypes.data_as(C.POINTER(C.c_int64))
        c.col = self.col.ctypes.data_as(C.POINTER(C.c_int32))
        c.val = self.val.ctypes.data_as(C.POINTER(C.c_double))
        c.symmetric = int(self.symmetric)
        c.is_f32 = int(self.is_f32)
        return c

    def to_dense(self) -> np.ndarray:
        d = np.zeros((self.n, self.n))
        for i in range(self.n):
            for e in range(self.rowptr[i], self.rowptr[i + 1]):
                d[i, self.col[e]] = self.val[e]
        return d


def _take_csr(c: _Csr, L) -> Csr:
    n = c.n
    nnz = c.rowptr[n]
    out = Csr(
        np.ctypeslib.as_array(c.rowptr, shape=(n + 1,)).copy(),
        np.ctypeslib.as_array(c.col, shape=(max(nnz, 1),))[:nnz].copy(),
        np.ctypeslib.as_array(c.val, shape=(max(nnz, 1),))[:nnz].copy(),
        bool(c.symmetric),
        bool(c.is_f32),
    )
    L.lo_csr_free(C.byref(c))
    return out


# ---- geometry / generators ------------------------------------------------

def axis_quotients(dims, lengths) -> np.ndarray:
    d = np.asarray(dims, dtype=np.int64)
    le = np.asarray(lengths, dtype=np.float64)
    q = np.zeros(3)
    lib().lo_axis_quotients(_ptr(d), _ptr(le), _ptr(q))
    return q


def harmonic_mean(a: float, b: float) -> float:
    return lib().lo_harmonic_mean(a, b)


def material_diagonal_lines(dims, max_material_num: int = 4) -> np.ndarray:
    d = np.asarray(dims, dtype=np.int64)
    m = np.zeros(int(np.prod(d)), dtype=np.uint8)
    lib().lo_material_diagonal_lines(_ptr(d), max_material_num, _ptr(m))
    return m


def material_flow_cylinder_gap(dims, radius: float) -> np.ndarray:
    d = np.asarray(dims, dtype=np.int64)
    m = np.zeros(int(np.prod(d)), dtype=np.uint8)
    lib().lo_material_flow_cylinder_gap(_ptr(d), radius, _ptr(m))
    return m


class Stencil:
    """7-point diffusion stencil matrix (lookup valuator when ``k`` is None,
    value valuator otherwise; values valuator with ``k_axes``, one
    conductivity array per axis)."""

    def __init__(self, dims, q=(1.0, 1.0, 1.0), mat=None, coeffs=(0.0, 1.0, 2.0, 3.0), k=None,
                 sol_start=1.0, sol_end=0.0, zero_to_one=True, k_axes=None, henry=None,
                 gaseous_mask=0):
        self.dims = tuple(int(v) for v in dims)
        self.n = int(np.prod(self.dims))
        self._mat = None if mat is None else np.ascontiguousarray(mat, dtype=np.uint8)
        self._kax = None
        if k_axes is not None:
            self._kax = [np.ascontiguousarray(v, dtype=np.float64) for v in k_axes]
            k = self._kax[0]
        self._k = None if k is None else np.ascontiguousarray(k, dtype=np.float64)
        s = _Stencil()
        for i in range(3):
            s.dims[i] = self.dims[i]
            s.q[i] = float(q[i])
        for i in range(4):
            s.coeffs[i] = float(coeffs[i])
        s.k = self._k.ctypes.data_as(C.POINTER(C.c_double)) if self._k is not None else None
        s.mat = self._mat.ctypes.data_as(C.POINTER(C.c_uint8)) if self._mat is not None else None
        s.sol_start = sol_start
        s.sol_end = sol_end
        s.zero_to_one = int(zero_to_one)
        if self._kax is not None:
            s.k1 = self._kax[1].ctypes.data_as(C.POINTER(C.c_double))
            s.k2 = self._kax[2].ctypes.data_as(C.POINTER(C.c_double))
        if henry is not None:
            # HenryDiffusionLookupProvider with this Henry constant
            s.henry = 1
            s.henry_constant = float(henry)
            s.gaseous_mask = int(gaseous_mask)
        lib().lo_stencil_init(C.byref(s))
        self._s = s
        self.conn = np.array(s.conn[:])

    def spmv(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n)
        lib().lo_stencil_spmv(C.byref(self._s), _ptr(x), _ptr(y))
        return y

    def diagonal(self) -> np.ndarray:
        d = np.empty(self.n)
        lib().lo_stencil_diagonal(C.byref(self._s), _ptr(d))
        return d

    def rhs(self) -> np.ndarray:
        b = np.empty(self.n)
        lib().lo_stencil_rhs(C.byref(self._s), _ptr(b))
        return b

    def effective_diffusion(self, lengths, sol, compress_map=None, none_mask=0):
        """EffDiffCalc: (effective diffusivity, area part) of `sol`."""
        le = np.ascontiguousarray(lengths, dtype=np.float64)
        x = np.ascontiguousarray(sol, dtype=np.float64)
        cm = None if compress_map is None else np.ascontiguousarray(compress_map, np.int64)
        ap = C.c_double()
        eff = lib().lo_effective_diffusion(C.byref(self._s), _ptr(le), int(none_mask), _ptr(x),
                                           None if cm is None else _ptr(cm), C.byref(ap))
        return float(eff), float(ap.value)

    def to_csr(self):
        L = lib()
        c = _Csr()
        cmap = np.empty(self.n, dtype=np.int64)
        if L.lo_stencil_to_csr(C.byref(self._s), C.byref(c), _ptr(cmap)):
            raise MemoryError("stencil to CSR failed")
        return _take_csr(c, L), cmap


def gen_27pt(dims, k) -> Csr:
    L = lib()
    d = np.asarray(dims, dtype=np.int64)
    k = np.ascontiguousarray(k, dtype=np.float64)
    c = _Csr()
    if L.lo_gen_27pt(_ptr(d), _ptr(k), C.byref(c)):
        raise MemoryError("27-point generation failed")
    return _take_csr(c, L)


def gen_7pt(dims, k) -> Csr:
    L = lib()
    d = np.asarray(dims, dtype=np.int64)
    k = np.ascontiguousarray(k, dtype=np.float64)
    c = _Csr()
    if L.lo_gen_7pt(_ptr(d), _ptr(k), C.byref(c)):
        raise MemoryError("7-point generation failed")
    return _take_csr(c, L)


def gen_convdiff(dims, v) -> Csr:
    L = lib()
    d = np.asarray(dims, dtype=np.int64)
    vv = np.ascontiguousarray(v, dtype=np.float64)
    c = _Csr()
    if L.lo_gen_convdiff(_ptr(d), _ptr(vv), C.byref(c)):
        raise MemoryError("convection-diffusion generation failed")
    return _take_csr(c, L)


# ---- CSR kernels -----------------------------------------------------------

def spmv(a: Csr, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(a.n)
    c = a._c()
    lib().lo_csr_spmv(C.byref(c), _ptr(x), _ptr(y))
    return y


def residual(a: Csr, b: np.ndarray, x: np.ndarray) -> np.ndarray:
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    r = np.empty(a.n)
    c = a._c()
    lib().lo_csr_residual(C.byref(c), _ptr(b), _ptr(x), _ptr(r))
    return r


def jacobi_sweep(a: Csr, b, x_in=None, relax=1.0) -> np.ndarray:
    c = a._c()
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.empty(a.n)
    xi = None if x_in is None else np.ascontiguousarray(x_in, dtype=np.float64)
    lib().lo_jacobi_sweep(C.byref(c), relax, None if xi is None else _ptr(xi), _ptr(out), _ptr(b))
    return out


def sor_sweep(a: Csr, b, x_in=None, relax=1.0, forward=True, ultra=False, nparts=1,
              order=None) -> np.ndarray:
    c = a._c()
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.zeros(a.n)
    xi = None if x_in is None else np.ascontiguousarray(x_in, dtype=np.float64)
    xp = None if xi is None else _ptr(xi)
    if order is None:
        lib().lo_sor_sweep(C.byref(c), relax, xp, _ptr(out), _ptr(b), int(forward), int(ultra),
                           nparts)
    else:
        o = np.ascontiguousarray(order, dtype=np.int32)
        lib().lo_sor_sweep_ordered(C.byref(c), relax, xp, _ptr(out), _ptr(b), int(forward),
                                   int(ultra), _ptr(o))
    return out


def sor_sweep_f32(a: Csr, b, order, x_in=None, relax=1.0, forward=True,
                  ultra=False) -> np.ndarray:
    """Ordered SOR sweep in float arithmetic (the precision form's smoother)."""
    c = a._c()
    b = np.ascontiguousarray(b, dtype=np.float32)
    out = np.zeros(a.n, dtype=np.float32)
    xi = None if x_in is None else np.ascontiguousarray(x_in, dtype=np.float32)
    o = np.ascontiguousarray(order, dtype=np.int32)
    lib().lo_sor_sweep_ordered_f32(C.byref(c), C.c_float(relax), None if xi is None else _ptr(xi),
                                   _ptr(out), _ptr(b), int(forward), int(ultra), _ptr(o))
    return out


def colour_jp(a: Csr, seed: int):
    c = a._c()
    col = np.empty(a.n, dtype=np.int32)
    nc = lib().lo_colour_jp(C.byref(c), seed, _ptr(col))
    return col, int(nc)


def colour_smallest_last(a: Csr):
    c = a._c()
    col = np.empty(a.n, dtype=np.int32)
    nc = lib().lo_colour_smallest_last(C.byref(c), _ptr(col))
    return col, int(nc)


def colour_order(colour: np.ndarray, ncolours: int) -> np.ndarray:
    colour = np.ascontiguousarray(colour, dtype=np.int32)
    order = np.empty(len(colour), dtype=np.int32)
    lib().lo_colour_order(len(colour), _ptr(colour), ncolours, _ptr(order))
    return order


def cholesky_factor(a: Csr) -> np.ndarray:
    c = a._c()
    l = np.zeros((a.n, a.n))
    if lib().lo_cholesky_factor(C.byref(c), _ptr(l)):
        raise np.linalg.LinAlgError("matrix not positive definite")
    return l


def cholesky_solve(l: np.ndarray, b: np.ndarray) -> np.ndarray:
    l = np.ascontiguousarray(l, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty(len(b))
    lib().lo_cholesky_solve(len(b), _ptr(l), _ptr(b), _ptr(x))
    return x


def lu_factor(a: Csr) -> np.ndarray:
    """Dense L (unit diagonal, below) and U (on and above the diagonal) of
    the unpivoted LU (lu/decomposition.hpp)."""
    c = a._c()
    lu = np.zeros((a.n, a.n))
    if lib().lo_lu_factor(C.byref(c), _ptr(lu)):
        raise np.linalg.LinAlgError("zero pivot")
    return lu


def lu_solve(lu: np.ndarray, b: np.ndarray) -> np.ndarray:
    lu = np.ascontiguousarray(lu, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty(len(b))
    lib().lo_lu_solve(len(b), _ptr(lu), _ptr(b), _ptr(x))
    return x


# ---- AMG -------------------------------------------------------------------

def amg_params(**kw) -> _AmgParams:
    p = _AmgParams()
    lib().lo_amg_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def amg_partitions(n: int, level: int = 0, **kw) -> int:
    p = amg_params(**kw)
    return int(lib().lo_amg_partitions(n, level, C.byref(p)))


def amg_strength(a: Csr, theta: float = 1.0 / 3.0):
    c = a._c()
    dep = np.zeros(a.nnz, dtype=np.uint8)
    inf = np.zeros(a.nnz, dtype=np.uint8)
    iso = np.zeros(a.n, dtype=np.uint8)
    lib().lo_amg_strength(C.byref(c), theta, _ptr(dep), _ptr(inf), _ptr(iso))
    return dep, inf, iso


def amg_aggregate(a: Csr, dep, inf, iso, min_size=6, max_size=9, nparts=1, aggressive=False):
    L = lib()
    c = a._c()
    agg = np.empty(a.n, dtype=np.uint32)
    lp = C.POINTER(C.c_int64)()
    ls = C.POINTER(C.c_int32)()
    stats = np.zeros(5, dtype=np.int64)
    nc = L.lo_amg_aggregate(C.byref(c), _ptr(dep), _ptr(inf), _ptr(iso), min_size, max_size,
                            nparts, int(aggressive), _ptr(agg), C.byref(lp), C.byref(ls),
                            _ptr(stats))
    list_ptr = np.ctypeslib.as_array(lp, shape=(nc + 1,)).copy()
    total = int(list_ptr[-1])
    lst = np.ctypeslib.as_array(ls, shape=(max(total, 1),))[:total].copy()
    L.free(C.cast(lp, C.c_void_p))
    L.free(C.cast(ls, C.c_void_p))
    return int(nc), agg, list_ptr, lst, stats


def amg_galerkin(a: Csr, nc: int, agg, list_ptr, lst, coarse_f32=False) -> Csr:
    L = lib()
    c = a._c()
    out = _Csr()
    agg = np.ascontiguousarray(agg, dtype=np.uint32)
    list_ptr = np.ascontiguousarray(list_ptr, dtype=np.int64)
    lst = np.ascontiguousarray(lst, dtype=np.int32)
    if L.lo_amg_galerkin(C.byref(c), nc, _ptr(agg), _ptr(list_ptr), _ptr(lst), int(coarse_f32),
                         C.byref(out)):
        raise MemoryError("galerkin failed")
    return _take_csr(out, L)


def _agg_maps(maps):
    """(agg, list_ptr, list) triples -> C maps plus the arrays they point into"""
    keep, cm = [], (_AggMap * max(len(maps), 1))()
    for k, (agg, list_ptr, lst) in enumerate(maps):
        agg = np.ascontiguousarray(agg, dtype=np.uint32)
        list_ptr = np.ascontiguousarray(list_ptr, dtype=np.int64)
        lst = np.ascontiguousarray(lst, dtype=np.int32)
        if list_ptr.ndim != 1 or len(list_ptr) < 1:
            raise ValueError(f"aggregate map {k}: list_ptr needs ncoarse + 1 entries")
        keep += [agg, list_ptr, lst]
        cm[k] = _AggMap(len(agg), len(list_ptr) - 1, agg.ctypes.data, list_ptr.ctypes.data,
                        lst.ctypes.data)
    return cm, keep


def agg_map_check(agg, list_ptr, lst) -> bool:
    """lo_agg_map_check: the fine->coarse map and the coarse->fine lists agree"""
    cm, _keep = _agg_maps([(agg, list_ptr, lst)])
    return lib().lo_agg_map_check(C.byref(cm[0])) == 0


class Amg:
    """Oracle aggregation-AMG hierarchy + V-cycle (owns C memory).

    With ``maps`` (a sequence of (agg, list_ptr, list) per level) the
    aggregation of level k is replaced by maps[k], as lineal's FileAggregator
    does (aggregation/independent.hpp:279-298).  With ``finest_colours``
    (colour per row, ``ncolours`` classes) the colour-ordered smoother
    (smoother_parts=0) of level 0 follows that colouring instead of
    Jones-Plassmann."""

    def __init__(self, a: Csr, maps=None, finest_colours=None, ncolours=0, **params):
        self._a = a
        self._c = a._c()
        self._p = amg_params(**params)
        self._h = _Amg()
        if finest_colours is not None:
            if maps is not None:
                raise ValueError("finest_colours and maps do not combine")
            fc = np.ascontiguousarray(finest_colours, dtype=np.int32)
            if fc.shape != (a.n,):
                raise ValueError("finest_colours needs one colour per row")
            rc = lib().lo_amg_setup_coloured(C.byref(self._c), C.byref(self._p), _ptr(fc),
                                             int(ncolours), C.byref(self._h))
            if rc == LO_ERR_BAD_MAP:
                raise ValueError("finest colour outside [0, ncolours)")
        elif maps is None:
            rc = lib().lo_amg_setup(C.byref(self._c), C.byref(self._p), C.byref(self._h))
        else:
            cm, _keep = _agg_maps(maps)
            rc = lib().lo_amg_setup_given(C.byref(self._c), C.byref(self._p), cm, len(maps),
                                          C.byref(self._h))
        if rc != 0:
            lib().lo_amg_free(C.byref(self._h))
            self._h = None
            if rc == LO_ERR_NO_MAP:
                raise ValueError("no aggregate map for a level the hierarchy needs")
            if rc == LO_ERR_BAD_MAP:
                raise ValueError("aggregate map does not fit its level")
            raise np.linalg.LinAlgError("coarsest matrix not positive definite")

    @property
    def nlevels(self) -> int:
        return int(self._h.nlevels)

    def level_size(self, l: int) -> int:
        return int(self._h.lv[l].a.n)

    def level_csr(self, l: int) -> Csr:
        lv = self._h.lv[l].a
        n = lv.n
        nnz = lv.rowptr[n]
        return Csr(np.ctypeslib.as_array(lv.rowptr, shape=(n + 1,)).copy(),
                   np.ctypeslib.as_array(lv.col, shape=(max(nnz, 1),))[:nnz].copy(),
                   np.ctypeslib.as_array(lv.val, shape=(max(nnz, 1),))[:nnz].copy(),
                   bool(lv.symmetric), bool(lv.is_f32))

    def level_agg(self, l: int) -> np.ndarray:
        return np.ctypeslib.as_array(self._h.lv[l].agg, shape=(self.level_size(l),)).copy()

    def level_map(self, l: int):
        """(agg, list_ptr, list) of level l (fine -> coarse ids, coarse -> fine lists)"""
        if not 0 <= l < self.nlevels - 1:
            raise IndexError(f"level {l} has no aggregate map")
        lv = self._h.lv[l]
        nc = self.level_size(l + 1)
        list_ptr = np.ctypeslib.as_array(lv.list_ptr, shape=(nc + 1,)).copy()
        total = int(list_ptr[-1])
        lst = np.ctypeslib.as_array(lv.list, shape=(max(total, 1),))[:total].copy()
        return self.level_agg(l), list_ptr, lst

    def level_order(self, l: int):
        o = self._h.lv[l].order
        if not o:
            return None
        return np.ctypeslib.as_array(o, shape=(self.level_size(l),)).copy()

    def vcycle(self, b: np.ndarray) -> np.ndarray:
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self._a.n)
        lib().lo_amg_vcycle(C.byref(self._h), _ptr(b), _ptr(x))
        return x

    def close(self):
        if self._h is not None:
            lib().lo_amg_free(C.byref(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _solve(fn, a: Csr, b, x0=None, precon=PRECON_NONE, relax=1.0, ultra=False, nparts=1,
           amg: Amg | None = None, rtol=1e-8, maxit=1000, rere_period=8):
    c = a._c()
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(a.n) if x0 is None else np.array(x0, dtype=np.float64)
    m = _Precon()
    m.kind = precon
    m.relax = relax
    m.ultra = int(ultra)
    m.nparts = nparts
    m.amg = C.pointer(amg._h) if amg is not None else None
    hist = np.zeros(maxit + 1)
    it = fn(C.byref(c), _ptr(b), _ptr(x), C.byref(m), rtol, maxit, rere_period, _ptr(hist))
    return x, int(it), hist[: it + 1]


def pcg(a: Csr, b, **kw):
    return _solve(lib().lo_pcg, a, b, **kw)


def pbicgstab(a: Csr, b, **kw):
    return _solve(lib().lo_pbicgstab, a, b, **kw)
