"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and
exports every entry point that include/lineal_gb300.h declares.  No compute
calls are made (there is no GPU here)."""

import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lineal_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(lgx_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def library():
    from lineal_gb300 import build

    return build.build()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "lgx_spmv" in names and "lgx_pcg" in names and "lgx_amg_setup" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(library):
    out = subprocess.run(["nm", "-D", "--defined-only", library], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"


def test_library_loads_without_gpu(library):
    lib = ctypes.CDLL(library)
    lib.lgx_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.lgx_version()
    lib.lgx_status_string.restype = ctypes.c_char_p
    assert lib.lgx_status_string(0) == b"ok"


def test_invalid_arguments_are_statuses(library):
    import lineal_gb300 as g

    lib = g.lib()
    # null handles are rejected on the host before any device work
    assert lib.lgx_spmv(None, None, None, None) == 1
    assert lib.lgx_matrix_info(None, None, None, None, None) == 1
    assert lib.lgx_matrix_autotune(None, 5, None, None) == 1
    assert lib.lgx_amg_autotune(None, 5, None, 0, None, None) == 1
    assert lib.lgx_amg_level_lists(None, 0, None, None, None, None) == 1
    assert lib.lgx_direct_create(None, 0, None, None) == 1
    assert lib.lgx_amg_setup_log(None, None, 0, None, None) == 1
    assert lib.lgx_direct_solve(None, None, None, None) == 1
    assert lib.lgx_direct_destroy(None) == 0
    assert lib.lgx_lincomb(-1, 1.0, None, 1.0, None, None, None) == 1
    assert lib.lgx_lincomb(0, 1.0, None, 1.0, None, None, None) == 0
    assert lib.lgx_fill(5, 1.0, None, None) == 1
    assert lib.lgx_amg_autotune_reset(None) == 1
    assert b"null" in lib.lgx_last_error()


def test_concept_layer_compiles_and_links(library):
    """include/lineal_gb300/lineal.hpp compiles in a complete program (the
    one the GPU suite runs) and links against the library."""
    from lineal_gb300 import build

    for name in ("concepts_demo", "direct_demo", "vector_demo", "aggs_io_demo",
                 "aggs_solver_demo", "access_demo"):
        exe = build.build_cpp_demo(name=name)
        assert os.path.isfile(exe) and os.access(exe, os.X_OK)


def test_ctypes_structs_match_the_header(tmp_path):
    """Every ABI struct the Python front end mirrors with ctypes has the C
    header's size and field offsets (a compiled probe of the header)."""
    import ctypes

    import lineal_gb300 as g

    pairs = {"lgx_tune_entry": g._TuneEntry, "lgx_amg_level_log": g._AmgLevelLog,
             "lgx_amg_params": g._AmgParams, "lgx_solve_params": g._SolveParams,
             "lgx_agg_map": g._AggMap, "lgx_convdiff_system": g._ConvDiffSystem}
    lines = ["#include <cstddef>", "#include <cstdio>", '#include "lineal_gb300.h"',
             "int main() {"]
    for cname, py in pairs.items():
        lines.append(f'  std::printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'  std::printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.cpp"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "probe")
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    "-I", "/usr/local/cuda/include", str(src), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(line.split()[:2]): int(line.split()[2]) for line in out if line}
    for cname, py in pairs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)


def test_box_info_quotients_match_the_oracle():
    """BoxInfo's axis quotients (box-equidistant.hpp:67-79) computed by the
    library's host code equal the oracle's bit for bit; bad boxes are
    refused.  Host-only call: no GPU needed."""
    import numpy as np

    import lineal_gb300 as g
    import oracle as lo

    rng = np.random.default_rng(1)
    boxes = [((4, 9, 7), (4.0, 9.0, 7.0)), ((64, 64, 64), (64.0, 64.0, 64.0)),
             ((4, 8, 4), (4.0, 8.0, 4.0)), ((17, 13, 19), (1.3, 0.7, 2.1))]
    boxes += [(tuple(int(c) for c in rng.integers(1, 300, 3)),
               tuple(float(v) for v in rng.uniform(0.01, 50.0, 3))) for _ in range(50)]
    for cells, lengths in boxes:
        got = g.BoxInfo(cells, lengths).axis_quotients()
        np.testing.assert_array_equal(got, lo.axis_quotients(cells, lengths))
    for cells, lengths in (((0, 4, 4), (1.0, 1.0, 1.0)), ((4, 4, 4), (1.0, -1.0, 1.0)),
                           ((4, 4, 4), (1.0, float("inf"), 1.0))):
        with pytest.raises(g.LinealError):
            g.BoxInfo(cells, lengths).axis_quotients()
