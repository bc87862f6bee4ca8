"""Builds the lineal_gb300 CUDA library for sm_103a (GB300).

Each translation unit under ``csrc/`` is compiled by nvcc in parallel and
linked into ``lineal_gb300/_lib/liblineal_gb300.so``; the C++ concept layer
test program (``tests/cpp/concepts_demo.cpp``) is linked against it when
requested.  No cmake, no torch extension machinery: plain nvcc command lines.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liblineal_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE,
                     "--expt-relaxed-constexpr"]


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(INCLUDE, "lineal_gb300.h"))
    srcs = sources()
    objs = [os.path.join(OBJ_DIR, os.path.basename(s)[:-3] + ".o") for s in srcs]
    cc = nvcc()

    def compile_one(pair):
        src, obj = pair
        if not force and not _stale(obj, [src] + headers):
            return None
        cmd = [cc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return f"{src}:\n{r.stdout}\n{r.stderr}"
        return None

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        errors = [e for e in ex.map(compile_one, zip(srcs, objs)) if e]
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if force or _stale(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


def build_cpp_demo(verbose: bool = False, name: str = "concepts_demo") -> str:
    """Compiles a C++ concept-layer program of tests/cpp (concepts_demo,
    direct_demo, vector_demo, aggs_io_demo, aggs_solver_demo, access_demo)
    that drives the library through include/lineal_gb300/lineal.hpp."""
    lib = build(verbose=verbose)
    src = os.path.join(ROOT, "tests", "cpp", name + ".cpp")
    out = os.path.join(OUT_DIR, name)
    if _stale(out, [src, lib, os.path.join(INCLUDE, "lineal_gb300", "lineal.hpp"),
                    os.path.join(INCLUDE, "lineal_gb300.h")]):
        cmd = [nvcc(), "-std=c++20", "-O2", "-I" + INCLUDE, src, "-o", out, "-L" + OUT_DIR,
               "-llineal_gb300", "-Xlinker", "-rpath=" + OUT_DIR]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
