"""Generate the golden fixtures under tests/golden/ from the lineal reference.

Run once, in a container that has the reference checkout:

    python tests/golden/make_golden.py <path of the lineal checkout>

It executes the reference's own Python scripts (nothing is re-implemented
here) and stores their results as compressed numpy archives:

* sor_python_reference.npz -- test/python-reference/sor.py: the 4x8x4
  flow-cylinder-gap problem, its dense matrix (defs/diffusion_matrix.py),
  x_true = 1..128, b = A x_true, and all 129 lexicographic SOR iterates that
  the script prints (relax 1).
* cholesky_python_reference.npz -- test/python-reference/cholesky.py: the
  n=32 tridiagonal matrix, numpy's Cholesky factor and the two solves.
* UFZ_CT_02_LHS.smf / UFZ_CT_02_RHS.dvf -- the binary matrix/vector fixtures
  of test/data, copied byte for byte (the IO round-trip test needs the exact
  bytes).
"""

from __future__ import annotations

import json
import os
import runpy
import shutil
import subprocess
import sys

import numpy as np


def _run_quiet(pyref: str, script: str) -> dict:
    """Execute a reference script and return its globals, discarding stdout."""
    sys.path.insert(0, pyref)
    devnull = open(os.devnull, "w")
    old = sys.stdout
    sys.stdout = devnull
    try:
        return runpy.run_path(os.path.join(pyref, script), run_name="golden")
    finally:
        sys.stdout = old
        devnull.close()
        sys.path.pop(0)


def main(ref: str) -> None:
    out = os.path.dirname(os.path.abspath(__file__))
    pyref = os.path.join(ref, "test", "python-reference")

    # sor.py: run the script itself and parse the JSON lines it prints.
    proc = subprocess.run([sys.executable, "sor.py"], cwd=pyref, check=True,
                          capture_output=True, text=True)
    iterates = np.array([json.loads(line) for line in proc.stdout.splitlines() if line.strip()])
    g = _run_quiet(pyref, "sor.py")
    np.savez_compressed(
        os.path.join(out, "sor_python_reference.npz"),
        dims=np.array(g["info"].dims, dtype=np.int64),
        lengths=np.array(g["info"].lengths, dtype=np.float64),
        coeffs=np.array(g["info"].diff_coeffs, dtype=np.float64),
        radius=np.float64(g["radius"]),
        relax=np.float64(g["relax"]),
        materials=np.array(g["materials"], dtype=np.uint8),
        lhs=np.asarray(g["lhs"], dtype=np.float64),
        x_true=np.asarray(g["vec"], dtype=np.float64),
        rhs=np.asarray(g["rhs"], dtype=np.float64),
        iterates=iterates,
    )

    # cholesky.py: run it and keep its globals.
    c = _run_quiet(pyref, "cholesky.py")
    np.savez_compressed(
        os.path.join(out, "cholesky_python_reference.npz"),
        lhs=c["lhs"], chol=c["chol"], rhs=c["rhs"], aux=c["aux"], sol=c["sol"],
    )

    data = os.path.join(ref, "test", "data")
    for f in ("UFZ_CT_02_LHS.smf", "UFZ_CT_02_RHS.dvf"):
        shutil.copyfile(os.path.join(data, f), os.path.join(out, f))
    print("golden fixtures written to", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the lineal checkout>")
    main(sys.argv[1])
