"""The C++ concept layer (include/lineal_gb300/lineal.hpp) drives the library
like lineal's own test helpers drive lineal: a compiled program instantiates
ConjugateGradientsSolver<MultiGridSolver> and runs run_iterative_solver; a
second one uses the host element access (vector elements, CSR rows)."""

import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_concepts_demo_runs(cuda):
    from lineal_gb300 import build

    exe = build.build_cpp_demo()
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "concepts_demo ok" in out.stdout


def test_access_demo_runs(cuda):
    from lineal_gb300 import build

    exe = build.build_cpp_demo(name="access_demo")
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "access_demo ok" in out.stdout
