"""lgx_lincomb / lgx_fill (lineal's add, subtract, scale and constant
expressions, component-wise/vector-expression.hpp:67-91, 140-167) bit for
bit against numpy, which rounds every product and sum on its own as lineal
does, and the C++ layer's free operations (tests/cpp/vector_demo.cpp)."""

import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 257, 1_000_003])
def test_lincomb_bits(cuda, n):
    rng = np.random.default_rng(n)
    x, y = rng.uniform(-3, 3, n), rng.uniform(-3, 3, n)
    for alpha, beta in ((1.0, 1.0), (1.0, -1.0), (0.7071067811865476, -1.25e-3), (-2.0, 3.5)):
        got = cuda.lincomb(alpha, x, beta, y).cpu().numpy()
        np.testing.assert_array_equal(got, alpha * x + beta * y)
    np.testing.assert_array_equal(cuda.lincomb(1.0 / 3.0, x).cpu().numpy(), (1.0 / 3.0) * x)
    # in place: out = out + x
    out = cuda._dvec(y)
    cuda.lincomb(1.0, out, 1.0, x, out=out)
    np.testing.assert_array_equal(out.cpu().numpy(), y + x)
    np.testing.assert_array_equal(cuda.fill(n, -2.5).cpu().numpy(), np.full(n, -2.5))


def test_cpp_vector_operations(cuda):
    from lineal_gb300 import build

    exe = build.build_cpp_demo(name="vector_demo")
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "vector_demo ok" in out.stdout
