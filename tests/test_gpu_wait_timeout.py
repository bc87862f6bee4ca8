"""Failure detection without a GPU fault: a kernel's bounded wait on a
barrier that nothing completes gives up after about a second, the library
reports the time-out as a status, and the context stays usable."""

import time

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_reports(cuda):
    t0 = time.perf_counter()
    st = cuda.lib().lgx_wait_selftest(cuda._stream())
    elapsed = time.perf_counter() - t0
    assert st == 2  # LGX_ERR_CUDA
    assert "timed out" in cuda.lib().lgx_last_error().decode()
    assert 0.2 < elapsed < 30.0
    # the flag was cleared and the context still computes correctly
    ref = lo.gen_27pt((9, 10, 11), np.exp(np.random.default_rng(0).standard_normal(990)))
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    x = np.random.default_rng(1).uniform(-1, 1, ref.n)
    np.testing.assert_array_equal(cuda.spmv(m, x).cpu().numpy(), lo.spmv(ref, x))
    res = cuda.pcg(m, lo.spmv(ref, x), precon=cuda.PRECON_JACOBI, rtol=1e-10, maxit=500)
    assert res.rel_residual <= 1e-10
