"""lgx_dot_static, the allocation-free dot product, through the C ABI.

Collected last so that it also runs after every other GPU test in the same
process; it passes alone in a fresh process as well.  Each size is computed
twice in a row by lgx_dot_static and compared with lgx_dot on the same
inputs (same grid and summation order, so the tolerance below is only a
safety margin)."""

import ctypes

import pytest

RTOL = 1e-14
MAX_N = 1024 * 256 * 8  # partial sums held by the static scratch x elements per partial


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.gpu
@pytest.mark.parametrize("n", [0, 1, 17, 1_000_003, MAX_N])
def test_dot_static_matches_dot(cuda, n):
    import torch

    lib = cuda.lib()
    gen = torch.Generator(device="cuda").manual_seed(1234 + n)
    a = torch.rand(n, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
    b = torch.rand(n, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
    ref = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.lgx_dot(n, _ptr(a), _ptr(b), _ptr(ref), stream) == 0
    for _ in range(2):  # two calls in a row reuse the same static scratch
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        assert lib.lgx_dot_static(n, _ptr(a), _ptr(b), _ptr(out), stream) == 0, \
            lib.lgx_last_error()
        torch.cuda.synchronize()
        r, o = float(ref.item()), float(out.item())
        assert abs(o - r) <= RTOL * max(abs(r), 1e-300), (n, o, r)
    if n:
        prod = a.cpu() * b.cpu()
        exact, scale = float(prod.sum()), float(prod.abs().sum())
        assert abs(float(ref.item()) - exact) <= 1e-13 * scale


@pytest.mark.gpu
def test_dot_static_rejects_sizes_beyond_maximum(cuda):
    import torch

    lib = cuda.lib()
    a = torch.zeros(MAX_N + 1, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    status = lib.lgx_dot_static(MAX_N + 1, _ptr(a), _ptr(a), _ptr(out), stream)
    assert status == 1  # LGX_ERR_INVALID, decided on the host before any launch
    assert b"exceeds the maximum" in lib.lgx_last_error()
