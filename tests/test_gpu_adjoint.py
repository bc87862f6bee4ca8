"""Differentiation form: the adjoint gradient of x = A(theta)^-1 b for the
7-point diffusion operator with k = exp(theta), through the torch binding,
against FP64 central finite differences along random directions and against
the gradient formed from the oracle's CPU solves."""

import numpy as np
import pytest

import oracle as lo

pytestmark = pytest.mark.gpu


def _bump(dims):
    i, j, k = np.meshgrid(*[np.arange(d, dtype=np.float64) for d in dims], indexing="ij")
    c = [(d - 1) / 2 for d in dims]
    s = max(dims) / 6.0
    return np.exp(-((i - c[0]) ** 2 + (j - c[1]) ** 2 + (k - c[2]) ** 2) / (2 * s * s)).ravel()


def _grad_reference(dims, k, lam, x):
    """dL/dtheta from the face formula, in numpy."""
    n0, n1, n2 = dims
    K, L, X = (v.reshape(dims) for v in (k, lam, x))
    g = np.zeros(dims)
    for axis in range(3):
        sl_a = [slice(None)] * 3
        sl_b = [slice(None)] * 3
        sl_a[axis] = slice(0, dims[axis] - 1)
        sl_b[axis] = slice(1, dims[axis])
        ka, kb = K[tuple(sl_a)], K[tuple(sl_b)]
        t = (L[tuple(sl_a)] - L[tuple(sl_b)]) * (X[tuple(sl_a)] - X[tuple(sl_b)])
        s = ka + kb
        g[tuple(sl_a)] += 2 * ka * kb * kb / (s * s) * t
        g[tuple(sl_b)] += 2 * kb * ka * ka / (s * s) * t
    nb = np.zeros(dims)
    nb[0] += 1
    nb[n0 - 1] += 1
    g += nb * 2 * K * L * X
    return -g.ravel()


def test_sampled_outer(cuda):
    ref = lo.gen_27pt((7, 8, 9), np.exp(np.random.default_rng(0).standard_normal(504)))
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    rng = np.random.default_rng(1)
    u, v = rng.standard_normal(ref.n), rng.standard_normal(ref.n)
    got = cuda.sampled_outer(m, u, v, alpha=-1.0).cpu().numpy()
    rows = np.repeat(np.arange(ref.n), np.diff(ref.rowptr))
    np.testing.assert_array_equal(got, (-1.0 * u[rows]) * v[ref.col])


def _problem(dims, seed=4):
    n = int(np.prod(dims))
    rng = np.random.default_rng(seed)
    theta = rng.standard_normal(n)
    theta_t = theta + 0.3 * rng.standard_normal(n)
    return theta, theta_t, _bump(dims)


def _fd_check(cuda, dims, mixed, directions, seed=4, partition_size=500):
    """Largest relative gap between the adjoint gradient along random unit
    directions and FP64 central differences (h = 1e-6) of the loss."""
    import torch

    from lineal_gb300.autograd import (SolveOptions, accurate_system, diffusion7_solve,
                                       loss_difference_fd)

    theta0, theta_t, b0 = _problem(dims, seed)
    opts = SolveOptions(rtol=1e-11, mixed=mixed, min_coarsen_size=100,
                        partition_size=partition_size)
    fd_opts = SolveOptions(rtol=1e-10, min_coarsen_size=100, partition_size=partition_size)
    b = torch.as_tensor(b0, device="cuda")
    _, _, x_t = accurate_system(torch.as_tensor(theta_t, device="cuda"), b, dims, fd_opts)

    theta = torch.as_tensor(theta0, device="cuda").requires_grad_(True)
    x = diffusion7_solve(theta, b, dims, opts)
    (0.5 * torch.sum((x - x_t) ** 2)).backward()
    g = theta.grad.detach()
    rng = np.random.default_rng(5)
    h = 1e-6
    th0 = theta.detach()
    a0, h0, x0 = accurate_system(th0, b, dims, fd_opts)
    errs = []
    for _ in range(directions):
        v = rng.standard_normal(theta0.size)
        vt = torch.as_tensor(v / np.linalg.norm(v), device="cuda")
        fd = loss_difference_fd(th0, vt, h, dims, x0, x_t, a0, h0)
        gv = float(torch.dot(g, vt))
        errs.append(abs(fd - gv) / abs(gv))
    return max(errs)


@pytest.mark.parametrize("mixed", [False, True])
def test_adjoint_gradient_matches_finite_differences(cuda, mixed):
    assert _fd_check(cuda, (12, 13, 11), mixed, 8) <= 1e-6


def test_adjoint_gradient_matches_finite_differences_128(cuda):
    """The differentiation workload's own size: 128^3, theta ~ N(0, 1), 64
    random directions, h = 1e-6, mixed-precision forward and adjoint."""
    assert _fd_check(cuda, (128, 128, 128), True, 64, partition_size=4096) <= 1e-6


def test_delta_apply_equals_matrix_difference(cuda):
    """(A(theta + d) - A(theta)) x without forming the matrices equals the
    difference of the assembled products where that difference is accurate
    (a large step), and scales linearly for small steps."""
    import torch

    from lineal_gb300.autograd import diffusion7_delta_apply

    dims = (9, 10, 11)
    n = int(np.prod(dims))
    rng = np.random.default_rng(8)
    theta = rng.standard_normal(n)
    d = 1e-2 * rng.standard_normal(n)
    x = rng.uniform(-1, 1, n)
    want = (lo.spmv(lo.gen_7pt(dims, np.exp(theta + d)), x)
            - lo.spmv(lo.gen_7pt(dims, np.exp(theta)), x))
    t = lambda v: torch.as_tensor(v, device="cuda")  # noqa: E731
    got = diffusion7_delta_apply(t(theta), t(d), t(x), dims).cpu().numpy()
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    small = diffusion7_delta_apply(t(theta), t(1e-9 * d), t(x), dims).cpu().numpy()
    np.testing.assert_allclose(small * 1e9, got, rtol=5e-2, atol=1e-2 * np.abs(got).max())


def test_adjoint_gradient_matches_oracle_solves(cuda):
    import torch

    from lineal_gb300.autograd import SolveOptions, diffusion7_solve

    dims = (10, 9, 8)
    theta0, theta_t, b0 = _problem(dims, seed=7)
    opts = SolveOptions(rtol=1e-12, min_coarsen_size=100, partition_size=500)
    b = torch.as_tensor(b0, device="cuda")
    # oracle: x, x_t and lambda from CPU AMG-PCG solves, gradient by the face formula
    k, kt = np.exp(theta0), np.exp(theta_t)
    A, At = lo.gen_7pt(dims, k), lo.gen_7pt(dims, kt)
    kw = dict(precon=lo.PRECON_AMG, rtol=1e-12, maxit=500)
    x, _, _ = lo.pcg(A, b0, amg=lo.Amg(A, min_coarsen_size=100), **kw)
    xt, _, _ = lo.pcg(At, b0, amg=lo.Amg(At, min_coarsen_size=100), **kw)
    lam, _, _ = lo.pcg(A, x - xt, amg=lo.Amg(A, min_coarsen_size=100), **kw)
    want = _grad_reference(dims, k, lam, x)
    x_t = diffusion7_solve(torch.as_tensor(theta_t, device="cuda"), b, dims, opts).detach()
    theta = torch.as_tensor(theta0, device="cuda").requires_grad_(True)
    xg = diffusion7_solve(theta, b, dims, opts)
    (0.5 * torch.sum((xg - x_t) ** 2)).backward()
    got = theta.grad.cpu().numpy()
    assert np.linalg.norm(got - want) <= 1e-8 * np.linalg.norm(want)
    # the fused kernel equals the formula on the same inputs
    lam_d = torch.as_tensor(lam, device="cuda")
    direct = cuda.diffusion7_grad(dims, torch.as_tensor(k, device="cuda"), lam_d,
                                  torch.as_tensor(x, device="cuda")).cpu().numpy()
    np.testing.assert_allclose(direct, want, rtol=1e-12, atol=1e-14 * np.abs(want).max())


def test_compensated_residual_is_accurate(cuda):
    """Rows with heavy cancellation: the compensated residual equals the
    exactly rounded residual (rational arithmetic) to within 2 ulp."""
    from fractions import Fraction

    ref = lo.gen_27pt((5, 6, 7), np.exp(np.random.default_rng(3).standard_normal(210)))
    m = cuda.CsrMatrix.from_host(ref.rowptr, ref.col, ref.val)
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, ref.n)
    b = lo.spmv(ref, x) * (1 + 1e-12 * rng.standard_normal(ref.n))
    got = cuda.residual_compensated(m, b, x).cpu().numpy()
    for i in range(ref.n):
        exact = Fraction(b[i])
        for e in range(ref.rowptr[i], ref.rowptr[i + 1]):
            exact -= Fraction(ref.val[e]) * Fraction(x[ref.col[e]])
        want = float(exact)
        assert abs(got[i] - want) <= 2 * np.spacing(abs(want)), (i, got[i], want)
