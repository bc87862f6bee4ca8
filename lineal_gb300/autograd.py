"""Differentiable solves (the differentiation form), an optional thin torch
binding over the C ABI.

``diffusion7_solve(theta, b, dims)`` returns x = A(theta)^-1 b for the 7-point
operator of ``gen_7pt`` with per-cell conductivity k = exp(theta)
(harmonic-mean faces, Dirichlet rows on the axis-0 boundary), solved by
AMG-PCG on the GPU.  Its backward pass solves the adjoint system
A lambda = dL/dx with the same hierarchy (A is symmetric) and contracts
dL/dtheta = -lambda^T (dA/dtheta) x in one kernel (lgx_diffusion7_grad);
dL/db = lambda.  With ``mixed=True`` both solves run flexible CG over the
float V-cycle (FP64 outer iteration and residuals).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import (PRECON_AMG, Colouring, HierarchyWright, diffusion7_grad, gen_7pt, pcg,
               residual_compensated)


@dataclass
class SolveOptions:
    rtol: float = 1e-10
    maxit: int = 2000
    mixed: bool = False
    min_coarsen_size: int = 2000
    partition_size: int = 4096


def _red_black(dims):
    i, j, k = np.meshgrid(*[np.arange(d, dtype=np.int32) for d in dims], indexing="ij")
    return ((i + j + k) % 2).ravel().astype(np.int32)


def _function():
    import torch

    class Diffusion7Solve(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, b, dims, opts):
            k = torch.exp(theta.detach().to(torch.float64)).contiguous()
            a = gen_7pt(dims, k)
            col = Colouring.from_array(a, _red_black(dims), 2)
            h = HierarchyWright(cycle_f32=opts.mixed, min_coarsen_size=opts.min_coarsen_size,
                                partition_size=opts.partition_size).instantiate(
                                    a, finest_colouring=col)
            res = pcg(a, b.detach().to(torch.float64), precon=PRECON_AMG, amg=h,
                      rtol=opts.rtol, maxit=opts.maxit, flexible=opts.mixed)
            ctx.save_for_backward(k, res.x)
            ctx.state = (a, h, dims, opts)
            ctx.iterations = res.iterations
            return res.x

        @staticmethod
        def backward(ctx, gx):
            k, x = ctx.saved_tensors
            a, h, dims, opts = ctx.state
            lam = pcg(a, gx.contiguous().to(torch.float64), precon=PRECON_AMG, amg=h,
                      rtol=opts.rtol, maxit=opts.maxit, flexible=opts.mixed).x
            gtheta = diffusion7_grad(dims, k, lam, x) if ctx.needs_input_grad[0] else None
            gb = lam if ctx.needs_input_grad[1] else None
            return gtheta, gb, None, None

    return Diffusion7Solve


def diffusion7_forward(theta, b, dims, opts: SolveOptions | None = None, x0=None):
    """x = A(theta)^-1 b without the autograd graph, optionally from the
    initial guess x0 (the tolerance is relative to the initial residual)."""
    import torch

    opts = opts or SolveOptions()
    dims = tuple(int(d) for d in dims)
    k = torch.exp(theta.detach().to(torch.float64)).contiguous()
    a = gen_7pt(dims, k)
    col = Colouring.from_array(a, _red_black(dims), 2)
    h = HierarchyWright(cycle_f32=opts.mixed, min_coarsen_size=opts.min_coarsen_size,
                        partition_size=opts.partition_size).instantiate(a, finest_colouring=col)
    return pcg(a, b.detach().to(torch.float64), x0=x0, precon=PRECON_AMG, amg=h, rtol=opts.rtol,
               maxit=opts.maxit, flexible=opts.mixed).x


def refined_solve(a, b, x0, hierarchy, steps=6, rtol=1e-10):
    """Iterative refinement to full FP64 accuracy: residuals with compensated
    row sums (residual_compensated), corrections by AMG-PCG.  Returns x."""
    import torch

    x = x0.clone()
    bn = float(torch.linalg.norm(b))
    for _ in range(steps):
        r = residual_compensated(a, b, x)
        rn = float(torch.linalg.norm(r))
        if rn <= 1e-17 * bn:
            break
        d = pcg(a, r, precon=PRECON_AMG, amg=hierarchy, rtol=rtol, maxit=2000).x
        x = x + d
        if float(torch.linalg.norm(d)) <= 1e-16 * float(torch.linalg.norm(x)):
            break
    return x


def _operator(theta, dims):
    import torch

    k = torch.exp(theta.detach().to(torch.float64)).contiguous()
    a = gen_7pt(dims, k)
    col = Colouring.from_array(a, _red_black(dims), 2)
    return a, col


def accurate_forward(theta, b, dims, opts: SolveOptions | None = None, x0=None):
    """x = A(theta)^-1 b to full FP64 accuracy (refined solve)."""
    import torch

    opts = opts or SolveOptions()
    dims = tuple(int(d) for d in dims)
    a, col = _operator(theta, dims)
    h = HierarchyWright(min_coarsen_size=opts.min_coarsen_size,
                        partition_size=opts.partition_size).instantiate(a, finest_colouring=col)
    b = b.detach().to(torch.float64)
    if x0 is None:
        x0 = pcg(a, b, precon=PRECON_AMG, amg=h, rtol=opts.rtol, maxit=opts.maxit).x
    return refined_solve(a, b, x0, h)


def accurate_gradient(theta, b, dims, x_target, opts: SolveOptions | None = None):
    """dL/dtheta of L = 0.5 ||x - x_target||^2 with x and the adjoint lambda
    refined to full FP64 accuracy (the reference gradient of checks)."""
    import torch

    opts = opts or SolveOptions()
    dims = tuple(int(d) for d in dims)
    a, col = _operator(theta, dims)
    h = HierarchyWright(min_coarsen_size=opts.min_coarsen_size,
                        partition_size=opts.partition_size).instantiate(a, finest_colouring=col)
    b = b.detach().to(torch.float64)
    x = refined_solve(a, b, pcg(a, b, precon=PRECON_AMG, amg=h, rtol=opts.rtol,
                                maxit=opts.maxit).x, h)
    g = (x - x_target).contiguous()
    lam = refined_solve(a, g, pcg(a, g, precon=PRECON_AMG, amg=h, rtol=opts.rtol,
                                  maxit=opts.maxit).x, h)
    k = torch.exp(theta.detach().to(torch.float64)).contiguous()
    return diffusion7_grad(dims, k, lam, x)


def accurate_system(theta, b, dims, opts: SolveOptions | None = None):
    """(A, hierarchy, x) at theta with x = A^-1 b to full FP64 accuracy."""
    import torch

    opts = opts or SolveOptions()
    dims = tuple(int(d) for d in dims)
    a, col = _operator(theta, dims)
    h = HierarchyWright(min_coarsen_size=opts.min_coarsen_size,
                        partition_size=opts.partition_size).instantiate(a, finest_colouring=col)
    b = b.detach().to(torch.float64)
    x = refined_solve(a, b, pcg(a, b, precon=PRECON_AMG, amg=h, rtol=opts.rtol,
                                maxit=opts.maxit).x, h)
    return a, h, x


def diffusion7_delta_apply(theta, dtheta, x, dims):
    """(A(theta + dtheta) - A(theta)) x for the operator of gen_7pt with
    k = exp(theta), without forming either matrix.  A face coefficient is
    c = 2 / (e^-theta_i + e^-theta_j); its change is
    -2 du / (u (u + du)) with u = e^-theta_i + e^-theta_j and
    du = e^-theta_i expm1(-dtheta_i) + e^-theta_j expm1(-dtheta_j), and an
    axis-0 boundary face changes the diagonal by 2 e^theta expm1(dtheta).
    Every term is formed from expm1, so the O(|dtheta|) result keeps full
    FP64 relative accuracy (differencing the two assembled matrices would
    leave rounding errors of relative size eps / |dtheta|)."""
    import torch

    n0, n1, n2 = (int(d) for d in dims)
    th = theta.detach().to(torch.float64).reshape(n0, n1, n2)
    dt = dtheta.detach().to(torch.float64).reshape(n0, n1, n2)
    xx = x.detach().to(torch.float64).reshape(n0, n1, n2)
    em = torch.exp(-th)
    dm = em * torch.expm1(-dt)
    y = torch.zeros_like(xx)
    for ax in range(3):
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, -1)
        hi[ax] = slice(1, None)
        lo, hi = tuple(lo), tuple(hi)
        u = em[lo] + em[hi]
        du = dm[lo] + dm[hi]
        dc = -2.0 * du / (u * (u + du))
        f = dc * (xx[lo] - xx[hi])
        y[lo] += f
        y[hi] -= f
    dk = 2.0 * torch.exp(th) * torch.expm1(dt)
    y[0] += dk[0] * xx[0]
    y[-1] += dk[-1] * xx[-1]
    return y.reshape(-1)


def perturbed_correction(theta, dtheta, dims, x, a0, h0, steps=4, rtol=1e-10):
    """d = A(theta + dtheta)^-1 b - x for x = A(theta)^-1 b, solved from
    A(theta + dtheta) d = -(A(theta + dtheta) - A(theta)) x: a small
    right-hand side formed accurately (diffusion7_delta_apply), then defect
    correction with compensated residuals of A(theta + dtheta) and AMG-PCG
    solves with A(theta) (matrix a0, hierarchy h0) as the approximate inverse.
    d carries full FP64 relative accuracy although it is O(|dtheta|)."""
    import torch

    dims = tuple(int(d) for d in dims)
    a1, _ = _operator(theta + dtheta, dims)
    rhs = -diffusion7_delta_apply(theta, dtheta, x, dims)
    d = torch.zeros_like(rhs)
    rn0 = float(torch.linalg.norm(rhs))
    for _ in range(steps):
        r = residual_compensated(a1, rhs, d)
        if float(torch.linalg.norm(r)) <= 1e-17 * rn0:
            break
        d = d + pcg(a0, r, precon=PRECON_AMG, amg=h0, rtol=rtol, maxit=2000).x
    return d


def loss_difference_fd(theta, v, h, dims, x, x_target, a0, h0):
    """Central difference of L = 0.5 ||x - x_target||^2 along v,
    (L(theta + h v) - L(theta - h v)) / (2 h), with x(theta +- h v) =
    x + d+- from perturbed_correction (x, a0, h0: the accurate solution,
    matrix and hierarchy at theta).  The loss difference is formed as
    (d+ - d-).(x - x_target) + 0.5 (d+.d+ - d-.d-), so neither the rounding
    of the two large losses nor that of the assembled perturbed matrices
    (relative eps / h in A(theta +- h v) - A(theta)) swamps the O(h)
    difference: what remains is the O(h^2) truncation and FP64 rounding
    relative to the difference itself."""
    import torch

    dp = perturbed_correction(theta, h * v, dims, x, a0, h0)
    dm = perturbed_correction(theta, -h * v, dims, x, a0, h0)
    num = torch.dot(dp - dm, x - x_target) + 0.5 * (torch.dot(dp, dp) - torch.dot(dm, dm))
    return float(num) / (2.0 * h)


_FN = None


def diffusion7_solve(theta, b, dims, opts: SolveOptions | None = None):
    """x = A(theta)^-1 b, differentiable in theta and b."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(theta, b, tuple(int(d) for d in dims), opts or SolveOptions())
