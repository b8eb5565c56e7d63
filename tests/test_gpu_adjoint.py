"""Adjoint gradients of L = 0.5 ||x - x_t||^2 through A x = b (diffusion with
face conductivity k = exp(g), g a Gaussian random field):

* against dense torch autograd (torch.linalg.solve) on a 16^3 grid;
* against FP64 central finite differences on 32 random faces of the 96^3
  grid: dL/dk_f = (L(k_f + h) - L(k_f - h)) / (2h), where the loss
  difference is evaluated through the exact identity
  L+ - L- = (x+ - x-) . ((x+ + x-)/2 - x_t) with x+ - x- obtained from
  A(k+h) (x+ - x-) = -(A(k+h) - A(k-h)) x-, which keeps the difference
  accurate to the solver tolerance instead of losing it to cancellation.

Tolerance: 1e-6 relative (per gradient entry for FD, in norm for dense).
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _problem(n, seed=5):
    g = O.grid_grf(n, n, n, seed, 8.0)
    L, kf, kb = O.diffusion_from_cells(n, n, n, g)
    b = O.uniform(seed + 1, L.n)
    # smooth target: low-mode field from the same generators
    xt = 0.05 * np.cos(np.linspace(0, 6.0, L.n)) + 0.01 * O.grid_grf(n, n, n, seed + 2, 8.0)
    return L, kf, kb, b, xt


def _assemble(t, la, ua, kf, kb):
    """lower = upper = -k, diag = wall terms + sum of incident k (torch)."""
    import torch
    lower = -kf
    upper = -kf
    diag = kb.clone()
    diag = diag.index_add(0, la, kf).index_add(0, ua, kf)
    return diag, lower, upper


def test_adjoint_matches_dense_autograd_16():
    import torch

    from cufoam_gb300.autograd import LduPattern, ldu_solve
    n = 16
    L, kf, kb, b, xt = _problem(n)
    dev = "cuda"
    la = torch.from_numpy(L.lower_addr.astype(np.int64)).to(dev)
    ua = torch.from_numpy(L.upper_addr.astype(np.int64)).to(dev)
    kf_t = torch.tensor(kf, device=dev, requires_grad=True)
    b_t = torch.tensor(b, device=dev, requires_grad=True)
    xt_t = torch.tensor(xt, device=dev)
    kb_t = torch.tensor(kb, device=dev)
    pattern = LduPattern(L.n, L.lower_addr, L.upper_addr)

    diag, lower, upper = _assemble(torch, la, ua, kf_t, kb_t)
    x = ldu_solve(diag, lower, upper, b_t, pattern, {"tolerance": 1e-15, "maxIter": 20000})
    loss = 0.5 * ((x - xt_t) ** 2).sum()
    gk, gb = torch.autograd.grad(loss, (kf_t, b_t))

    kf_d = torch.tensor(kf, device=dev, requires_grad=True)
    b_d = torch.tensor(b, device=dev, requires_grad=True)
    diag_d, lower_d, upper_d = _assemble(torch, la, ua, kf_d, kb_t)
    A = torch.diag(diag_d)
    A = A.index_put((ua, la), lower_d, accumulate=True).index_put((la, ua), upper_d, accumulate=True)
    xd = torch.linalg.solve(A, b_d)
    loss_d = 0.5 * ((xd - xt_t) ** 2).sum()
    gk_d, gb_d = torch.autograd.grad(loss_d, (kf_d, b_d))
    assert torch.linalg.norm(x.detach() - xd.detach()) / torch.linalg.norm(xd) < 1e-10
    assert (torch.linalg.norm(gk - gk_d) / torch.linalg.norm(gk_d)).item() < 1e-6
    assert (torch.linalg.norm(gb - gb_d) / torch.linalg.norm(gb_d)).item() < 1e-6


def test_adjoint_matches_central_differences_96():
    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300.autograd import LduPattern, ldu_solve
    n = 96
    L, kf, kb, b, xt = _problem(n)
    dev = "cuda"
    la_np, ua_np = L.lower_addr, L.upper_addr
    la = torch.from_numpy(la_np.astype(np.int64)).to(dev)
    ua = torch.from_numpy(ua_np.astype(np.int64)).to(dev)
    kf_t = torch.tensor(kf, device=dev, requires_grad=True)
    kb_t = torch.tensor(kb, device=dev)
    b_t = torch.tensor(b, device=dev)
    xt_t = torch.tensor(xt, device=dev)
    pattern = LduPattern(L.n, la_np, ua_np)
    ctrl = {"tolerance": 1e-14, "maxIter": 100000}
    diag, lower, upper = _assemble(torch, la, ua, kf_t, kb_t)
    x = ldu_solve(diag, lower, upper, b_t, pattern, ctrl)
    loss = 0.5 * ((x - xt_t) ** 2).sum()
    (gk,) = torch.autograd.grad(loss, (kf_t,))
    gk = gk.cpu().numpy()

    faces = O.permutation(6, L.n_faces)[:32]
    ctx = pattern.ctx
    solver_ctrl = dict(ctrl)
    for f in faces:
        f = int(f)
        h = 1e-6 * abs(kf[f])
        o, u = int(la_np[f]), int(ua_np[f])

        def ldu_with(kval):
            d = L.diag.copy()
            lo = L.lower.copy()
            up = L.upper.copy()
            dk = kval - kf[f]
            d[o] += dk
            d[u] += dk
            lo[f] = -kval
            up[f] = -kval
            return d, lo, up

        dm, lom, upm = ldu_with(kf[f] - h)
        dp, lop, upp = ldu_with(kf[f] + h)
        Mm = cf.LduMatrix(L.n, dm, lom, upm, la_np, ua_np, context=ctx)
        xm = np.zeros(L.n)
        cf.cuFoamCG("x", Mm, solver_ctrl).solve(xm, b)
        # (A+ - A-) x- : only rows o and u, coefficient change 2h on the face
        rhs = np.zeros(L.n)
        rhs[o] = -(2 * h) * (xm[o] - xm[u])
        rhs[u] = -(2 * h) * (xm[u] - xm[o])
        Mp = cf.LduMatrix(L.n, dp, lop, upp, la_np, ua_np, context=ctx)
        dx = np.zeros(L.n)
        cf.cuFoamCG("dx", Mp, {"tolerance": 1e-13, "maxIter": 100000}).solve(dx, rhs)
        xp = xm + dx
        dL = float(dx @ (0.5 * (xp + xm) - xt))
        fd = dL / (2 * h)
        assert abs(gk[f] - fd) <= 1e-6 * max(abs(fd), 1e-8 * np.abs(gk).max()), (f, gk[f], fd)
        Mm.close()
        Mp.close()
