"""Adjoint of the FP64 path (lp_*_vjp, lp_field_energy_gradient): every
vector-Jacobian product against central finite differences of the forward
GPU map, the checkpointed gradient of the field energy through 50 steps
(Nx = 32, N = Nv = 16, A = 0.05, k = 0.5, nu = 0.02, dt = 0.01, checkpoint
every 10 steps) against central differences in A, nu and 8 seeded
directions of the initial state, and the same gradient composed step by step
through torch.autograd.Function wrappers of the C ABI (test harness only)."""
from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _params(lp, **kw):
    base = dict(nx1=4, nx2=1, nv=8, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.2, k_wave=0.5)
    base.update(kw)
    return lp.Params(**base, fixes=lp.FIX_DEFAULT, precision=lp.PREC_FP64)


def _ctx(lp, **kw):
    c = lp.Context(_params(lp, **kw))
    c.set_init(1)
    return c


def _dev(x):
    t = torch.tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    return t


def _fd(ctx, op, U, w, d, eps=1e-6):
    """<w, (F(U + eps d) - F(U - eps d)) / (2 eps)> for the forward map op."""
    ctx.set_state(U + eps * d)
    op()
    fp = ctx.get_state()
    ctx.set_state(U - eps * d)
    op()
    fm = ctx.get_state()
    return float(np.dot(w, (fp - fm) / (2 * eps)))


def _vjp(ctx, fn, U, w):
    ctx.set_state(U)
    lo, li = _dev(w), _dev(np.zeros_like(w))
    extra = fn(lo.data_ptr(), li.data_ptr())
    torch.cuda.synchronize()
    return li.cpu().numpy(), extra


@pytest.mark.parametrize("which", ["collision", "advection", "step"])
def test_vjp_matches_finite_differences(gpu_lib, which):
    ctx = _ctx(gpu_lib)
    U = ctx.get_state()
    rng = np.random.default_rng(7)
    w = rng.standard_normal(U.size)
    d = rng.standard_normal(U.size) * (np.abs(U) + 1e-3 * np.abs(U).max())
    op = {"collision": lambda: ctx.collision_step(), "advection": lambda: ctx.advect_step(),
          "step": lambda: ctx.step(1)}[which]
    fn = {"collision": ctx.collision_vjp, "advection": ctx.advect_vjp, "step": ctx.step_vjp}[which]
    lam, _ = _vjp(ctx, fn, U, w)
    adj = float(np.dot(d, lam))
    fd = _fd(ctx, op, U, w, d)
    assert abs(adj - fd) <= 1e-6 * abs(fd), (which, adj, fd)


def test_collision_vjp_nu(gpu_lib):
    lp = gpu_lib
    ctx = _ctx(lp)
    U = ctx.get_state()
    w = np.random.default_rng(3).standard_normal(U.size)
    _, dnu = _vjp(ctx, ctx.collision_vjp, U, w)
    h = 1e-6
    vals = []
    for nu in (0.05 + h, 0.05 - h):
        c = _ctx(lp, nu=nu)
        c.set_state(U)
        c.collision_step()
        vals.append(float(np.dot(w, c.get_state())))
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(dnu - fd) <= 1e-6 * abs(fd), (dnu, fd)


def test_field_energy_gradient_matches_fd(gpu_lib):
    ctx = _ctx(gpu_lib)
    U = ctx.get_state()
    lam = _dev(np.zeros_like(U))
    J = ctx.field_energy(lam.data_ptr())
    torch.cuda.synchronize()
    d = np.random.default_rng(5).standard_normal(U.size) * np.abs(U)
    eps = 1e-6
    ctx.set_state(U + eps * d)
    jp = ctx.field_energy()
    ctx.set_state(U - eps * d)
    jm = ctx.field_energy()
    fd = (jp - jm) / (2 * eps)
    assert J > 0
    assert abs(float(np.dot(d, lam.cpu().numpy())) - fd) <= 1e-7 * abs(fd)


# ---- the gradient workload: d(field energy at T = 0.5)/d(A, nu, f0) ----
CFG4 = dict(nx1=32, nx2=1, nv=16, n=16, lv=5.25, lx=4 * np.pi, nu=0.02, dt=0.01, a_amp=0.05, k_wave=0.5)
NSTEPS, CHECK = 50, 10


def _J_after(lp, U0=None, **kw):
    c = lp.Context(lp.Params(**dict(CFG4, **kw), fixes=lp.FIX_DEFAULT, precision=lp.PREC_FP64))
    c.set_init(1)
    if U0 is not None:
        c.set_state(U0)
    c.step(NSTEPS)
    return c.field_energy()


def test_gradient_through_50_steps(gpu_lib):
    lp = gpu_lib
    ctx = lp.Context(lp.Params(**CFG4, fixes=lp.FIX_DEFAULT, precision=lp.PREC_FP64))
    ctx.set_init(1)
    U0 = ctx.get_state()
    g = _dev(np.zeros_like(U0))
    J, dnu = ctx.field_energy_gradient(NSTEPS, CHECK, g.data_ptr())
    torch.cuda.synchronize()
    gU = g.cpu().numpy()
    assert np.array_equal(ctx.get_state(), U0)  # the state is the initial state again
    assert abs(J - _J_after(lp)) <= 1e-12 * abs(J)
    # A: the initial state is linear in A
    u1 = lp.Context(lp.Params(**dict(CFG4, a_amp=1.0), fixes=lp.FIX_DEFAULT, precision=lp.PREC_FP64))
    u0 = lp.Context(lp.Params(**dict(CFG4, a_amp=0.0), fixes=lp.FIX_DEFAULT, precision=lp.PREC_FP64))
    u1.set_init(1)
    u0.set_init(1)
    dA = float(np.dot(gU, u1.get_state() - u0.get_state()))
    h = 1e-6
    fdA = (_J_after(lp, a_amp=CFG4["a_amp"] + h) - _J_after(lp, a_amp=CFG4["a_amp"] - h)) / (2 * h)
    assert abs(dA - fdA) <= 1e-6 * abs(fdA), (dA, fdA)
    # J moves very little with nu (dJ/dnu = -5.2e-5 at J = 0.285): the
    # rounding noise of a central difference of the 50-step run is about
    # 1.5e-10 / h relative (1.2e-4 at h = 1e-6, 1.5e-6 at h = 1e-4), its
    # truncation error 1.6e-7 at h = 1e-3.  Central differences at h = 2e-3
    # and 1e-3 combined by Richardson extrapolation (truncation O(h^4)) stay
    # below both; h = 1e-6 agrees to its noise floor.
    def cd(hn):
        return (_J_after(lp, nu=CFG4["nu"] + hn) - _J_after(lp, nu=CFG4["nu"] - hn)) / (2 * hn)

    fdnu = (4 * cd(1e-3) - cd(2e-3)) / 3
    assert abs(dnu - fdnu) <= 1e-6 * abs(fdnu), (dnu, fdnu)
    fdnu_h = cd(h)
    assert abs(dnu - fdnu_h) <= 1e-3 * abs(fdnu_h), (dnu, fdnu_h)
    rng = np.random.default_rng(20261203)
    for i in range(8):
        d = rng.standard_normal(U0.size) * np.abs(U0)
        fd = (_J_after(lp, U0 + h * d) - _J_after(lp, U0 - h * d)) / (2 * h)
        adj = float(np.dot(gU, d))
        assert abs(adj - fd) <= 1e-6 * abs(fd), (i, adj, fd)


# ---- the same gradient through torch.autograd.Function wrappers ----
class _Step(torch.autograd.Function):
    @staticmethod
    def forward(fctx, U, lpctx):
        torch.cuda.synchronize()
        lpctx.set_state(U.detach().cpu().numpy())
        lpctx.step(1)
        fctx.save_for_backward(U)
        fctx.lpctx = lpctx
        return _dev(lpctx.get_state())

    @staticmethod
    def backward(fctx, g):
        (U,) = fctx.saved_tensors
        torch.cuda.synchronize()
        fctx.lpctx.set_state(U.detach().cpu().numpy())
        g = g.contiguous()
        gi = torch.zeros_like(g)
        torch.cuda.synchronize()
        fctx.lpctx.step_vjp(g.data_ptr(), gi.data_ptr())
        return gi, None


class _Energy(torch.autograd.Function):
    @staticmethod
    def forward(fctx, U, lpctx):
        torch.cuda.synchronize()
        lpctx.set_state(U.detach().cpu().numpy())
        fctx.save_for_backward(U)
        fctx.lpctx = lpctx
        return torch.tensor(lpctx.field_energy(), dtype=torch.float64, device="cuda")

    @staticmethod
    def backward(fctx, g):
        (U,) = fctx.saved_tensors
        torch.cuda.synchronize()
        fctx.lpctx.set_state(U.detach().cpu().numpy())
        lam = torch.zeros_like(U)
        torch.cuda.synchronize()
        fctx.lpctx.field_energy(lam.data_ptr())
        torch.cuda.synchronize()
        return g * lam, None


def test_autograd_composition_matches_checkpointed_gradient(gpu_lib):
    lp = gpu_lib
    ctx = _ctx(lp, nx1=8)
    U0 = ctx.get_state()
    g = _dev(np.zeros_like(U0))
    J_ref, _ = ctx.field_energy_gradient(5, 2, g.data_ptr())
    torch.cuda.synchronize()
    U = _dev(U0).requires_grad_(True)
    X = U
    for _ in range(5):
        X = _Step.apply(X, ctx)
    J = _Energy.apply(X, ctx)
    (gU,) = torch.autograd.grad(J, U)
    assert abs(J.item() - J_ref) <= 1e-12 * abs(J_ref)
    assert torch.linalg.norm(gU - g) <= 1e-10 * torch.linalg.norm(g)


@pytest.mark.parametrize("n,nv", [(8, 8), (16, 6), (24, 4)], ids=["n8", "n16", "n24"])
def test_collision_vjp_forms_agree(gpu_lib, n, nv):
    """ComputeQ's VJP as correlations of the adjoint with the convolution
    form's omega-factor arrays (3n/2-point DFTs, the default) against the
    gather over the pair table of the weighted sum, through one collision
    step's adjoint (40 cells: two 32-cell chunks of the correlation form)."""
    lp = gpu_lib
    ctx = _ctx(lp, nx1=40, n=n, nv=nv)
    ctx.advect_step()
    U = ctx.get_state()
    w = np.random.default_rng(11).standard_normal(U.size)
    out = {}
    for form in (1, 0):
        ctx.set_adjoint_form(form)
        out[form] = _vjp(ctx, ctx.collision_vjp, U, w)
    (l1, d1), (l0, d0) = out[1], out[0]
    assert np.linalg.norm(l0 - l1) <= 1e-12 * np.linalg.norm(l1)
    assert abs(d0 - d1) <= 1e-12 * abs(d1)
