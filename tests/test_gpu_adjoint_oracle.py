"""The GPU adjoint gradient against an independent FP64 reference gradient:
central differences of the CPU oracle's own time steps.  The physics of the
gradient workload (A = 0.05, k = 0.5, nu = 0.02, dt = 0.01, unit Maxwellian,
field energy J = 1/2 sum dx dy (E_0^2 + (E_1^2 + E_2^2)/12) over E_x and
E_y) on a reduced grid (Nx = 16, Nv = N = 8) through 10 steps with a
checkpoint every 5, so the oracle's forward runs take seconds: dJ/dA, dJ/dnu
and four seeded directions in f0, each to 1e-6."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import Case, FIX_DEFAULT, Oracle

pytestmark = pytest.mark.gpu

KW = dict(nx1=16, nx2=1, nv=8, n=8, lv=5.25, lx=4 * np.pi, nu=0.02, dt=0.01, a_amp=0.05, k_wave=0.5)
NSTEPS, CHECK = 10, 5


def _J_oracle(U0=None, **over):
    case = Case(**dict(KW, **over))
    O = Oracle(case, fixes=FIX_DEFAULT)
    U = O.set_init(1) if U0 is None else np.array(U0)
    for _ in range(NSTEPS):
        U = O.step(U)
    _, px, py, _ = O.poisson(U)
    dx, dy = case.lx / case.nx1, case.lx / case.nx2
    px, py = px.reshape(-1, 3), py.reshape(-1, 3)
    e = px[:, 0] ** 2 + (px[:, 1] ** 2 + px[:, 2] ** 2) / 12 + py[:, 0] ** 2 + (py[:, 1] ** 2 + py[:, 2] ** 2) / 12
    return 0.5 * dx * dy * float(e.sum())


def test_adjoint_gradient_vs_oracle_differences(gpu_lib):
    torch = pytest.importorskip("torch")
    lp = gpu_lib
    P = lp.Params(**KW, fixes=FIX_DEFAULT, precision=lp.PREC_FP64)
    ctx = lp.Context(P)
    ctx.set_init(1)
    U0 = ctx.get_state()
    g = torch.zeros(U0.size, dtype=torch.float64, device="cuda")
    J, dnu = ctx.field_energy_gradient(NSTEPS, CHECK, g.data_ptr())
    torch.cuda.synchronize()
    gU = g.cpu().numpy()
    assert abs(J - _J_oracle()) <= 1e-12 * abs(J)
    # A: the initial state is linear in A
    O = Oracle(Case(**dict(KW, a_amp=1.0)), fixes=FIX_DEFAULT)
    O0 = Oracle(Case(**dict(KW, a_amp=0.0)), fixes=FIX_DEFAULT)
    dA = float(np.dot(gU, O.set_init(1) - O0.set_init(1)))
    h = 1e-6
    fdA = (_J_oracle(a_amp=KW["a_amp"] + h) - _J_oracle(a_amp=KW["a_amp"] - h)) / (2 * h)
    assert abs(dA - fdA) <= 1e-6 * abs(fdA), (dA, fdA)

    # nu: Richardson extrapolation of central differences at 2e-3 and 1e-3
    # (J depends weakly on nu; smaller steps meet the rounding floor)
    def cd(hn):
        return (_J_oracle(nu=KW["nu"] + hn) - _J_oracle(nu=KW["nu"] - hn)) / (2 * hn)

    fdnu = (4 * cd(1e-3) - cd(2e-3)) / 3
    assert abs(dnu - fdnu) <= 1e-6 * abs(fdnu), (dnu, fdnu)
    rng = np.random.default_rng(20261205)
    for i in range(4):
        d = rng.standard_normal(U0.size) * np.abs(U0)
        fd = (_J_oracle(U0 + h * d) - _J_oracle(U0 - h * d)) / (2 * h)
        adj = float(np.dot(gU, d))
        assert abs(adj - fd) <= 1e-6 * abs(fd), (i, adj, fd)
