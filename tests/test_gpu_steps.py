"""Whole-step parity of the GPU path with the CPU oracle (defects F1-F3 fixed),
in the 1-D reduction (nx2 = 1) and the 2-D layout, FP64 at 1e-12 relative L2
in the state and the field; the mixed path against FP64 at 1e-6 with the
moments kept to 1e-12 by the collision step."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel
from oracle.oracle import Case, FIX_DEFAULT, Oracle

pytestmark = pytest.mark.gpu


def _pair(lp, case, precision=None, kind=1):
    P = lp.Params(nx1=case.nx1, nx2=case.nx2, nv=case.nv, n=case.n, lv=case.lv, lx=case.lx,
                  nu=case.nu, dt=case.dt, a_amp=case.a_amp, k_wave=case.k_wave,
                  fixes=FIX_DEFAULT, precision=lp.PREC_FP64 if precision is None else precision)
    ctx = lp.Context(P)
    O = Oracle(case, fixes=FIX_DEFAULT)
    U0 = O.set_init(kind)
    ctx.set_state(U0)
    return ctx, O, U0


CASES_1D = [Case(nx1=8, nx2=1, nv=8, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5,
                 k_wave=0.5),
            Case(nx1=6, nx2=1, nv=6, n=16, lv=5.25, lx=4 * np.pi, nu=0.01, dt=0.01, a_amp=0.01,
                 k_wave=0.5)]


@pytest.mark.parametrize("case", CASES_1D, ids=["n8", "n16"])
def test_steps_1d(gpu_lib, case):
    ctx, O, U = _pair(gpu_lib, case)
    for _ in range(3):
        U = O.step(U)
        ctx.step(1)
        Ug = ctx.get_state()
        assert rel(Ug, U) < 1e-12
    _, px_o, _, _ = O.poisson(U)
    _, px_g, _, _ = ctx.poisson()
    assert rel(px_g, px_o) < 1e-12


def test_steps_2d(gpu_lib):
    case = Case(nx1=3, nx2=3, nv=6, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.005, a_amp=0.5,
                k_wave=0.5)
    ctx, O, U = _pair(gpu_lib, case, kind=0)
    for _ in range(2):
        U = O.step(U)
    ctx.step(2)
    assert rel(ctx.get_state(), U) < 1e-12


def test_collision_conserves_moments(gpu_lib):
    case = Case(nx1=4, nx2=1, nv=8, n=16, lv=5.25, lx=4 * np.pi, nu=0.1, dt=0.01, a_amp=0.2,
                k_wave=0.5)
    for prec in (gpu_lib.PREC_FP64, gpu_lib.PREC_MIXED):
        ctx, O, U = _pair(gpu_lib, case, precision=prec)
        m0 = ctx.moments()
        ctx.collision_step()
        m1 = ctx.moments()
        assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-12, (prec, m1 - m0)  # mass
        assert np.all(np.abs(m1[1:4] - m0[1:4]) / abs(m0[0]) < 1e-12), (prec, m1 - m0)  # momentum
        assert abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-12, (prec, m1 - m0)  # kinetic energy


def test_mixed_vs_fp64(gpu_lib):
    case = Case(nx1=8, nx2=1, nv=8, n=16, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5,
                k_wave=0.5)
    ctx, O, U = _pair(gpu_lib, case, precision=gpu_lib.PREC_MIXED)
    for _ in range(3):
        U = O.step(U)
    ctx.step(3)
    assert rel(ctx.get_state(), U) < 1e-6


@pytest.mark.parametrize("nx1,nx2,nv", [(8, 1, 8), (8, 1, 6), (4, 3, 8)],
                         ids=["1d-fused-charge", "1d-separate-charge", "2d"])
def test_mixed_advection(gpu_lib, nx1, nx2, nv):
    """FP32 DG flux with FP64 stage combinations, charge and Poisson: the
    collisionless step against the FP64 oracle (nv^3 = 512 takes the fused
    charge partials, nv^3 = 216 the separate charge sum).  No cell centre
    sits on a zero of E_x: there the v1 upwind direction follows the sign of
    a field at rounding level, which only a bit-identical solve reproduces."""
    case = Case(nx1=nx1, nx2=nx2, nv=nv, n=8, lv=5.25, lx=4 * np.pi, nu=0.0, dt=0.01, a_amp=0.5,
                k_wave=0.5)
    ctx, O, U = _pair(gpu_lib, case, precision=gpu_lib.PREC_MIXED)
    for _ in range(4):
        U = O.step(U)
    ctx.step(4)
    Ug = ctx.get_state()
    assert rel(Ug, U) < 1e-6
    _, px_o, _, _ = O.poisson(U)
    _, px_g, _, _ = ctx.poisson()
    assert rel(px_g, px_o) < 1e-6


@pytest.mark.parametrize("n,nv", [(12, 6), (32, 4)], ids=["n12-pair-kernel", "n32-line-kernel"])
def test_mixed_vs_fp64_other_n(gpu_lib, n, nv):
    """The mixed path off the line-tiled sizes (n = 12: the FP32 pair kernel)
    and at the largest n (32: four k-tiles), against the FP64 GPU path."""
    lp = gpu_lib
    kw = dict(nx1=4, nx2=1, nv=nv, n=n, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5,
              fixes=FIX_DEFAULT)
    mix = lp.Context(lp.Params(**kw, precision=lp.PREC_MIXED))
    ref = lp.Context(lp.Params(**kw, precision=lp.PREC_FP64))
    mix.set_init(1)
    ref.set_init(1)
    m0 = mix.moments()
    mix.collision_step()
    ref.collision_step()
    assert rel(mix.get_state(), ref.get_state()) < 1e-6
    m1 = mix.moments()
    assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-12
    assert abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-12
