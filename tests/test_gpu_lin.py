"""The two-species variant (the reference's FullandLinear switch) on the GPU:
ComputeQ with its linear electron-ion term, the two conservations and RK4
against the reference's own FullandLinear build (golden vectors), and whole
steps against the oracle; the mixed path against FP64 with mass and energy
conserved (the linear operator does not conserve momentum)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_case, load_golden, rel
from oracle.oracle import Case, FIX_DEFAULT, Oracle

pytestmark = pytest.mark.gpu


def _ctx(lp, case, fixes, precision=None):
    P = lp.Params(nx1=case.nx1, nx2=case.nx2, nv=case.nv, n=case.n, lv=case.lv, lx=case.lx, nu=case.nu,
                  dt=case.dt, a_amp=case.a_amp, k_wave=case.k_wave, fixes=fixes,
                  precision=lp.PREC_FP64 if precision is None else precision, linear_ei=1)
    return lp.Context(P)


def test_golden_compute_conserve_rk4(gpu_lib):
    g = load_golden("ref_lin_n8")
    case = golden_case(g)
    ctx = _ctx(gpu_lib, case, 0)
    q, ql = ctx.compute_q_lin(g["f_cell"])
    assert rel(q, g["qhat"]) < 1e-12 and rel(ql, g["qhat_lin"]) < 1e-12
    qc, qlc = ctx.conserve_lin(g["qhat"], g["qhat_lin"])
    assert rel(qc, g["qhat_cons"]) < 1e-12 and rel(qlc, g["qlin_cons"]) < 1e-12
    ctx.set_state(g["rk4_state"])  # the reference's stride-6 reads (defect F1 kept)
    du = ctx.rk4_cell_lin(g["f_cell"], 1, g["qhat_cons"], g["qlin_cons"])
    assert rel(du, g["rk4_du"]) < 1e-12


CASE = Case(nx1=4, nx2=1, nv=4, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.3, k_wave=0.5,
            linear_ei=1)


def test_steps_vs_oracle(gpu_lib):
    ctx = _ctx(gpu_lib, CASE, FIX_DEFAULT)
    O = Oracle(CASE, fixes=FIX_DEFAULT)
    U = O.set_init(1)
    ctx.set_state(U)
    for _ in range(2):
        U = O.step(U)
        ctx.step(1)
        assert rel(ctx.get_state(), U) < 1e-12


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_collision_conserves_mass_energy(gpu_lib, prec):
    lp = gpu_lib
    ctx = _ctx(lp, CASE, FIX_DEFAULT, lp.PREC_FP64 if prec == "fp64" else lp.PREC_MIXED)
    ctx.set_init(1)
    m0 = ctx.moments()
    ctx.collision_step()
    m1 = ctx.moments()
    assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-12
    assert abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-12


def test_mixed_vs_fp64(gpu_lib):
    lp = gpu_lib
    a = _ctx(lp, CASE, FIX_DEFAULT, lp.PREC_MIXED)
    b = _ctx(lp, CASE, FIX_DEFAULT, lp.PREC_FP64)
    a.set_init(1)
    b.set_init(1)
    a.step(2)
    b.step(2)
    assert rel(a.get_state(), b.get_state()) < 1e-6


def test_mixed_vs_fp64_convolution_form(gpu_lib):
    """n = 16: the quadratic term in the convolution form (the default), the
    linear term by its window contraction; mass and energy conserved."""
    lp = gpu_lib
    case = Case(nx1=4, nx2=1, nv=8, n=16, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.3, k_wave=0.5,
                linear_ei=1)
    a = _ctx(lp, case, FIX_DEFAULT, lp.PREC_MIXED)
    b = _ctx(lp, case, FIX_DEFAULT, lp.PREC_FP64)
    a.set_init(1)
    assert a.autotune(reps=1)[1] in (0, 2, 4)
    a.set_schedule(32, 0)
    a.set_init(1)
    b.set_init(1)
    m0 = a.moments()
    a.step(2)
    b.step(2)
    assert rel(a.get_state(), b.get_state()) < 1e-6
    a2 = _ctx(lp, case, FIX_DEFAULT, lp.PREC_MIXED)
    a2.set_schedule(32, 0)
    a2.set_init(1)
    a2.collision_step()
    m1 = a2.moments()
    assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-12
    assert abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-12

