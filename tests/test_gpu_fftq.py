"""The convolution form of the mixed path's contraction (schedule form 0):
ComputeQ against the reference's own values (golden vectors, n = 8, 16, 24)
and the oracle (n = 32) at FP32 accuracy, against the line-tiled form of the
same context, whole collision steps against the FP64 path at 1e-6 with the
moments kept to 1e-12, and passes that split the cells into several
convolution chunks."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN_NAMES, golden_case, load_golden, rel
from oracle.oracle import Case, FIX_DEFAULT, Oracle

pytestmark = pytest.mark.gpu

# relative L2 error of an FP32 evaluation of Qhat (its terms cancel to a
# small remainder near equilibrium; the error enters f scaled by dt nu)
TOL_Q = 2e-5


def _ctx(lp, case, precision, fixes=FIX_DEFAULT):
    P = lp.Params(nx1=case.nx1, nx2=case.nx2, nv=case.nv, n=case.n, lv=case.lv, lx=case.lx, nu=case.nu,
                  dt=case.dt, a_amp=case.a_amp, k_wave=case.k_wave, fixes=fixes, precision=precision)
    return lp.Context(P)


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_compute_q_golden(gpu_lib, name):
    g = load_golden(name)
    ctx = _ctx(gpu_lib, golden_case(g), gpu_lib.PREC_MIXED, fixes=0)
    ctx.set_schedule(32, 0)
    q_conv = ctx.compute_q(g["f_cell"])
    assert rel(q_conv, g["qhat"]) < TOL_Q
    ctx.set_schedule(32, 2)
    q_lines = ctx.compute_q(g["f_cell"])
    assert rel(q_conv, q_lines) < TOL_Q


def test_compute_q_n32(gpu_lib):
    case = Case(nx1=2, nx2=1, nv=4, n=32, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    O = Oracle(case, fixes=FIX_DEFAULT)
    v, _, _, _ = O.grids()
    V1, V2, V3 = np.meshgrid(v, v, v, indexing="ij")
    f = (np.exp(-((V1 - 0.7) ** 2 + V2 ** 2 + V3 ** 2) / 2)
         + 0.4 * np.exp(-((V1 + 1.2) ** 2 + (V2 - 0.3) ** 2 + 1.5 * V3 ** 2) / 2)).reshape(-1)
    ctx = _ctx(gpu_lib, case, gpu_lib.PREC_MIXED)
    ctx.set_schedule(32, 0)
    assert rel(ctx.compute_q(f), O.compute_q(f)) < TOL_Q


# (n = 24 with lv 5.25 or 6 and nv < n grows without bound in the oracle too)
@pytest.mark.parametrize("n,nv,lv", [(8, 8, 5.25), (16, 8, 5.25), (24, 8, 5.0), (32, 4, 5.25)])
def test_collision_vs_fp64(gpu_lib, n, nv, lv):
    lp = gpu_lib
    case = Case(nx1=4, nx2=1, nv=nv, n=n, lv=lv, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    mix = _ctx(lp, case, lp.PREC_MIXED)
    ref = _ctx(lp, case, lp.PREC_FP64)
    mix.set_schedule(32, 0)
    mix.set_init(1)
    ref.set_init(1)
    m0 = mix.moments()
    for _ in range(2):
        mix.collision_step()
        ref.collision_step()
    assert rel(mix.get_state(), ref.get_state()) < 1e-6
    m1 = mix.moments()
    assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-12
    assert np.all(np.abs(m1[1:4] - m0[1:4]) / abs(m0[0]) < 1e-12)
    assert abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-12


def test_steps_vs_oracle(gpu_lib):
    case = Case(nx1=8, nx2=1, nv=8, n=16, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    ctx = _ctx(gpu_lib, case, gpu_lib.PREC_MIXED)
    ctx.set_schedule(32, 0)
    O = Oracle(case, fixes=FIX_DEFAULT)
    U = O.set_init(1)
    ctx.set_state(U)
    for _ in range(3):
        U = O.step(U)
    ctx.step(3)
    assert rel(ctx.get_state(), U) < 1e-6


def test_chunked_passes(gpu_lib):
    """160 cells: passes of 160 cells split into convolution chunks of 64, 64
    and 32 cells, and passes of 96; both equal the line-tiled form."""
    lp = gpu_lib
    case = Case(nx1=160, nx2=1, nv=4, n=16, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    states = []
    for sched in [(160, 2), (160, 0), (96, 0)]:
        ctx = _ctx(lp, case, lp.PREC_MIXED)
        ctx.set_schedule(*sched)
        ctx.set_init(1)
        ctx.collision_step()
        states.append(ctx.get_state())
    assert rel(states[1], states[0]) < 1e-6
    assert rel(states[2], states[1]) < 1e-6


def test_set_schedule_rejects(gpu_lib):
    lp = gpu_lib
    case = Case(nx1=4, nx2=1, nv=4, n=12, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    ctx = _ctx(lp, case, lp.PREC_MIXED)  # n = 12: no line-tiled or convolution form
    with pytest.raises(lp.LPError):
        ctx.set_schedule(32, 0)
    with pytest.raises(lp.LPError):
        ctx.set_schedule(48, 2)
    ctx.set_schedule(32, 2)


@pytest.mark.parametrize("n,nv", [(16, 5), (16, 7), (8, 28)], ids=["nv5", "nv7", "nv28"])
def test_collision_odd_and_large_nv(gpu_lib, n, nv):
    """The mixed projection's odd-Nv branches (guarded factor loads, the
    scalar axis-3/axis-2 loops) and its eight-outputs-per-thread variant
    (Nv in 25..32) against the FP64 path, with mass and energy kept."""
    lp = gpu_lib
    case = Case(nx1=2, nx2=1, nv=nv, n=n, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    mix = _ctx(lp, case, lp.PREC_MIXED)
    ref = _ctx(lp, case, lp.PREC_FP64)
    mix.set_init(1)
    ref.set_init(1)
    m0 = mix.moments()
    mix.collision_step()
    ref.collision_step()
    assert rel(mix.get_state(), ref.get_state()) < 1e-6
    m1 = mix.moments()
    assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-12
    assert abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-12
