"""The two kernel forms of the convolution form of ComputeQ (mixed path):
form 1 keeps the axis-2 spectra on chip (axis-3 DFTs into device memory,
then one kernel per (k3, group of cells) for the axis-2 DFTs, the axis-1
sums and the inverse axis-2 DFTs), form 0 runs them as three kernels through
device memory.  Both evaluate the same FP32 operations except where the
b-arrays' axis-1 weight enters (before the axis-2 DFT in form 1, after it in
form 0).  ComputeQ at every supported n (the reference's golden vectors at
n = 8, 16, 24, the oracle at n = 32) and whole collision steps, including
passes split into several convolution chunks, agree to FP32 rounding between
the forms, and each stays within the FP32 tolerance of the reference
values."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN_NAMES, golden_case, load_golden, rel
from oracle.oracle import Case, FIX_DEFAULT, Oracle

pytestmark = pytest.mark.gpu

TOL_Q = 2e-5    # FP32 evaluation of Qhat against FP64 reference values
TOL_FORMS = 1e-6  # the two forms: FP32 evaluations of the same sums


def _ctx(lp, case, precision=None, fixes=FIX_DEFAULT):
    P = lp.Params(nx1=case.nx1, nx2=case.nx2, nv=case.nv, n=case.n, lv=case.lv, lx=case.lx, nu=case.nu,
                  dt=case.dt, a_amp=case.a_amp, k_wave=case.k_wave, fixes=fixes,
                  precision=lp.PREC_MIXED if precision is None else precision)
    return lp.Context(P)


def _both_forms(ctx, run):
    out = {}
    for form in (0, 1):
        ctx.set_convolution_form(form)
        assert ctx.convolution_form() == form
        out[form] = run()
        ctx.synchronize()  # no bounded wait of the fused kernel ran out
    return out[0], out[1]


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_compute_q_forms_golden(gpu_lib, name):
    g = load_golden(name)
    ctx = _ctx(gpu_lib, golden_case(g), fixes=0)
    ctx.set_schedule(32, 0)
    q0, q1 = _both_forms(ctx, lambda: ctx.compute_q(g["f_cell"]))
    assert rel(q1, q0) < TOL_FORMS
    assert rel(q1, g["qhat"]) < TOL_Q


def test_compute_q_forms_n32(gpu_lib):
    case = Case(nx1=2, nx2=1, nv=4, n=32, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    O = Oracle(case, fixes=FIX_DEFAULT)
    v, _, _, _ = O.grids()
    V1, V2, V3 = np.meshgrid(v, v, v, indexing="ij")
    f = (np.exp(-((V1 - 0.7) ** 2 + V2 ** 2 + V3 ** 2) / 2)
         + 0.4 * np.exp(-((V1 + 1.2) ** 2 + (V2 - 0.3) ** 2 + 1.5 * V3 ** 2) / 2)).reshape(-1)
    ctx = _ctx(gpu_lib, case)
    ctx.set_schedule(32, 0)
    q0, q1 = _both_forms(ctx, lambda: ctx.compute_q(f))
    assert rel(q1, q0) < TOL_FORMS
    assert rel(q1, O.compute_q(f)) < TOL_Q


# every supported n; nx1 = 160 with passes of 160 cells and convolution
# chunks of at most 64 cells (LP_FQ_CHUNK=64) splits each pass into chunks of
# 64, 64 and 32 cells; the 2-D case runs 12 x 8
@pytest.mark.parametrize("nx1,nx2,n,nv,lv,chunk", [(40, 1, 8, 8, 5.25, 0), (160, 1, 16, 4, 5.25, 64),
                                                    (64, 1, 24, 8, 5.0, 0), (12, 8, 24, 8, 5.0, 0),
                                                    (36, 1, 32, 4, 5.25, 0)],
                         ids=["n8", "n16-chunks", "n24", "n24-2d", "n32"])
def test_collision_step_forms(gpu_lib, monkeypatch, nx1, nx2, n, nv, lv, chunk):
    lp = gpu_lib
    case = Case(nx1=nx1, nx2=nx2, nv=nv, n=n, lv=lv, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    if chunk:
        monkeypatch.setenv("LP_FQ_CHUNK", str(chunk))
    ctx = _ctx(lp, case)
    monkeypatch.delenv("LP_FQ_CHUNK", raising=False)
    ctx.set_schedule(min(160, ((nx1 * nx2 + 31) // 32) * 32), 0)
    ctx.set_init(1)
    U0 = ctx.get_state()
    m0 = ctx.moments()

    def run():
        ctx.set_state(U0)
        ctx.collision_step()
        return ctx.get_state(), ctx.moments()

    (u0, _), (u1, m1) = _both_forms(ctx, run)
    assert rel(u1, u0) < TOL_FORMS
    # the collision keeps mass, momentum and kinetic energy
    assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-12
    assert np.all(np.abs(m1[1:4] - m0[1:4]) / abs(m0[0]) < 1e-12)
    assert abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-12
    ref = _ctx(lp, case, precision=lp.PREC_FP64)
    ref.set_state(U0)
    ref.collision_step()
    assert rel(u1, ref.get_state()) < 1e-6


def test_graph_replay_after_form_change(gpu_lib):
    """Changing the form drops the captured step graph: the next full steps
    (captured again) run the new form's kernels and match the steps of the
    other form."""
    lp = gpu_lib
    case = Case(nx1=64, nx2=1, nv=8, n=24, lv=5.0, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    ctx = _ctx(lp, case)
    ctx.set_schedule(64, 0)
    ctx.set_init(1)
    U0 = ctx.get_state()
    ctx.set_convolution_form(0)
    ctx.step(2)
    s0 = ctx.get_state()
    ctx.set_convolution_form(1)
    ctx.set_state(U0)
    ctx.step(2)
    ctx.synchronize()
    s1 = ctx.get_state()
    assert rel(s1, s0) < TOL_FORMS
    with pytest.raises(lp.LPError):
        ctx.set_convolution_form(2)


@pytest.mark.parametrize("n,nv", [(24, 8), (16, 4)])
def test_chunked_convolution_passes(gpu_lib, monkeypatch, n, nv):
    """LP_FQ_CHUNK=32 at context creation splits each 96-cell pass into three
    convolution chunks of 32 cells.  Every cell's sums, and its conservation
    partials, are the same operations in the same order as in one chunk of
    96, so a whole time step matches the unsplit context bit for bit, in
    both kernel forms."""
    lp = gpu_lib
    case = Case(nx1=96, nx2=1, nv=nv, n=n, lv=5.0, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)

    def run(chunk):
        if chunk:
            monkeypatch.setenv("LP_FQ_CHUNK", str(chunk))
        else:
            monkeypatch.delenv("LP_FQ_CHUNK", raising=False)
        ctx = _ctx(lp, case)
        ctx.set_schedule(96, 0)
        ctx.set_init(1)
        U0 = ctx.get_state()
        out = []
        for form in (0, 1):
            ctx.set_convolution_form(form)
            ctx.set_state(U0)
            ctx.step(1)
            ctx.synchronize()
            out.append(ctx.get_state())
        return out

    whole, split = run(0), run(32)
    monkeypatch.delenv("LP_FQ_CHUNK", raising=False)
    for form in (0, 1):
        assert np.array_equal(split[form], whole[form])
