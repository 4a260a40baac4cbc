"""The convolution form of ComputeQ in FP64, the FP64 path's default for
n in {8, 16, 24, 32} on a uniform node grid.

- Against the reference's golden ComputeQ at n = 8 and 16 (its own grids,
  no fixes) to 1e-12.
- Against the pair form (LP_FQ64=0 at context creation) at every n:
  ComputeQ to 1e-13 (measured 1.5e-15 to 6.6e-15), a whole collision
  step's increment to 1e-11 (measured 3.1e-13 at n = 16).
- Against the oracle to 1e-12, and to 1e-11 at n = 32.  Both GPU forms
  differ from it by the same amount (measured 2.0e-14, 2.2e-13 and 9.0e-13
  at n = 8, 16, 24; 5.0e-12 at n = 32 with v in [-5.25, 5.25]^3): they
  start from the GPU's FP64 transform of f, which rounds differently from
  the oracle's, and ComputeQ carries that absolute error into its small
  outputs (tests/test_oracle_convolution_form.py measures the effect on the
  oracle's own transform; there the convolution form's FP64 sums match the
  oracle's direct sum to 1.2e-14).
- The fallback where defect F11 leaves the middle node off zero (n = 24
  without the fix): the context keeps the pair form, so its results are the
  pair form's bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_case, load_golden, rel
from oracle.oracle import Case, FIX_DEFAULT, Oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12       # FP64 against the reference's golden values
TOL_FORMS = 1e-13  # ComputeQ of the two FP64 forms on the GPU
# a collision step's increment (a small difference after four stages, the
# conservation and the projection) of the two forms: 3.1e-13 at n = 16
TOL_STEP = 1e-11
TOL_ORACLE = {8: 1e-12, 16: 1e-12, 24: 1e-12, 32: 1e-11}


def _ctx(lp, monkeypatch, case, fixes, pair=False):
    if pair:
        monkeypatch.setenv("LP_FQ64", "0")
    else:
        monkeypatch.delenv("LP_FQ64", raising=False)
    P = lp.Params(nx1=case.nx1, nx2=case.nx2, nv=case.nv, n=case.n, lv=case.lv, lx=case.lx, nu=case.nu,
                  dt=case.dt, a_amp=case.a_amp, k_wave=case.k_wave, fixes=fixes, precision=lp.PREC_FP64)
    ctx = lp.Context(P)
    monkeypatch.delenv("LP_FQ64", raising=False)
    return ctx


def _f(O, n):
    v, _, _, _ = O.grids()
    V1, V2, V3 = np.meshgrid(v, v, v, indexing="ij")
    return (np.exp(-((V1 - 0.7) ** 2 + V2 ** 2 + V3 ** 2) / 2)
            + 0.4 * np.exp(-((V1 + 1.2) ** 2 + (V2 - 0.3) ** 2 + 1.5 * V3 ** 2) / 2)).reshape(-1)


@pytest.mark.parametrize("name", ["ref_n8", "ref_n16"])
def test_compute_q_golden(gpu_lib, monkeypatch, name):
    g = load_golden(name)
    case = golden_case(g)
    q1 = _ctx(gpu_lib, monkeypatch, case, 0).compute_q(g["f_cell"])
    q0 = _ctx(gpu_lib, monkeypatch, case, 0, pair=True).compute_q(g["f_cell"])
    assert rel(q1, g["qhat"]) < TOL
    assert rel(q1, q0) < TOL_FORMS


@pytest.mark.parametrize("n", [8, 16, 24, 32])
def test_compute_q_oracle(gpu_lib, monkeypatch, n):
    case = Case(nx1=2, nx2=1, nv=4, n=n, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    O = Oracle(case, fixes=FIX_DEFAULT)
    f = _f(O, n)
    q1 = _ctx(gpu_lib, monkeypatch, case, FIX_DEFAULT).compute_q(f)
    q0 = _ctx(gpu_lib, monkeypatch, case, FIX_DEFAULT, pair=True).compute_q(f)
    assert rel(q1, O.compute_q(f)) < TOL_ORACLE[n]
    assert rel(q1, q0) < TOL_FORMS


def test_f11_unfixed_keeps_the_pair_form(gpu_lib, monkeypatch):
    """n = 24 without the F11 fix: the middle node is 8.9e-16, not 0, so the
    context evaluates ComputeQ in the pair form whatever LP_FQ64 says."""
    g = load_golden("ref_n24")
    case = golden_case(g)
    q1 = _ctx(gpu_lib, monkeypatch, case, 0).compute_q(g["f_cell"])
    q0 = _ctx(gpu_lib, monkeypatch, case, 0, pair=True).compute_q(g["f_cell"])
    assert np.array_equal(q1, q0)
    assert rel(q1, g["qhat"]) < TOL


# 1-D and 2-D grids; nx1 = 96 at n = 24 splits a pass of 96 cells into FP64
# convolution chunks of 64 + 32, nx1 = 40 at n = 32 one of 64 into 32 + 32
@pytest.mark.parametrize("nx1,nx2,n,nv", [(40, 1, 8, 8), (12, 4, 16, 4), (36, 1, 24, 8), (96, 1, 24, 4),
                                          (40, 1, 32, 4)],
                         ids=["n8", "n16-2d", "n24", "n24-chunks", "n32-chunks"])
def test_collision_step(gpu_lib, monkeypatch, nx1, nx2, n, nv):
    lp = gpu_lib
    case = Case(nx1=nx1, nx2=nx2, nv=nv, n=n, lv=5.0, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    out = []
    for pair in (False, True):
        ctx = _ctx(lp, monkeypatch, case, FIX_DEFAULT, pair=pair)
        ctx.set_init(1)
        U0 = ctx.get_state()
        m0 = ctx.moments()
        ctx.collision_step()
        m1 = ctx.moments()
        # the collision keeps mass, momentum and kinetic energy
        assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-12
        assert np.all(np.abs(m1[1:4] - m0[1:4]) / abs(m0[0]) < 1e-12)
        assert abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-12
        out.append(ctx.get_state() - U0)
    assert rel(out[0], out[1]) < TOL_STEP
