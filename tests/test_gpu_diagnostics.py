"""Device diagnostics and state files: lp_diagnostics (moments after a
Poisson solve of the state, electric energy, entropy), the (x1, v1)
marginal, the reference's moment and entropy lines, and snapshot
append/restart in the reference's raw format -- against the oracle."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import rel
from oracle.oracle import Case, FIX_DEFAULT, Oracle

pytestmark = pytest.mark.gpu

CASE = Case(nx1=8, nx2=1, nv=8, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)


def _ctx(lp):
    P = lp.Params(nx1=CASE.nx1, nx2=CASE.nx2, nv=CASE.nv, n=CASE.n, lv=CASE.lv, lx=CASE.lx, nu=CASE.nu,
                  dt=CASE.dt, a_amp=CASE.a_amp, k_wave=CASE.k_wave, fixes=FIX_DEFAULT, precision=lp.PREC_FP64)
    ctx = lp.Context(P)
    O = Oracle(CASE, fixes=FIX_DEFAULT)
    U = O.set_init(1)
    for _ in range(2):
        U = O.step(U)
    ctx.set_state(U)
    return ctx, O, U


def test_diagnostics_match_oracle(gpu_lib):
    ctx, O, U = _ctx(gpu_lib)
    d = ctx.diagnostics()
    _, px, py, _ = O.poisson(U)
    m = O.moments(U, px, py)
    assert abs(d[0] - m[0]) <= 1e-12 * abs(m[0])
    assert np.all(np.abs(d[1:4] - m[1:4]) <= 1e-12 * abs(m[0]))
    assert abs(d[4] - m[4]) <= 1e-12 * abs(m[4])
    assert abs(d[5] - m[5]) <= 1e-12 * abs(m[5])
    assert abs(d[6] - np.sqrt(m[5])) <= 1e-12 * np.sqrt(m[5])
    assert abs(d[8] - (m[4] + m[5])) <= 1e-12 * abs(m[4] + m[5])
    ent = O.entropy(U)
    assert abs(d[9] - ent) <= 1e-5 * abs(ent)  # FP32 integrand


def test_marginal_matches_oracle(gpu_lib):
    ctx, O, U = _ctx(gpu_lib)
    assert np.array_equal(ctx.marginal_x1v1(), O.marginal_x1v1(U))


def test_moment_and_entropy_lines(gpu_lib, tmp_path):
    ctx, O, U = _ctx(gpu_lib)
    mp, ep = str(tmp_path / "moments.dc"), str(tmp_path / "entropy.dc")
    ctx.diagnostics_append(mp, ep)
    ctx.step(1)
    ctx.diagnostics_append(mp, ep)
    mom = [list(map(float, l.split())) for l in open(mp).read().splitlines()]
    ent = [list(map(float, l.split())) for l in open(ep).read().splitlines()]
    assert len(mom) == 2 and all(len(r) == 9 for r in mom)
    assert len(ent) == 2 and all(len(r) == 3 for r in ent)
    d = ctx.diagnostics()
    assert np.allclose(mom[1], d[:9], rtol=1e-7, atol=0)  # printed with 8 significant digits
    assert abs(ent[1][1] - np.log(abs(ent[1][0]))) <= 1e-6


def test_state_append_restart(gpu_lib, tmp_path):
    ctx, O, U = _ctx(gpu_lib)
    path = str(tmp_path / "U.dc")
    ctx.state_append(path)
    ctx.step(1)
    U1 = ctx.get_state()
    ctx.state_append(path)
    assert os.path.getsize(path) == 2 * U.size * 8
    ctx.set_state(U)
    ctx.state_restart(path)
    assert np.array_equal(ctx.get_state(), U1)
    with open(path, "ab") as f:  # a partial snapshot makes the file unreadable
        f.write(b"\0" * 8)
    with pytest.raises(gpu_lib.LPError):
        ctx.state_restart(path)
    assert rel(np.fromfile(path, dtype=np.float64)[:U.size], U) == 0.0
