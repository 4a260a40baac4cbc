"""The GPU path against the CPU oracle at the grids of the named workloads,
not only on toy grids (defects F1-F3, F11, F12 fixed on both sides):

- weak Landau damping: Nx = 24 (1-D), Nv = N = 16, v in [-5.25, 5.25]^3,
  A = 0.01, k = 0.5, nu = 0.01, dt = 0.01 -- states and E_x after 1, 5 and
  10 full time steps;
- strong Landau damping: Nx = 64, Nv = N = 24, v in [-6, 6]^3, A = 0.5,
  nu = 0.05, dt = 0.005 -- one full time step of all 64 cells, and the
  conservation of mass, momentum and kinetic energy by one collision step;
- two-stream: Nx = 256, Nv = N = 32, v in [-8, 8]^3, u = 2, A = 0.01,
  k = 0.3, nu = 0.01, dt = 0.0025 -- one collision step of four sampled
  spatial cells (the oracle collides them one at a time).

FP64 within 1e-12 relative L2 in U and E_x; the mixed path within 1e-6 of
the same oracle states.  Also: the initial condition of lp_set_init against
the reference's SetInit_LD (golden U_init) and the oracle's restatement of
its unit-Maxwellian and two-stream variants, and the Landau damping rate of
the GPU's collisionless step against linear theory."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN_NAMES, golden_case, load_golden, rel
from landau_rate import GAMMA_K05, OMEGA_K05, rate
from oracle.oracle import Case, FIX_DEFAULT, Oracle

pytestmark = pytest.mark.gpu

WEAK = Case(nx1=24, nx2=1, nv=16, n=16, lv=5.25, lx=4 * np.pi, nu=0.01, dt=0.01, a_amp=0.01, k_wave=0.5)
STRONG = Case(nx1=64, nx2=1, nv=24, n=24, lv=6.0, lx=4 * np.pi, nu=0.05, dt=0.005, a_amp=0.5, k_wave=0.5)
TWOSTREAM = Case(nx1=256, nx2=1, nv=32, n=32, lv=8.0, lx=2 * np.pi / 0.3, nu=0.01, dt=0.0025, a_amp=0.01,
                 k_wave=0.3)


def _ctx(lp, case, precision):
    return lp.Context(lp.Params(nx1=case.nx1, nx2=case.nx2, nv=case.nv, n=case.n, lv=case.lv, lx=case.lx,
                                nu=case.nu, dt=case.dt, a_amp=case.a_amp, k_wave=case.k_wave,
                                fixes=FIX_DEFAULT, precision=precision))


def _ex(ctx):
    _, px, _, _ = ctx.poisson()
    return px


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_set_init_matches_reference(gpu_lib, name):
    """kind 0 is SetInit_LD of the reference (source/SetInit_1.cpp:60-115)."""
    g = load_golden(name)
    c = golden_case(g)
    ctx = gpu_lib.Context(gpu_lib.Params(nx1=c.nx1, nx2=c.nx2, nv=c.nv, n=c.n, lv=c.lv, lx=c.lx, nu=c.nu,
                                         dt=c.dt, a_amp=c.a_amp, k_wave=c.k_wave, fixes=0))
    ctx.set_init(0)
    assert rel(ctx.get_state(), g["U_init"]) < 1e-14
    ctx.close()


@pytest.mark.parametrize("case,kind", [(WEAK, 1), (STRONG, 1), (Case(nx1=8, nx2=1, nv=32, n=8, lv=8.0,
                                                                      lx=2 * np.pi / 0.3, a_amp=0.01,
                                                                      k_wave=0.3), 2)],
                         ids=["weak-maxwellian", "strong-maxwellian", "two-stream"])
def test_set_init_variants_match_oracle(gpu_lib, case, kind):
    ctx = _ctx(gpu_lib, case, gpu_lib.PREC_FP64)
    ctx.set_init(kind, 2.0)
    U = Oracle(case, fixes=FIX_DEFAULT).set_init(kind, 2.0)
    assert rel(ctx.get_state(), U) < 1e-14
    ctx.close()


@pytest.fixture(scope="module")
def weak_oracle():
    """Oracle states (and E_x) of the weak-damping workload after 1, 5, 10 steps."""
    O = Oracle(WEAK, fixes=FIX_DEFAULT)
    U = O.set_init(1)
    out = {0: (U, None)}
    for s in range(1, 11):
        U = O.step(U)
        if s in (1, 5, 10):
            out[s] = (U.copy(), O.poisson(U)[1])
    return out


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)], ids=["fp64", "mixed"])
def test_weak_damping_steps(gpu_lib, weak_oracle, precision, tol):
    ctx = _ctx(gpu_lib, WEAK, precision)
    ctx.set_state(weak_oracle[0][0])
    done = 0
    for s in (1, 5, 10):
        ctx.step(s - done)
        done = s
        U, ex = weak_oracle[s]
        assert rel(ctx.get_state(), U) < tol, s
        assert rel(_ex(ctx), ex) < tol, s
    ctx.close()


@pytest.fixture(scope="module")
def strong_oracle():
    O = Oracle(STRONG, fixes=FIX_DEFAULT)
    U0 = O.set_init(1)
    U1 = O.step(U0)
    return U0, U1, O.poisson(U1)[1]


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)], ids=["fp64", "mixed"])
def test_strong_damping_full_step(gpu_lib, strong_oracle, precision, tol):
    U0, U1, ex1 = strong_oracle
    ctx = _ctx(gpu_lib, STRONG, precision)
    ctx.set_state(U0)
    ctx.step(1)
    assert rel(ctx.get_state(), U1) < tol
    assert rel(_ex(ctx), ex1) < tol
    ctx.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_strong_damping_collision_conserves(gpu_lib, precision):
    """Mass, the three momenta and kinetic energy through one collision step
    of all 64 cells, from the state after one advection step (so every cell
    carries a different, non-Maxwellian distribution)."""
    ctx = _ctx(gpu_lib, STRONG, precision)
    ctx.set_init(1)
    ctx.advect_step()
    m0 = ctx.moments()
    ctx.collision_step()
    m1 = ctx.moments()
    assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-12
    assert np.all(np.abs(m1[1:4] - m0[1:4]) / abs(m0[0]) < 1e-12)
    assert abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-12
    ctx.close()


TS_CELLS = (0, 1, 77, 200)


@pytest.fixture(scope="module")
def twostream_oracle():
    """The two-stream state and the oracle's collision of TS_CELLS, one cell
    at a time (nodes -> ComputeQ -> conserve -> RK4, slots {0,3,4,5,6})."""
    O = Oracle(TWOSTREAM, fixes=FIX_DEFAULT)
    U0 = O.set_init(2, 2.0)
    nv3 = TWOSTREAM.nv ** 3
    cells = {}
    for s in TS_CELLS:
        ucell = U0.reshape(TWOSTREAM.ncell, nv3 * 7)[s]
        f = O.nodes(U0, s)
        du = O.rk4(f, O.conserve(O.compute_q(f)), ucell).reshape(nv3, 5)
        new = ucell.reshape(nv3, 7).copy()
        new[:, [0, 3, 4, 5, 6]] = du
        cells[s] = new
    return U0, cells


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)], ids=["fp64", "mixed"])
def test_twostream_collision_cells(gpu_lib, twostream_oracle, precision, tol):
    U0, cells = twostream_oracle
    nv3 = TWOSTREAM.nv ** 3
    ctx = _ctx(gpu_lib, TWOSTREAM, precision)
    ctx.set_state(U0)
    for s in TS_CELLS:
        ctx.collision_step(s, s + 1)
    U = ctx.get_state().reshape(TWOSTREAM.ncell, nv3, 7)
    for s in TS_CELLS:
        assert rel(U[s], cells[s]) < tol, s
    # the other cells are untouched
    U0c = U0.reshape(TWOSTREAM.ncell, nv3, 7)
    assert np.array_equal(U[2], U0c[2]) and np.array_equal(U[255], U0c[255])
    ctx.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_landau_damping_rate(gpu_lib, precision):
    """Collisionless weak damping (nu = 0) on the GPU: the frequency and
    damping rate of |E| match linear theory for k = 0.5 (omega = 1.4156,
    gamma = -0.1533) with the field-integral fix F12."""
    case = Case(**{**WEAK.__dict__, "nu": 0.0})
    ctx = _ctx(gpu_lib, case, precision)
    ctx.set_init(1)
    ts, ee = [], []
    for s in range(0, 1001, 2):
        if s:
            ctx.step(2)
        ts.append(s * case.dt)
        ee.append(ctx.diagnostics()[5])
    omega, gamma, peaks = rate(ts, ee, t_max=10.0)
    assert len(peaks) >= 4
    assert abs(omega - OMEGA_K05) / OMEGA_K05 < 0.01, omega
    assert abs(gamma - GAMMA_K05) / abs(GAMMA_K05) < 0.06, gamma
    ctx.close()
