"""GPU path (through the C ABI) against the golden vectors of the reference's
own routines, routine by routine, with the reference's defects F1-F3 left in
(fixes=0) so the verbatim outputs apply.  FP64 tolerances: 1e-12 relative L2
(the GPU contracts to FMA and reduces in its own order)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN_NAMES, golden_case, load_golden, rel

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module", params=GOLDEN_NAMES)
def gctx(request, gpu_lib):
    g = load_golden(request.param)
    c = golden_case(g)
    P = gpu_lib.Params(nx1=c.nx1, nx2=c.nx2, nv=c.nv, n=c.n, lv=c.lv, lx=c.lx, nu=c.nu, dt=c.dt,
                       a_amp=c.a_amp, k_wave=c.k_wave, fixes=0, precision=gpu_lib.PREC_FP64)
    ctx = gpu_lib.Context(P)
    yield g, ctx
    ctx.close()


def test_tables(gctx):
    g, ctx = gctx
    c1, c2, cct = ctx.conservation_rows()
    assert np.array_equal(c1[[0, 4]], g["c1_rows"]) and np.array_equal(c2[[1, 2, 3]], g["c2_rows"])
    assert rel(cct, g["cct_inv"]) < 1e-14
    for r, row in zip(g["w_rows"], g["w_vals"]):
        assert np.array_equal(ctx.weights_rows(int(r), int(r) + 1)[0], row)


def test_fft3d_fs(gctx):
    g, ctx = gctx
    assert rel(ctx.fft3d(g["fft_in"]), g["fft_out"]) < 1e-13
    assert rel(ctx.fs(g["fft_in"]), g["fs_out"]) < 1e-13


def test_nodes(gctx):
    g, ctx = gctx
    ctx.set_state(g["U_nodes"])
    f = ctx.nodes(ncollide=int(g["case"][0]))
    assert rel(f, g["nodes"]) < 1e-14


def test_compute_q(gctx):
    g, ctx = gctx
    assert rel(ctx.compute_q(g["f_cell"]), g["qhat"]) < TOL


def test_conserve(gctx):
    g, ctx = gctx
    assert rel(ctx.conserve(g["qhat"]), g["qhat_cons"]) < TOL


def test_rk4_zero_state(gctx):
    g, ctx = gctx
    ctx.set_state(np.zeros_like(g["U_init"]))
    du = ctx.rk4_cell(g["f_cell"], int(g["rk4_cell"]), g["qhat_cons"])
    assert rel(du, g["rk4_du"]) < TOL


def test_poisson(gctx):
    g, ctx = gctx
    ctx.set_state(g["U_init"])
    potc, px, py, fl = ctx.poisson()
    assert rel(potc, g["pois_potc"]) < TOL
    assert rel(px, g["pois_phix"]) < TOL
    # E_y of an x2-independent state is rounding noise; compare on the E_x scale
    scale = np.linalg.norm(g["pois_phix"])
    assert np.linalg.norm(py - g["pois_phiy"]) / scale < TOL
    assert rel(fl[:6], g["pois_fields"][:6]) < TOL
    assert np.linalg.norm(fl[6:12] - g["pois_fields"][6:12]) / scale < TOL


def test_rk3(gctx):
    g, ctx = gctx
    ctx.set_state(g["rk3_in"])
    ctx.advect_step()
    assert rel(ctx.get_state(), g["rk3_out"]) < TOL


def test_collision_verbatim(gctx):
    g, ctx = gctx
    nx1, nv = int(g["case"][0]), int(g["case"][2])
    ctx.set_state(g["coll_in"])
    ctx.collision_step()
    U = ctx.get_state().reshape(-1, 7)[: nx1 * nv ** 3]
    assert rel(U[:, [0, 3, 4, 5, 6]].ravel(), g["coll_du"]) < TOL


def test_moments(gctx):
    g, ctx = gctx
    ctx.set_state(g["rk3_out"])
    m = ctx.moments()
    assert np.allclose(m[:5], g["moments"][:5], rtol=1e-13, atol=1e-14 * abs(g["moments"][0]))


# At the strong-damping workload's velocity grid (Nv = N = 24, v in [-6, 6]^3;
# fixture ref_nv24): ComputeQ, the projection, RK4 from the zero state and
# the verbatim collision driver of the two collided cells of a 2 x 2 grid.
# Defect F11 is present at this grid (eta[n/2] != 0) and the verbatim step
# blows the state up by ~1e10, which amplifies rounding ~2e3-fold (a 1e-16
# relative change of the node values moves RK4's output by ~2e-13,
# tests/test_oracle_golden_nv24.py); the GPU sums in its own order, so RK4 and
# the collision driver are held to TOL_F11.  ComputeQ and the projection
# precede the growth and keep TOL.  The F11-fixed step at this grid is
# compared with the oracle at 1e-12 in tests/test_gpu_configs.py.
TOL_F11 = 1e-10
@pytest.fixture(scope="module")
def gctx24(gpu_lib):
    g = load_golden("ref_nv24")
    c = golden_case(g)
    P = gpu_lib.Params(nx1=c.nx1, nx2=c.nx2, nv=c.nv, n=c.n, lv=c.lv, lx=c.lx, nu=c.nu, dt=c.dt,
                       a_amp=c.a_amp, k_wave=c.k_wave, fixes=0, precision=gpu_lib.PREC_FP64)
    ctx = gpu_lib.Context(P)
    yield g, c, ctx
    ctx.close()


def test_compute_q_conserve_nv24(gctx24):
    g, _, ctx = gctx24
    assert rel(ctx.compute_q(g["f_cell"]), g["qhat"]) < TOL
    assert rel(ctx.conserve(g["qhat"]), g["qhat_cons"]) < TOL


def test_rk4_zero_state_nv24(gctx24):
    g, c, ctx = gctx24
    ctx.set_state(np.zeros(c.size * 7))
    du = ctx.rk4_cell(g["f_cell"], int(g["rk4_cell"]), g["qhat_cons"])
    assert rel(du, g["rk4_du"]) < TOL_F11


def test_collision_verbatim_nv24(gctx24):
    from oracle.oracle import Oracle
    g, c, ctx = gctx24
    ctx.set_state(Oracle(c, fixes=0).set_init(0))  # SetInit_LD, pinned by the fixture's hash
    ctx.collision_step()
    U = ctx.get_state().reshape(-1, 7)[: c.nx1 * c.nv ** 3]
    assert rel(U[:, [0, 3, 4, 5, 6]].ravel(), g["coll_du"]) < TOL_F11
