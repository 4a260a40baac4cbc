"""The CPU oracle against the golden vectors of the reference's own routines
(tests/golden/make_golden.py).  Bit-exact where the oracle keeps the
reference's operation order; reductions whose order the reference leaves to
OpenMP are compared at 1e-14."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN_NAMES, golden_case, load_golden, rel
from oracle.oracle import Oracle


@pytest.fixture(scope="module", params=GOLDEN_NAMES)
def gold(request):
    g = load_golden(request.param)
    return g, Oracle(golden_case(g), fixes=0)


def test_grids_and_tables(gold):
    g, O = gold
    v, eta, wt, sc = O.grids()
    assert np.array_equal(v, g["v"]) and np.array_equal(eta, g["eta"]) and np.array_equal(wt, g["wt"])
    assert np.array_equal(sc[:13], g["scalars"][:13])
    c1, c2, cct = O.cons()
    assert np.array_equal(c1[[0, 4]], g["c1_rows"])
    assert np.array_equal(c2[[1, 2, 3]], g["c2_rows"])
    assert rel(cct, g["cct_inv"]) < 1e-14


def test_weight_rows(gold):
    g, O = gold
    n3 = O.n3
    for r, row in zip(g["w_rows"], g["w_vals"]):
        mine = np.array([O.weight(int(r), o) for o in range(n3)])
        assert np.array_equal(mine, row)


def test_transforms(gold):
    g, O = gold
    assert np.array_equal(O.fft3d(g["fft_in"]), g["fft_out"])
    assert np.array_equal(O.fs(g["fft_in"]), g["fs_out"])


def test_initial_state_and_nodes(gold):
    g, O = gold
    assert np.array_equal(O.set_init(0), g["U_init"])
    nx1 = O.case.nx1
    nodes = np.stack([O.nodes(g["U_nodes"], i) for i in range(nx1)])
    assert np.array_equal(nodes, g["nodes"])


def test_compute_q_conserve(gold):
    g, O = gold
    q = O.compute_q(g["f_cell"])
    assert np.array_equal(q, g["qhat"])
    assert rel(O.conserve(g["qhat"]), g["qhat_cons"]) < 1e-14


def test_intmodes(gold):
    g, O = gold
    for idx, val in zip(g["im_idx"], g["im_vals"]):
        assert np.array_equal(O.intmodes(*map(int, idx)), val)


def test_rk4_zero_state(gold):
    g, O = gold
    cell = int(g["rk4_cell"])
    ucell = np.zeros(O.nv3 * 7)
    du = O.rk4(g["f_cell"], g["qhat_cons"], ucell, direct=True)
    assert rel(du, g["rk4_du"]) < 1e-13
    du_sep = O.rk4(g["f_cell"], g["qhat_cons"], ucell, direct=False)
    assert rel(du_sep, g["rk4_du"]) < 1e-12
    assert cell >= 0


def test_poisson(gold):
    g, O = gold
    potc, px, py, fl = O.poisson(g["U_init"])
    assert np.array_equal(potc, g["pois_potc"])
    assert np.array_equal(px, g["pois_phix"])
    assert np.array_equal(py, g["pois_phiy"])
    assert np.array_equal(fl, g["pois_fields"])
    dims, ab, piv = O.band()
    assert np.array_equal(dims, g["band_dims"])
    assert np.array_equal(ab, g["band_ab"]) and np.array_equal(piv, g["band_piv"])


def test_rk3(gold):
    g, O = gold
    assert np.array_equal(O.rk3(g["rk3_in"]), g["rk3_out"])


def test_collision_driver_verbatim(gold):
    g, O = gold
    nx1, nv3 = O.case.nx1, O.nv3
    U = O.collide(g["coll_in"], direct=True)
    du = U.reshape(-1, 7)[: nx1 * nv3][:, [0, 3, 4, 5, 6]].ravel()
    assert rel(du, g["coll_du"]) < 1e-13


def test_moments(gold):
    g, O = gold
    m = O.moments(g["rk3_out"], g["moments_phix"], g["moments_phiy"])
    # the reference reduces these sums in OpenMP order; the momentum sums cancel
    assert np.allclose(m, g["moments"], rtol=1e-13, atol=1e-14 * abs(g["moments"][0]))


def test_entropy(gold):
    g, O = gold
    # int f log f over the first nx1 spatial cells (the reference's i < Nx),
    # summed in OpenMP order by the reference
    e = O.entropy(g["rk3_out"])
    assert abs(e - float(g["entropy"])) <= 1e-13 * abs(float(g["entropy"]))


def test_marginal_x1v1(gold):
    g, O = gold
    m = O.marginal_x1v1(g["rk3_out"])
    assert np.array_equal(m.ravel(), g["marginal_x1v1"].ravel())
