"""The oracle's two-species variant (the reference's FullandLinear switch)
against golden vectors from the reference built with that switch: linear
weight rows, CCt_linear and ComputeQ bit for bit, the two conservations and
RK4 within OpenMP reduction-order rounding."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_case, load_golden, rel
from oracle.oracle import FIX_F1, Oracle


@pytest.fixture(scope="module")
def lin():
    g = load_golden("ref_lin_n8")
    case = golden_case(g)
    case.linear_ei = 1
    return g, Oracle(case, fixes=0)


def test_weights_lin(lin):
    g, O = lin
    for r, row in zip(g["wl_rows"], g["wl_vals"]):
        got = np.array([O.weight_lin(int(r), o) for o in range(row.size)])
        assert np.array_equal(got, row)


def test_cct_lin(lin):
    g, O = lin
    assert np.array_equal(O.cct_lin(), g["cct_lin"])


def test_compute_q_lin(lin):
    g, O = lin
    q, ql = O.compute_q_lin(g["f_cell"])
    assert np.array_equal(q, g["qhat"]) and np.array_equal(ql, g["qhat_lin"])


def test_conserve_lin(lin):
    g, O = lin
    q, ql = O.conserve_lin(g["qhat"], g["qhat_lin"])
    assert rel(q, g["qhat_cons"]) < 1e-13 and rel(ql, g["qlin_cons"]) < 1e-13


def test_rk4_lin(lin):
    g, _ = lin
    case = golden_case(g)
    case.linear_ei = 1
    O = Oracle(case, fixes=FIX_F1)
    nv3 = case.nv ** 3
    U = np.zeros(case.size * 7)
    U[7 * nv3:14 * nv3] = g["rk4_cell_state"]
    du = O.rk4_lin(g["f_cell"], g["qhat_cons"], g["qlin_cons"], U, 1)
    assert rel(du, g["rk4_du"]) < 1e-13
