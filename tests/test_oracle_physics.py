"""Known answer of the collisionless path, independent of the reference's own
numbers: linear Landau damping at k = 0.5 (A = 0.01, unit Maxwellian,
Nx = 24, Nv = 16, v in [-5.25, 5.25]^3, dt = 0.01, nu = 0; the weak-damping
workload with collisions off) on the CPU oracle.

With the field-integral fix F12 the oracle's RK3 + LDG Poisson reproduce
linear theory (omega = 1.4156, gamma = -0.1533).  Without it -- the
reference's behaviour, source/PoissonFunctions.cpp:1435-1440 feeding
source/advection_1.cpp:184-192 -- the force is 1/dx too strong and the
plasma oscillates near omega = 1.70."""
from __future__ import annotations

import numpy as np

from landau_rate import GAMMA_K05, OMEGA_K05, rate
from oracle.oracle import Case, FIX_DEFAULT, FIX_F12, Oracle

CASE = dict(nx1=24, nx2=1, nv=16, n=16, lv=5.25, lx=4 * np.pi, nu=0.0, dt=0.01, a_amp=0.01,
            k_wave=0.5)


def _series(fixes, nsteps, every=2):
    O = Oracle(Case(**CASE), fixes=fixes)
    U = O.set_init(1)
    ts, ee = [], []
    for s in range(nsteps + 1):
        if s % every == 0:
            _, px, py, _ = O.poisson(U)
            ts.append(s * CASE["dt"])
            ee.append(O.moments(U, px, py)[5])
        U = O.rk3(U)
    return ts, ee


def test_landau_damping_rate_with_f12():
    ts, ee = _series(FIX_DEFAULT, 1000)
    omega, gamma, peaks = rate(ts, ee, t_max=10.0)
    assert len(peaks) >= 4
    assert abs(omega - OMEGA_K05) / OMEGA_K05 < 0.01, omega
    assert abs(gamma - GAMMA_K05) / abs(GAMMA_K05) < 0.06, gamma


def test_reference_field_scaling_shifts_frequency():
    ts, ee = _series(FIX_DEFAULT & ~FIX_F12, 600)
    omega, _, peaks = rate(ts, ee, t_max=6.0)
    assert len(peaks) >= 3
    assert 1.6 < omega < 1.8, omega


def test_dg_mass_matrix_of_the_collision_basis():
    """The collided DG coefficients of a velocity cell (slots 0, 3-6: 1,
    the three centred linears and |xi|^2 in cell units xi in [-1/2, 1/2]^3)
    have the mass matrix whose inverse the RK4 update applies
    (source/collisionRoutines_1.cpp:894-901: the moments tp0..tp5 enter as
    tp0 + U5/4 and U0/4 + 19 U5/240, and the new coefficients are
    19 tp0/4 - 15 tp5, 12 tp_i and 60 tp5 - 15 tp0).  Gauss-Legendre
    quadrature over the unit cell gives the matrix and its inverse."""
    x, w = np.polynomial.legendre.leggauss(4)
    x, w = x / 2, w / 2  # nodes and weights on [-1/2, 1/2]
    X1, X2, X3 = np.meshgrid(x, x, x, indexing="ij")
    W = np.einsum("i,j,k->ijk", w, w, w)
    basis = [np.ones_like(X1), X1, X2, X3, X1 ** 2 + X2 ** 2 + X3 ** 2]
    M = np.array([[np.sum(W * a * b) for b in basis] for a in basis])
    # the forward map the reference applies: moments from coefficients
    assert np.allclose(M[0], [1, 0, 0, 0, 1 / 4], atol=1e-15)
    assert np.allclose(M[4], [1 / 4, 0, 0, 0, 19 / 240], atol=1e-15)
    assert np.allclose(np.diag(M)[1:4], 1 / 12, atol=1e-15)
    Minv = np.linalg.inv(M)
    assert np.allclose(Minv[0, [0, 4]], [19 / 4, -15], atol=1e-12)
    assert np.allclose(Minv[4, [0, 4]], [-15, 60], atol=1e-12)
    assert np.allclose(np.diag(Minv)[1:4], 12, atol=1e-12)
    assert np.allclose(Minv[1:4, [0, 4]], 0, atol=1e-12)
