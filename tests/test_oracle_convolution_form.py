"""The factorisation behind the convolution form of ComputeQ, checked on the
CPU against the oracle's direct windowed sum (oracle/lp_oracle.c,
lpo_compute_q, after source/collisionRoutines_1.cpp:739-822).

The oracle's weight is W(xi, omega) = A(omega) - d^T Shat(omega) d
(A = ahat, or 0 where |omega| = 0; source/collisionRoutines_1.cpp:30-69),
with d = eta(xi) - eta(omega) = (u - h) h_eta on the uniform node grid and
u = xi + h - omega.  So the windowed sum over omega of
h_eta^3 wt wt wt W F(omega) F(u) is a sum of seven convolutions of
omega-factors with polynomials in u.  This model takes A and Shat from the
oracle's own tables, forms the seven pairs as the GPU kernels do, convolves
them with zero-padded FFTs in FP64 and compares with the oracle's sum.  It
checks the algebra and the index window that the mixed path's and the FP64
path's convolution kernels evaluate.  The two-species variant's linear term
factorises the same way (nine convolutions of F-independent omega-factors
with F times a polynomial in u, weighted by the output's node coordinate);
its model is checked against the oracle's linear term here too."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import Case, FIX_DEFAULT, Oracle

# on the oracle's own transform and tables the model's FFT sums and the
# oracle's direct sum differ only in the order of the same FP64 terms:
# measured 3.4e-15, 2.5e-15 and 1.2e-14 at n = 8, 16, 24
TOL = {8: 1e-13, 16: 1e-13, 24: 1e-13}


def convolution_model(O, case, f):
    n, h = case.n, case.n // 2
    v, eta, wt, _ = O.grids()
    h_eta = eta[1] - eta[0]
    ah, sh, rz = O.omega_tables()
    F = O.fft3d(f.astype(np.complex128)).reshape(n, n, n)
    cw = (h_eta ** 3) * wt[:, None, None] * wt[None, :, None] * wt[None, None, :]
    A = np.where(rz, 0.0, ah).reshape(n, n, n)
    S = sh.reshape(n, n, n, 6)
    d = (np.arange(n) - h) * h_eta  # the polynomial factor per axis, (u - h) h_eta
    du = [d[:, None, None], d[None, :, None], d[None, None, :]]
    # (S index, axes i, j, multiplicity) of -d^T Shat d
    terms = [(0, 0, 0, 1.0), (1, 0, 1, 2.0), (2, 0, 2, 2.0), (3, 1, 1, 1.0), (4, 1, 2, 2.0), (5, 2, 2, 1.0)]
    pairs = [(cw * A * F, F)]
    for s, i, j, mult in terms:
        pairs.append((-mult * cw * S[..., s] * F, du[i] * du[j] * F))
    # linear convolution (a * b)(xi + h) on [h, h + n)^3: FFTs of size 2n per axis
    shape = (2 * n,) * 3
    acc = np.zeros(shape, np.complex128)
    for a, b in pairs:
        acc += np.fft.fftn(a, shape, axes=(0, 1, 2)) * np.fft.fftn(b, shape, axes=(0, 1, 2))
    full = np.fft.ifftn(acc, axes=(0, 1, 2))
    return full[h:h + n, h:h + n, h:h + n].reshape(-1)


@pytest.mark.parametrize("n", [8, 16, 24])
def test_convolution_form_matches_direct_sum(n):
    case = Case(nx1=2, nx2=1, nv=4, n=n, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    O = Oracle(case, fixes=FIX_DEFAULT)
    v, _, _, _ = O.grids()
    V1, V2, V3 = np.meshgrid(v, v, v, indexing="ij")
    f = (np.exp(-((V1 - 0.7) ** 2 + V2 ** 2 + V3 ** 2) / 2)
         + 0.4 * np.exp(-((V1 + 1.2) ** 2 + (V2 - 0.3) ** 2 + 1.5 * V3 ** 2) / 2)).reshape(-1)
    q = O.compute_q(f)
    qm = convolution_model(O, case, f)
    err = np.linalg.norm(qm - q) / np.linalg.norm(q)
    assert err < TOL[n], err


def test_weight_is_the_quadratic_form():
    """W(xi, omega) from the oracle equals A(omega) - d^T Shat(omega) d with
    d = (xi - omega) h_eta per axis, at every omega and a spread of xi."""
    case = Case(nx1=2, nx2=1, nv=4, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    O = Oracle(case, fixes=FIX_DEFAULT)
    n = case.n
    _, eta, _, _ = O.grids()
    h_eta = eta[1] - eta[0]
    ah, sh, rz = O.omega_tables()
    rng = np.random.default_rng(7)
    for om in range(n ** 3):
        l, m, q = om // (n * n), (om // n) % n, om % n
        for xi in rng.integers(0, n ** 3, 4):
            i, j, k = xi // (n * n), (xi // n) % n, xi % n
            dv = np.array([i - l, j - m, k - q]) * h_eta
            s = sh[om]
            Sm = np.array([[s[0], s[1], s[2]], [s[1], s[3], s[4]], [s[2], s[4], s[5]]])
            w = (0.0 if rz[om] else ah[om]) - dv @ Sm @ dv
            assert abs(O.weight(xi, om) - w) <= 1e-12 * (abs(ah[om]) + np.abs(Sm).sum() * (dv @ dv) + 1e-300)


@pytest.mark.parametrize("n,bound", [(8, 1e-14), (16, 1e-13), (24, 1e-12)])
def test_sensitivity_to_the_transform(n, bound):
    """ComputeQ carries an absolute error of the transform into its small
    outputs: a perturbation of 1e-16 max|F| in every mode of the oracle's own
    F (about one rounding of a DFT of it) moves the result by 3.0e-15,
    3.7e-14 and 1.7e-13 (relative L2) at n = 8, 16, 24, while |F| spans 17
    to 19 decades.  Two FP64 transforms of f that round differently (the
    GPU's and the oracle's) therefore give ComputeQ results that differ by
    this much whatever form sums them."""
    case = Case(nx1=2, nx2=1, nv=4, n=n, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    O = Oracle(case, fixes=FIX_DEFAULT)
    v, _, _, _ = O.grids()
    V1, V2, V3 = np.meshgrid(v, v, v, indexing="ij")
    f = (np.exp(-((V1 - 0.7) ** 2 + V2 ** 2 + V3 ** 2) / 2)
         + 0.4 * np.exp(-((V1 + 1.2) ** 2 + (V2 - 0.3) ** 2 + 1.5 * V3 ** 2) / 2)).reshape(-1)
    q0 = convolution_model(O, case, f)
    exact = O.fft3d
    rng = np.random.default_rng(1)

    def perturbed(x):
        F = exact(x)
        s = 1e-16 * np.abs(F).max()
        return F + s * (rng.standard_normal(F.shape) + 1j * rng.standard_normal(F.shape))

    O.fft3d = perturbed
    q1 = convolution_model(O, case, f)
    err = np.linalg.norm(q1 - q0) / np.linalg.norm(q0)
    assert bound / 30 < err < bound, err



def linear_term_model(O, case, f):
    """The two-species variant's linear term (lpo_compute_q_lin, after
    source/collisionRoutines_1.cpp:551-635 with the weight of :71-96):
    sum over omega of h_eta^3 wt wt wt scale3 Wlin(xi, omega) F(u) with
    Wlin = -sum_ij Shat_ij(omega) eta(xi)_i (eta(xi)_j - eta(omega)_j).
    With eta(xi)_j - eta(omega)_j = (u_j - h) h_eta it is
    -scale3 sum_i eta(xi)_i sum_j (A_ij * B_j)(xi + h): nine convolutions of
    the F-independent A_ij = cw Shat_ij with B_j = (u_j - h) h_eta F."""
    n, h = case.n, case.n // 2
    _, eta, wt, sc = O.grids()
    h_eta, s3 = sc[1], sc[6]
    _, sh, _ = O.omega_tables()
    F = O.fft3d(f.astype(np.complex128)).reshape(n, n, n)
    cw = (h_eta ** 3) * wt[:, None, None] * wt[None, :, None] * wt[None, None, :]
    S = sh.reshape(n, n, n, 6)
    sidx = [[0, 1, 2], [1, 3, 4], [2, 4, 5]]
    d = (np.arange(n) - h) * h_eta
    du = [d[:, None, None], d[None, :, None], d[None, None, :]]
    ez = [eta[:, None, None], eta[None, :, None], eta[None, None, :]]
    shape, ax = (2 * n,) * 3, (0, 1, 2)
    Bh = [np.fft.fftn(du[j] * F, shape, axes=ax) for j in range(3)]
    out = np.zeros((n, n, n), np.complex128)
    for i in range(3):
        acc = sum(np.fft.fftn(cw * S[..., sidx[i][j]], shape, axes=ax) * Bh[j] for j in range(3))
        out += ez[i] * np.fft.ifftn(acc, axes=ax)[h:h + n, h:h + n, h:h + n]
    return (-s3 * out).reshape(-1)


@pytest.mark.parametrize("n", [8, 16, 24])
def test_linear_term_as_convolutions(n):
    case = Case(nx1=2, nx2=1, nv=4, n=n, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    O = Oracle(case, fixes=FIX_DEFAULT)
    v, _, _, _ = O.grids()
    V1, V2, V3 = np.meshgrid(v, v, v, indexing="ij")
    f = (np.exp(-((V1 - 0.7) ** 2 + V2 ** 2 + V3 ** 2) / 2)
         + 0.4 * np.exp(-((V1 + 1.2) ** 2 + (V2 - 0.3) ** 2 + 1.5 * V3 ** 2) / 2)).reshape(-1)
    _, ql = O.compute_q_lin(f)
    qm = linear_term_model(O, case, f)
    err = np.linalg.norm(qm - ql) / np.linalg.norm(ql)
    assert err < 1e-13, err
