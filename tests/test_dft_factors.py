"""The factored form of the per-axis transforms that the mixed path's
register FFTs use (CPU): each per-axis matrix of fft3D and FS is
post[a] w^((a i) mod n) pre[i] with w = exp(-+2 pi i / n), pre the input
phase and trapezoid weight, post the output phase.  The factored 3-D
transforms are checked against the oracle's fft3D and FS, and the
Cooley-Tukey plan of the register FFT (radix 2, 3, 4, 8 stages, twiddles
r^((a1 i2) mod N), outputs a1 + N1 a2) against numpy's DFT."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import Case, FIX_DEFAULT, Oracle


def _factors(O, n):
    v, eta, wt, sc = O.grids()
    L_eta, h_eta, h_v, L_v, scale = sc[0], sc[1], sc[2], sc[3], sc[5]
    i = np.arange(n)
    pre_f = scale * h_v * wt * np.exp(1j * i * L_eta * h_v)
    post_f = np.exp(1j * L_v * eta)
    inv_s = 1.0 / (2.0 * L_v * scale)
    pre_i = inv_s * np.exp(-1j * i * L_v * h_eta)
    post_i = np.exp(-1j * L_eta * v)
    core = np.outer(i, i) % n
    A_f = post_f[:, None] * np.exp(-2j * np.pi * core / n) * pre_f[None, :]
    A_i = post_i[:, None] * np.exp(2j * np.pi * core / n) * pre_i[None, :]
    return A_f, A_i


def _apply3(A, x, n):
    x = x.reshape(n, n, n)
    return np.einsum("al,bm,cq,lmq->abc", A, A, A, x).reshape(-1)


@pytest.mark.parametrize("n", [8, 16, 24, 32])
def test_factored_transforms_match_oracle(n):
    case = Case(nx1=2, nx2=1, nv=4, n=n, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    O = Oracle(case, fixes=FIX_DEFAULT)
    A_f, A_i = _factors(O, n)
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n ** 3) + 1j * rng.standard_normal(n ** 3)
    ref = O.fft3d(x)
    got = _apply3(A_f, x, n)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)
    ref = O.fs(x)  # the full complex inverse (the stages keep its real part)
    got = _apply3(A_i, x, n)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)


PLANS = {8: (8, 1), 16: (4, 4), 24: (3, 8), 32: (4, 8)}


def _small_dft(v, S):
    K = len(v)
    k = np.arange(K)
    return np.exp(S * 2j * np.pi * np.outer(k, k) / K) @ v


def _fft_plan(x, S):
    """Restatement of the register FFT's index plan: N1-point DFTs over the
    inputs N2 i1 + i2, twiddles r^((a1 i2) mod N), N2-point DFTs, output
    a1 + N1 a2 (the small DFTs in closed form on the device)."""
    N = len(x)
    N1, N2 = PLANS[N]
    if N2 == 1:
        return _small_dft(x, S)
    w = np.exp(S * 2j * np.pi * np.arange(N) / N)
    z = np.zeros((N1, N2), complex)
    for i2 in range(N2):
        v = _small_dft(x[i2::N2][:N1], S)
        for a1 in range(N1):
            z[a1, i2] = v[a1] * w[(a1 * i2) % N]
    out = np.zeros(N, complex)
    for a1 in range(N1):
        y = _small_dft(z[a1], S)
        for a2 in range(N2):
            out[a1 + N1 * a2] = y[a2]
    return out


@pytest.mark.parametrize("n", [8, 16, 24, 32])
@pytest.mark.parametrize("S", [-1, 1])
def test_fft_plan(n, S):
    rng = np.random.default_rng(100 + n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x) if S < 0 else np.fft.ifft(x) * n
    assert np.allclose(_fft_plan(x, S), ref, rtol=0, atol=1e-12 * np.abs(ref).max())
