"""Generates the golden vectors in tests/golden/*.npz from the reference's own
routines, compiled from the reference checkout by oracle/build_ref.sh (this
script runs only where that checkout exists; the fixtures it writes are
committed and travel everywhere).

Each fixture holds seeded inputs and the reference outputs of: grids, the
conservation rows and inverse Gram matrix, rows of the weight table, fft3D,
FS, SetInit_LD, setInit_spectral, ComputeQ, conserveAllMoments, IntModes,
RK4 (zero state, so the stride defect F1 does not enter), pois2d, the band
factors, one RK3 step, the verbatim collision driver and the moments.

The fixture ref_nv24 runs the reference at the strong-damping workload's
velocity grid (Nv = N = 24, Lv = 6) on a 2 x 2 spatial grid: ComputeQ,
conserveAllMoments, RK4 from the zero state and the verbatim collision driver
of its two collided cells, from the SetInit_LD state (stored as a SHA-256 of
its bytes: the oracle's and the library's initial states are compared bit for
bit with the other fixtures' U_init, and the hash pins this one too).

The two-species fixture (ref_lin_n8) comes from the reference compiled with
its FullandLinear switch: the linear weight rows, CCt_linear, ComputeQ with
its linear part, the two conservations and RK4 (state with equal stride-6 and
stride-7 slots, so the slot defect F1 reads the same values either way).

    python tests/golden/make_golden.py [fixture names]   # default: all
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Case, Reference  # noqa: E402

SEED = 20261203

# (name, case): small 2-D cases the reference can run (nx1 = nx2 <= 49).
CASES = [
    ("ref_n8", Case(nx1=3, nx2=3, nv=6, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.005,
                    a_amp=0.5, k_wave=0.5)),
    ("ref_n16", Case(nx1=2, nx2=2, nv=4, n=16, lv=5.25, lx=4 * np.pi, nu=0.01, dt=0.01,
                     a_amp=0.01, k_wave=0.5)),
    ("ref_n24", Case(nx1=2, nx2=2, nv=4, n=24, lv=6.0, lx=4 * np.pi, nu=0.05, dt=0.005,
                     a_amp=0.5, k_wave=0.5)),
]


def make(name, case, rng):
    R = Reference(case, with_weights=True)
    n, nv, n3, nv3 = case.n, case.nv, case.n ** 3, case.nv ** 3
    out = {"case": np.array([case.nx1, case.nx2, case.nv, case.n], np.int64),
           "case_f": np.array([case.lv, case.lx, case.nu, case.dt, case.a_amp, case.k_wave])}
    v, eta, wt, sc = R.grids()
    out.update(v=v, eta=eta, wt=wt, scalars=sc)
    c1, c2, cct = R.cons()
    out.update(c1_rows=c1[[0, 4]], c2_rows=c2[[1, 2, 3]], cct_inv=cct)
    rows = np.sort(rng.choice(n3, 6, replace=False))
    out.update(w_rows=rows, w_vals=np.stack([R.weights(int(r), int(r) + 1)[0] for r in rows]))
    x = rng.standard_normal(n3) + 1j * rng.standard_normal(n3)
    out.update(fft_in=x, fft_out=R.fft3d(x), fs_out=R.fs(x))
    U = R.set_init_ld()
    out.update(U_init=U)
    # node sampling with slot 2 == slot 3 so that defect F2 does not enter
    U2 = U.copy().reshape(-1, 7)
    U2[:, 2] = U2[:, 3]
    U2 = U2.ravel()
    fnodes = R.set_init_spectral(U2)
    out.update(U_nodes=U2, nodes=fnodes)
    f = fnodes[1].copy()
    q = R.compute_q(f)
    qc = R.conserve(q)
    out.update(f_cell=f, qhat=q, qhat_cons=qc)
    picks = rng.integers(0, [n, n, n, nv, nv, nv], size=(8, 6))
    out.update(im_idx=picks, im_vals=np.stack([R.intmodes(*map(int, p)) for p in picks]))
    Uz = np.zeros_like(U)
    out.update(rk4_cell=np.int64(1), rk4_du=R.rk4(f, 1, qc, Uz))
    potc, px, py, fl = R.pois2d(U)
    out.update(pois_potc=potc, pois_phix=px, pois_phiy=py, pois_fields=fl)
    dims, ab, piv = R.band()
    out.update(band_dims=dims, band_ab=ab, band_piv=piv)
    Up = U + 1e-3 * rng.standard_normal(U.shape) * np.abs(U).max()
    U3, p3, x3, y3 = R.rk3(Up)
    out.update(rk3_in=Up, rk3_out=U3)
    out.update(coll_in=Up, coll_du=R.collision_cells(Up, 0, case.nx1))
    out.update(moments=R.moments(U3, x3, y3), moments_phix=x3, moments_phiy=y3)
    out.update(entropy=np.float64(R.entropy(U3)), marginal_x1v1=R.marginal_x1v1(U3))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KiB")


def make_rng_skip(case, rng):
    """The draws make() takes from the seeded stream, without the reference."""
    n, nv, n3 = case.n, case.nv, case.n ** 3
    rng.choice(n3, 6, replace=False)
    rng.standard_normal(n3), rng.standard_normal(n3)
    rng.integers(0, [n, n, n, nv, nv, nv], size=(8, 6))
    rng.standard_normal(case.size * 7)


LIN_CASE = ("ref_lin_n8", Case(nx1=2, nx2=2, nv=4, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01,
                                a_amp=0.2, k_wave=0.5, linear_ei=1))


def make_lin(name, case, rng):
    R = Reference(case, with_weights=True)
    n3 = case.n ** 3
    out = {"case": np.array([case.nx1, case.nx2, case.nv, case.n], np.int64),
           "case_f": np.array([case.lv, case.lx, case.nu, case.dt, case.a_amp, case.k_wave])}
    rows = np.sort(rng.choice(n3, 6, replace=False))
    out.update(wl_rows=rows, wl_vals=np.stack([R.weights_lin(int(r), int(r) + 1)[0] for r in rows]))
    out.update(cct_lin=R.cct_lin())
    U = R.set_init_ld()
    U2 = U.copy().reshape(-1, 7)
    U2[:, 2] = U2[:, 3]
    U2 = U2.ravel()
    f = R.set_init_spectral(U2)[1].copy()
    q, ql = R.compute_q_lin(f)
    qc, qlc = R.conserve_lin(q, ql)
    out.update(f_cell=f, qhat=q, qhat_lin=ql, qhat_cons=qc, qlin_cons=qlc)
    # a state whose stride-6 reads of cell 1 see the stride-7 slots {0,3,4,5,6}
    nv3 = case.nv ** 3
    Us = np.zeros_like(U)
    src = U.reshape(-1, 7)[nv3:2 * nv3]
    for kt in range(nv3):
        k = nv3 + kt
        Us[6 * k + 0], Us[6 * k + 2], Us[6 * k + 3] = src[kt, 0], src[kt, 3], src[kt, 4]
        Us[6 * k + 4], Us[6 * k + 5] = src[kt, 5], src[kt, 6]
    out.update(rk4_state=Us, rk4_cell_state=src.ravel(), rk4_du=R.rk4_lin(f, 1, qc, qlc, Us))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KiB")


NV24_CASE = ("ref_nv24", Case(nx1=2, nx2=2, nv=24, n=24, lv=6.0, lx=4 * np.pi, nu=0.05, dt=0.005,
                              a_amp=0.5, k_wave=0.5))


def make_nv24(name, case):
    """About two minutes of the reference's CPU time (RK4's IntModes calls
    and two collided cells dominate)."""
    R = Reference(case, with_weights=True)
    out = {"case": np.array([case.nx1, case.nx2, case.nv, case.n], np.int64),
           "case_f": np.array([case.lv, case.lx, case.nu, case.dt, case.a_amp, case.k_wave])}
    U = R.set_init_ld()
    out.update(U_init_sha256=np.frombuffer(hashlib.sha256(U.tobytes()).digest(), np.uint8))
    U2 = U.copy().reshape(-1, 7)
    U2[:, 2] = U2[:, 3]  # node sampling without defect F2, as in the other fixtures
    f = R.set_init_spectral(U2.ravel())[1].copy()
    q = R.compute_q(f)
    qc = R.conserve(q)
    out.update(f_cell=f, qhat=q, qhat_cons=qc)
    out.update(rk4_cell=np.int64(1), rk4_du=R.rk4(f, 1, qc, np.zeros_like(U)))
    out.update(coll_du=R.collision_cells(U, 0, case.nx1))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KiB")


def main(names=None):
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    want = lambda nm: not names or nm in names  # noqa: E731
    rng = np.random.default_rng(SEED)
    for name, case in CASES:
        if want(name):
            make(name, case, rng)
        else:  # keep the seeded stream of the later fixtures
            make_rng_skip(case, rng)
    if want(LIN_CASE[0]):
        make_lin(*LIN_CASE, np.random.default_rng(SEED + 1))
    if want(NV24_CASE[0]):
        make_nv24(*NV24_CASE)


if __name__ == "__main__":
    main(sys.argv[1:])
