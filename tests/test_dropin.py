"""The C++ drop-in layer (reference routine names and signatures over the C
ABI), driven by a reference-style program that defines the reference's
globals, against the CPU oracle with the reference's behaviour (fixes = 0)."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import PKG, rel
from oracle.oracle import Case, Oracle

pytestmark = pytest.mark.gpu


def _read(path):
    out = {}
    with open(path, "rb") as fh:
        while True:
            nm = fh.read(16)
            if not nm:
                break
            cnt = int(np.frombuffer(fh.read(8), np.int64)[0])
            out[nm.rstrip(b"\0").decode()] = np.frombuffer(fh.read(8 * cnt), np.float64).copy()
    return out


def test_dropin_routines(gpu_lib, tmp_path):
    driver = os.path.join(PKG, "_build", "dropin_driver")
    assert os.path.exists(driver), "the drop-in driver was not built"
    case = Case(nx1=3, nx2=3, nv=6, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.005, a_amp=0.5, k_wave=0.5)
    O = Oracle(case, fixes=0)
    rng = np.random.default_rng(20261203)
    U = O.set_init(0)
    U = U + 1e-3 * np.abs(U).max() * rng.standard_normal(U.shape)
    f = O.nodes(U, 1)
    qin = O.compute_q(f)
    x = rng.standard_normal(case.n ** 3) + 1j * rng.standard_normal(case.n ** 3)
    inp = tmp_path / "in.bin"
    outp = tmp_path / "out.bin"
    with open(inp, "wb") as fh:
        for a in (U, f, qin.view(np.float64), x.view(np.float64)):
            fh.write(np.ascontiguousarray(a, np.float64).tobytes())
    subprocess.run([driver, str(inp), str(outp), str(case.nx1), str(case.nv), str(case.n), repr(case.lv),
                    repr(case.lx), repr(case.nu), repr(case.dt), repr(case.a_amp), repr(case.k_wave)],
                   check=True, timeout=300)
    r = _read(outp)
    n3 = case.n ** 3
    c1, c2, cct = O.cons()
    assert np.array_equal(r["c1_0"], c1[0]) and np.array_equal(r["c1_4"], c1[4]) and np.array_equal(r["c2_1"], c2[1])
    assert rel(r["cct"], cct.ravel()) < 1e-14
    assert np.array_equal(r["w_mid"], np.array([O.weight(n3 // 2, o) for o in range(n3)]))
    assert rel(r["fft3d"].view(np.complex128), O.fft3d(x)) < 1e-13
    assert rel(r["fs"].view(np.complex128), O.fs(x)) < 1e-13
    assert rel(r["computeq"].view(np.complex128), qin) < 1e-12
    qc = O.conserve(qin)
    assert rel(r["conserve"].view(np.complex128), qc) < 1e-12
    du = O.rk4(f, qc, np.zeros(O.nv3 * 7), direct=False)
    assert rel(r["rk4"], du) < 1e-12
    nodes = np.stack([O.nodes(U, i) for i in range(case.nx1)])
    assert rel(r["nodes"], nodes.ravel()) < 1e-14
    potc, px, py, fl = O.poisson(U)
    assert rel(r["potc"], potc) < 1e-12 and rel(r["phix"], px) < 1e-12
    assert rel(r["ie_x"], fl[0]) < 1e-12
    assert rel(r["rk3"], O.rk3(U)) < 1e-12
    assert rel(r["collide"], O.collide(U, direct=False)) < 1e-12
