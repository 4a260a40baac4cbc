"""The axis-3 DG projection pass on the tensor cores (tcgen05.mma, TF32
operands split into head and tail) against the CUDA-core pass it replaces
(LP_PJ3_TC=0 at context creation) and against the FP64 path: one mixed
collision step at n = 16 and n = 24 with 64, 128 and 96 cells per pass (the
128-row tiles hold two pencils, one pencil, or a pencil and a part), the
state within 1e-9 of the CUDA-core pass and 1e-6 of FP64, mass, momentum and
energy kept to 1e-12."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import rel
from oracle.oracle import FIX_DEFAULT

pytestmark = pytest.mark.gpu


def _ctx(lp, kw, precision, tc):
    old = os.environ.get("LP_PJ3_TC")
    os.environ["LP_PJ3_TC"] = "1" if tc else "0"
    try:
        return lp.Context(lp.Params(**kw, fixes=FIX_DEFAULT, precision=precision))
    finally:
        if old is None:
            del os.environ["LP_PJ3_TC"]
        else:
            os.environ["LP_PJ3_TC"] = old


@pytest.mark.parametrize("nx1,nv,n", [(64, 24, 24), (128, 16, 16), (40, 8, 16), (80, 8, 16)],
                         ids=["n24-64cells", "n16-128cells", "n16-nv8-40cells", "n16-nv8-80cells"])
def test_tc_projection_collision_step(gpu_lib, nx1, nv, n):
    lp = gpu_lib
    kw = dict(nx1=nx1, nx2=1, nv=nv, n=n, lv=6.0, lx=4 * np.pi, nu=0.05, dt=0.005, a_amp=0.5, k_wave=0.5)
    out = {}
    for name, prec, tc in (("tc", lp.PREC_MIXED, True), ("cuda", lp.PREC_MIXED, False), ("fp64", lp.PREC_FP64, False)):
        c = _ctx(lp, kw, prec, tc)
        c.set_init(1)
        c.advect_step()
        m0 = c.moments()
        c.collision_step()
        c.synchronize()
        out[name] = (c.get_state(), m0, c.moments())
        c.close()
    U_tc, m0, m1 = out["tc"]
    assert rel(U_tc, out["cuda"][0]) < 1e-9
    assert rel(U_tc, out["fp64"][0]) < 1e-6
    assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-12
    assert np.all(np.abs(m1[1:4] - m0[1:4]) / abs(m0[0]) < 1e-12)
    assert abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-12
