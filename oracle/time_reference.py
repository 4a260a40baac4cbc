"""Times the reference's own CPU build (oracle/_ref/libref.so, compiled from the
reference checkout by oracle/build_ref.sh) on the weak Landau damping workload:
Nx = 24 (the reference's 2-D layout, 24 x 24 spatial cells), Nv = N = 16,
v in [-5.25, 5.25]^3, A = 0.01, k = 0.5, nu = 0.01, dt = 0.01.

One time step is the reference's loop body (source/LP_ompi_1.cpp:496-568):
RK3 with its three pois2d solves (advection_1.cpp:428-601), then ComputeQ,
conserveAllMoments and RK4 for the collided cells -- the reference collides
cells s < Nx only (its defect F3), 24 cells -- and the scatter of dU into U.
Weights, tables and the initial state are built once, outside the timing.
The full run is 100 steps; this script times `--steps` of them and reports
the per-step time and the 100-step extrapolation.  Test and measurement
infrastructure; it runs only where the reference checkout was built.

    OMP_NUM_THREADS=8 python oracle/time_reference.py --steps 2
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# import the oracle package from the repository root (not this directory's
# oracle.py as a top-level module)
sys.path = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path.insert(0, os.path.dirname(HERE))

from oracle.oracle import Case, Reference, reference_available  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=2)
    args = ap.parse_args()
    if not reference_available():
        print(json.dumps({"unavailable": "oracle/_ref/libref.so was not built (no reference checkout)"}))
        return 0
    case = Case(nx1=24, nx2=24, nv=16, n=16, lv=5.25, lx=4 * np.pi, nu=0.01, dt=0.01, a_amp=0.01, k_wave=0.5)
    t0 = time.perf_counter()
    R = Reference(case, with_weights=True)
    U = R.set_init_ld()
    t_setup = time.perf_counter() - t0
    nv3 = case.nv ** 3
    rk3, coll = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        U, _, _, _ = R.rk3(U)
        t1 = time.perf_counter()
        du = R.collision_cells(U, 0, case.nx1).reshape(case.nx1 * nv3, 5)
        rec = U.reshape(-1, 7)
        rec[:case.nx1 * nv3, [0, 3, 4, 5, 6]] = du
        t2 = time.perf_counter()
        rk3.append(t1 - t0)
        coll.append(t2 - t1)
    step = float(np.mean(rk3) + np.mean(coll))
    out = {"workload": "weak Landau damping, Nx=24 (reference 2-D layout), Nv=N=16, 100 steps",
           "threads": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
           "cpu": os.uname().machine, "setup_s": t_setup, "steps_timed": args.steps,
           "rk3_s_per_step": float(np.mean(rk3)), "collision_s_per_step": float(np.mean(coll)),
           "collided_cells_per_step": case.nx1, "collision_s_per_cell_step": float(np.mean(coll)) / case.nx1,
           "step_s": step, "extrapolated_100_steps_s": 100 * step, "finite": bool(np.isfinite(U).all())}
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
