"""Benchmark of the collision hot path: collision+conserve cell-steps/s.

Workload (strong Landau damping, 1-D reduction of the reference's 2-D grid):
Nx = 64 spatial cells, Nv = N = 24 (24^3 DG velocity cells, 24^3 spectral
nodes), v in [-6, 6]^3, A = 0.5, k = 0.5, nu = 0.05, dt = 0.005, unit
Maxwellian initial state.  One "step" is one collision step of every spatial
cell: node sampling, 4 x (transform + weighted contraction + moment-conserving
projection), 3 inverse transforms and the DG projection with the dU scatter.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64]
  python bench.py --impl reference ...   # the CPU implementation of the path

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "landau-poisson-solver-2d_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

WORKLOAD = dict(nx1=64, nx2=1, nv=24, n=24, lv=6.0, lx=4 * np.pi, nu=0.05, dt=0.005, a_amp=0.5,
                k_wave=0.5)
METRIC = "collision+conserve cell-steps/s"
UNIT = "cell-steps/s"
L2_FLUSH_BYTES = 512 << 20
# DRAM bytes of one contraction of this workload in the line-tiled form
# (both k-tiles of k_cq_lines, dram__bytes_read.sum + dram__bytes_write.sum
# from one ncu capture of
# `bench.py --steps 2 --warmup 1 --no-cpu-baseline --fp64-steps 0`)
CONTRACT_TRAFFIC_BYTES = 105.24e6 + 100.49e6
PROFILES = os.path.join(ROOT, "profiles")


def profiled_traffic(kernel):
    """DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch
    of `kernel` from the committed ncu summaries under profiles/: the first
    summary with a line `traffic <kernel>: <read MB> + <write MB> MB` (the
    capture of the same command, kernel and workload).  Returns (bytes,
    summary file) or (None, None) when no summary covers the kernel."""
    import re
    if not os.path.isdir(PROFILES):
        return None, None
    pat = re.compile(r"^traffic\s+" + re.escape(kernel) + r":\s*([0-9.]+)\s*\+\s*([0-9.]+)\s*MB", re.M)
    for name in sorted(os.listdir(PROFILES)):
        if not name.endswith(".md"):
            continue
        with open(os.path.join(PROFILES, name)) as f:
            m = pat.search(f.read())
        if m:
            return (float(m.group(1)) + float(m.group(2))) * 1e6, "profiles/" + name
    return None, None


def profiled_fma_pipe(kernel):
    """Fraction of cycles the FP32 FMA pipe was busy in one launch of
    `kernel` (sm__pipe_fma_cycles_active), from the committed ncu summaries
    under profiles/: a line `fma_pipe <kernel>: <percent> %`.  Returns
    (fraction, summary file) or (None, None)."""
    import re
    if not os.path.isdir(PROFILES):
        return None, None
    pat = re.compile(r"^fma_pipe\s+" + re.escape(kernel) + r":\s*([0-9.]+)\s*%", re.M)
    for name in sorted(os.listdir(PROFILES)):
        if not name.endswith(".md"):
            continue
        with open(os.path.join(PROFILES, name)) as f:
            m = pat.search(f.read())
        if m:
            return float(m.group(1)) / 100.0, "profiles/" + name
    return None, None


def fq_kernel_model(n, cells):
    """Algorithmic DRAM bytes and FP32 flops per launch of the four kernels of
    the convolution form (complex FP32 intermediates of 8 bytes, q in FP64):
    each kernel reads its input arrays once and writes its outputs once."""
    M, h = 3 * n // 2, n // 2
    c8 = 8 * cells
    x, g, hh = 13 * n * M * M, n * M * M, n * n * M
    # valid (i, l) pairs of the direct axis-1 sum: 0 <= i + h - l < n
    pairs = sum(1 for i in range(n) for l in range(n) if 0 <= i + h - l < n)
    x1 = 10 * n * n * M  # axis-3 spectra of the 10 source arrays
    model = {
        # fused form: axis-3 DFTs into X1; axis-2 DFTs, axis-1 sums and
        # inverse axis-2 DFTs with the axis-2 spectra in shared memory
        "k_fq_x1": (n ** 3 * c8 + 7 * n ** 3 * 4 + x1 * c8, None),
        "k_fq_yz": (x1 * c8 + hh * c8, 7 * pairs * 8.0 * M * M * cells),
        # three-pass form: X1 and X2 fused, the X1 outputs in shared memory
        "k_fq_x12": (n ** 3 * c8 + 7 * n ** 3 * 4 + x * c8, None),
        "k_fq_y": (x * c8 + g * c8, 7 * pairs * 8.0 * M * M * cells),
        "k_fq_z1": (g * c8 + hh * c8, None),
        "k_fq_z2": (hh * c8 + n ** 3 * 16 * cells, None),
    }
    return model


def fq_kernels(form):
    """(name, lp_time_kernel code) of the convolution form's kernels: form 1
    (axis-2 spectra on chip) or 0 (three passes through DRAM)."""
    if form == 1:
        return [("k_fq_x1", 4), ("k_fq_yz", 6), ("k_fq_z2", 8)]
    return [("k_fq_x12", 4), ("k_fq_y", 6), ("k_fq_z1", 7), ("k_fq_z2", 8)]


class _Dev:
    """A device buffer of float64 values seen by torch (no copy)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False),
                                         "version": 3, "strides": None}


def _drift(m, m0):
    """Relative changes of mass, momentum (on the mass scale), kinetic energy
    and total (kinetic + electric) energy between two moment vectors
    {mass, p1, p2, p3, kinetic, electric}.  For the difference of two paths'
    changes, pass m = m0 + (change of one) - (change of the other)."""
    return {"mass": float(abs(m[0] - m0[0]) / abs(m0[0])),
            "momentum": float(np.max(np.abs(m[1:4] - m0[1:4])) / abs(m0[0])),
            "kinetic": float(abs(m[4] - m0[4]) / abs(m0[4])),
            "total_energy": float(abs(m[4] + m[5] - m0[4] - m0[5]) / abs(m0[4] + m0[5]))}


def accuracy_report(lp, make, schedule, nsteps, stream):
    """Error and conservation of the mixed path at the workload's own size,
    against the plain FP64 GPU path (itself within 1e-12 of the FP64 oracle
    on this workload's full step, tests/test_gpu_configs.py):

    - collision only: mass, momenta and kinetic energy through one collision
      step of all 64 cells, from the state after one advection step, for
      both paths;
    - full time steps: `nsteps` steps (advection + collision) of both paths
      from the same initial state; the relative L2 difference of the states
      every step (sampled into the line every nsteps/10 steps) and the drift
      of mass, momentum and energy of each path, and of mixed minus FP64.
    Norms are taken on the device, on the contexts' stream."""
    import torch
    out = {"steps": nsteps}
    coll = {}
    for prec in ("mixed", "fp64"):
        c = make(prec)
        if prec == "mixed":
            c.set_schedule(*schedule)
        c.advect_step()
        m0 = c.diagnostics()[:6]
        c.collision_step()
        d = _drift(c.diagnostics()[:6], m0)
        d.pop("total_energy")
        coll[prec] = d
        c.close()
    out["collision_only_drift"] = coll
    ref, mix = make("fp64"), make("mixed")
    mix.set_schedule(*schedule)
    n = ref.params.size * 7
    with torch.cuda.stream(stream):
        Ur = torch.as_tensor(_Dev(ref.state_device_ptr(), n), device="cuda")
        Um = torch.as_tensor(_Dev(mix.state_device_ptr(), n), device="cuda")
        # moments and the electric energy of a Poisson solve of each state
        r0, x0 = ref.diagnostics()[:6], mix.diagnostics()[:6]
        errs, dr, dm, dd = [], [], [], []
        for _ in range(nsteps):
            ref.step(1)
            mix.step(1)
            ref.synchronize()
            mix.synchronize()
            errs.append(float((torch.linalg.vector_norm(Um - Ur) / torch.linalg.vector_norm(Ur)).item()))
            r1, x1 = ref.diagnostics()[:6], mix.diagnostics()[:6]
            a, b = _drift(r1, r0), _drift(x1, x0)
            dr.append(a)
            dm.append(b)
            dd.append(_drift(r0 + (x1 - x0) - (r1 - r0), r0))
        finite = bool(torch.isfinite(Um).all().item())
    every = max(1, nsteps // 10)
    out["rel_err_vs_fp64"] = {"every": every, "values": errs[every - 1::every], "first": errs[0],
                              "max": max(errs), "final": errs[-1]}

    def mx(rows):
        return {k: max(r[k] for r in rows) for k in rows[0]}

    out["full_step_drift_max"] = {"fp64": mx(dr), "mixed": mx(dm), "mixed_minus_fp64": mx(dd)}
    out["full_step_drift_final"] = {"fp64": dr[-1], "mixed": dm[-1], "mixed_minus_fp64": dd[-1]}
    out["finite"] = finite
    ref.close()
    mix.close()
    return out


def _config(extra=None):
    cfg = {"workload": "strong Landau damping, Nx=64 (1-D), Nv=N=24, v in [-6,6]^3, nu=0.05, "
                       "dt=0.005; one collision step of all 64 spatial cells",
           "nx1": 64, "nx2": 1, "nv": 24, "n": 24, "cells_per_step": 64,
           "l2": "flushed between timed steps (512 MiB write)"}
    if extra:
        cfg.update(extra)
    return cfg


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 3 + i and r[3 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_baseline(sample_cells=1, threads=None):
    """The CPU restatement of the path (oracle port, same algorithm and cost
    structure as the reference: direct weighted sums and per-(mode, v-cell)
    IntModes projection) on a bounded sample of the workload."""
    from oracle.oracle import Case, FIX_DEFAULT, Oracle
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    case = Case(**WORKLOAD)
    O = Oracle(case, fixes=FIX_DEFAULT)
    U = O.set_init(1)
    nv3 = case.nv ** 3
    ucell = U.reshape(case.ncell, nv3 * 7)
    t0 = time.perf_counter()
    for s in range(sample_cells):
        f = O.nodes(U, s)
        q = O.conserve(O.compute_q(f))
        O.rk4(f, q, ucell[s], direct=True)
    dt = time.perf_counter() - t0
    return sample_cells / dt, dt


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(cores)
    vals = []
    for i in range(args.warmup + args.steps):
        v, _ = cpu_baseline(1)
        if i >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals)) if vals else 0.0
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / value if value else None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded analytic initial state)",
            "config": _config({"sample": "1 spatial cell per step (the full step is 64 cells)"}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "1 spatial cell of the 64-cell collision step per timed step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def batch_runs(seed=20261203, count=64):
    """64 independent runs drawn from a seed: Nx uniform in {16, 32, 64, 128},
    N = Nv uniform in {16, 24, 32}, A log-uniform in [1e-3, 0.5], k uniform in
    [0.3, 0.6], nu log-uniform in [1e-3, 1e-1]; v in [-5.25, 5.25]^3, perturbed
    unit Maxwellian; dt = min(0.01, 0.25 dx / 5.25), inside the SSP-RK3 / P1
    upwind stability bound of every run (dt = 0.01 is not, for the finest
    grids: Nx = 128 at k = 0.6 gives a Courant number of 0.64)."""
    rng = np.random.default_rng(seed)
    runs = []
    for _ in range(count):
        nx = int(rng.choice([16, 32, 64, 128]))
        nn = int(rng.choice([16, 24, 32]))
        a = float(np.exp(rng.uniform(np.log(1e-3), np.log(0.5))))
        k = float(rng.uniform(0.3, 0.6))
        nu = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-1))))
        lx = 2 * np.pi / k
        dt = min(0.01, 0.25 * (lx / nx) / 5.25)
        runs.append(dict(nx1=nx, nx2=1, nv=nn, n=nn, lv=5.25, lx=lx, nu=nu, dt=dt, a_amp=a, k_wave=k))
    return runs


TWOSTREAM = dict(nx1=256, nx2=1, nv=32, n=32, lv=8.0, lx=2 * np.pi / 0.3, nu=0.01, dt=0.0025,
                 a_amp=0.01, k_wave=0.3)
WEAK = dict(nx1=24, nx2=1, nv=16, n=16, lv=5.25, lx=4 * np.pi, nu=0.01, dt=0.01, a_amp=0.01, k_wave=0.5)
# The reference's own CPU build on this workload (oracle/time_reference.py,
# its 2-D layout with the 24 collided cells of its loop, 8 Xeon threads at
# 2.7 GHz): 56.7 s per time step, 100 steps extrapolated to 5672 s.
WEAK_REFERENCE_S_PER_STEP = 56.7


def run_workload(args, emit=True):
    """Secondary workloads, one JSON line each: `batch` (64 seeded uneven runs
    in one batch, full time steps from the batch's per-step graph, schedules
    picked by the autotuner), `twostream` (the large two-stream instance,
    Nx = 256, N = Nv = 32, full time steps, plus its error against FP64) and
    `weak` (the whole 100-step weak-damping run).  emit=False returns the
    line instead of printing it."""
    import torch
    import lp_gb300 as lp
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    prec = lp.PREC_MIXED if args.precision == "mixed" else lp.PREC_FP64

    def timed(fn, k, w):
        with torch.cuda.stream(stream):
            for _ in range(w):
                fn()
            torch.cuda.synchronize()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(k)]
            for i in range(k):
                flush.zero_()
                ev[i][0].record(stream)
                fn()
                ev[i][1].record(stream)
            torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / 1e3

    extra = {}
    if args.workload == "weak":
        # the whole 100-step run of weak Landau damping, per precision, from
        # the initial state resident on the device; diagnostics every step
        # on the device (no host copies of the state)
        runs = {}
        clk = ClockSampler(0)
        clk.__enter__()
        for prec_name, pr in (("mixed", lp.PREC_MIXED), ("fp64", lp.PREC_FP64)):
            c = lp.Context(lp.Params(**WEAK, fixes=lp.FIX_DEFAULT, precision=pr))
            c.set_stream(stream.cuda_stream)
            c.set_init(1)
            c.step(1)
            c.set_init(1)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                e0.record(stream)
                c.step(100)
                e1.record(stream)
            torch.cuda.synchronize()
            runs[prec_name] = {"run_s": e0.elapsed_time(e1) / 1e3, "diagnostics_after": c.diagnostics()[:6].tolist()}
            c.close()
        clk.__exit__(None, None, None)
        cells = WEAK["nx1"] * 100
        t = runs["mixed" if prec == lp.PREC_MIXED else "fp64"]["run_s"]
        extra["runs"] = runs
        extra["reference_cpu"] = {"s_per_step": WEAK_REFERENCE_S_PER_STEP,
                                  "run_s_extrapolated": 100 * WEAK_REFERENCE_S_PER_STEP,
                                  "kind": "reference", "cores": 8,
                                  "how": "oracle/time_reference.py: the reference's own sources built here, "
                                         "2 steps timed on 8 Xeon threads, 100 extrapolated"}
        cfg = {"workload": "weak Landau damping, Nx=24 (1-D), N=Nv=16, v in [-5.25,5.25]^3, A=0.01, k=0.5, "
                           "nu=0.01, dt=0.01; the whole 100-step run", "steps_in_run": 100,
               "precision": args.precision}
        line = {"metric": "whole-run full-step cell-steps/s", "value": cells / t, "unit": "cell-steps/s",
                "n_gpus": 1, "steps": 100, "warmup": 1, "ms_per_step": 1e3 * t / 100, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64" if args.precision == "mixed" else "f64",
                "data": "synthetic (analytic initial state)", "config": cfg, "clocks": clk.summary()}
        line.update(extra)
        if not emit:
            return line
        print(json.dumps(line), flush=True)
        return 0
    if args.workload == "batch":
        specs = batch_runs()
        b = lp.Batch([lp.Params(**r, fixes=lp.FIX_DEFAULT, precision=prec) for r in specs])
        b.set_stream(stream.cuda_stream)
        for i in range(len(specs)):
            b.set_init(i, 1)
        t0 = time.perf_counter()
        b.autotune(reps=2)
        extra["autotune_s"] = time.perf_counter() - t0
        extra["classes"] = [dict(zip(["n", "nv", "runs", "cells", "cells_per_pass", "line_warps",
                                      "collision_ms"], c)) for c in b.classes()]
        cells = sum(r["nx1"] * r["nx2"] for r in specs)
        with ClockSampler(0) as clk:
            t = timed(lambda: b.step(1), args.steps, args.warmup)
        m = [b.moments(i) for i in range(len(specs))]
        extra["finite"] = bool(all(np.all(np.isfinite(x)) for x in m))
        if prec == lp.PREC_MIXED and args.fp64_steps > 0:
            # error against FP64 on a sample of the runs (the first 8, every N
            # of the draw among them): the same runs as a mixed and an FP64
            # batch, full steps from the same initial states
            sub = specs[:8]
            mb = lp.Batch([lp.Params(**r, fixes=lp.FIX_DEFAULT, precision=lp.PREC_MIXED) for r in sub])
            fb = lp.Batch([lp.Params(**r, fixes=lp.FIX_DEFAULT, precision=lp.PREC_FP64) for r in sub])
            for i in range(len(sub)):
                mb.set_init(i, 1)
                fb.set_init(i, 1)
            m0 = [mb.moments(i) for i in range(len(sub))]
            mb.step(args.fp64_steps)
            fb.step(args.fp64_steps)
            errs, drift, drift64 = [], [], []
            for i in range(len(sub)):
                Um, Uf = mb.get_state(i), fb.get_state(i)
                errs.append(float(np.linalg.norm(Um - Uf) / np.linalg.norm(Uf)))
                m1, f1 = mb.moments(i), fb.moments(i)
                drift.append(float(abs(m1[0] - m0[i][0]) / abs(m0[i][0])))
                drift64.append(float(abs(f1[0] - m0[i][0]) / abs(m0[i][0])))
            extra["rel_err_vs_fp64"] = {"runs": len(sub), "steps": args.fp64_steps, "max": max(errs),
                                        "per_run": errs, "n_of_runs": [r["n"] for r in sub]}
            # relative mass change of the sample over the same steps, mixed and
            # FP64 (the full step lets mass leave through the velocity boundary)
            extra["mass_drift_max"] = {"mixed": max(drift), "fp64": max(drift64)}
            mb.close()
            fb.close()
        cfg = {"workload": "64 seeded uneven runs (Nx in {16,32,64,128}, N=Nv in {16,24,32}, "
                           "A, k, nu drawn), one full time step of every run per step",
               "seed": 20261203, "runs": len(specs), "cells_per_step": cells,
               "l2": "flushed between timed steps (512 MiB write)", "precision": args.precision}
        metric, unit = "batched full-step cell-steps/s", "cell-steps/s"
    else:
        P = lp.Params(**TWOSTREAM, fixes=lp.FIX_DEFAULT, precision=prec)
        ctx = lp.Context(P)
        ctx.set_stream(stream.cuda_stream)
        ctx.set_init(2, 2.0)
        cells = TWOSTREAM["nx1"]
        # the library's autotuner picks the collision schedule (outside the timed region)
        sched = ctx.autotune(reps=1)
        extra["schedule"] = {"cells_per_pass": sched[0], "line_warps": sched[1],
                             "convolution_form": ctx.convolution_form()}
        with ClockSampler(0) as clk:
            t = timed(lambda: ctx.step(1), args.steps, args.warmup)
        with torch.cuda.stream(stream):
            flush.zero_()
            extra["contraction_ms"] = ctx.time_kernel(0, reps=3)
        if prec == lp.PREC_MIXED and args.fp64_steps > 0:
            ref = lp.Context(lp.Params(**TWOSTREAM, fixes=lp.FIX_DEFAULT, precision=lp.PREC_FP64))
            mix = lp.Context(P)
            ref.set_init(2, 2.0)
            mix.set_init(2, 2.0)
            m0 = mix.moments()
            ref.step(args.fp64_steps)
            mix.step(args.fp64_steps)
            Ur, Um = ref.get_state(), mix.get_state()
            extra["rel_err_vs_fp64"] = float(np.linalg.norm(Um - Ur) / np.linalg.norm(Ur))
            extra["err_steps"] = args.fp64_steps
            m1 = mix.moments()
            extra["mass_drift"] = float(abs(m1[0] - m0[0]) / abs(m0[0]))
        cfg = {"workload": "two-stream, Nx=256 (1-D), N=Nv=32, v in [-8,8]^3, u=2, A=0.01, k=0.3, "
                           "nu=0.01, dt=0.0025; one full time step per step",
               "cells_per_step": cells, "l2": "flushed between timed steps (512 MiB write)",
               "precision": args.precision}
        metric, unit = "full-step cell-steps/s", "cell-steps/s"
    line = {"metric": metric, "value": cells * args.steps / t, "unit": unit, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded analytic initial states)", "config": cfg,
            "clocks": clk.summary()}
    line.update(extra)
    if not emit:
        return line
    print(json.dumps(line), flush=True)
    return 0


def secondary_lines(args):
    """Short runs of the secondary workloads for the headline line: the
    batch of 64 uneven runs and the two-stream instance (3 timed full steps
    after 2 warm-up steps each, the two-stream error against FP64 after one
    step) and the whole weak-damping run."""
    out = {}
    for name in ("batch", "twostream", "weak"):
        a = argparse.Namespace(**vars(args))
        a.workload, a.steps, a.warmup, a.fp64_steps = name, 3, 2, 1
        try:
            out[name] = run_workload(a, emit=False)
        except Exception as e:  # reported, not hidden: the headline line still prints
            out[name] = {"error": f"{type(e).__name__}: {e}"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--accuracy-steps", type=int, default=200,
                    help="full time steps of the mixed and FP64 paths compared after the timing")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the short runs of the batch, two-stream and whole-run workloads")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="landau64", choices=["landau64", "batch", "twostream", "weak"])
    ap.add_argument("--schedule", default=None,
                    help="cells_per_pass,line_warps for the collision (skips the autotuner)")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="only run this many collision steps of the workload (for ncu launch lists)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "landau64":
        return run_workload(args)

    import torch
    import lp_gb300 as lp

    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def make(prec):
        P = lp.Params(**WORKLOAD, fixes=lp.FIX_DEFAULT,
                      precision=lp.PREC_MIXED if prec == "mixed" else lp.PREC_FP64)
        ctx = lp.Context(P)
        ctx.set_stream(stream.cuda_stream)
        ctx.set_init(1)
        return ctx

    def timed(ctx, fn, k, w):
        with torch.cuda.stream(stream):
            for _ in range(w):
                fn()
            torch.cuda.synchronize()
            if ws > 1:
                torch.distributed.barrier()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(k)]
            total = 0.0
            for i in range(k):
                flush.zero_()
                ev[i][0].record(stream)
                fn()
                ev[i][1].record(stream)
            torch.cuda.synchronize()
            total = sum(a.elapsed_time(b) for a, b in ev) / 1e3
        return total

    ctx = make(args.precision)
    cells = WORKLOAD["nx1"] * WORKLOAD["nx2"]
    # the library's autotuner picks the collision schedule (outside the timed region)
    if args.schedule:
        schedule = tuple(int(x) for x in args.schedule.split(","))
        ctx.set_schedule(*schedule)
    else:
        schedule = ctx.autotune(reps=2)
    if args.profile_steps > 0:
        with torch.cuda.stream(stream):
            for _ in range(args.profile_steps):
                ctx.collision_step()
            torch.cuda.synchronize()
        U = ctx.get_state()
        print(json.dumps({"profile_steps": args.profile_steps, "schedule": schedule,
                          "finite": bool(np.isfinite(U).all())}), flush=True)
        return 0
    with ClockSampler(local) as clk:
        t = timed(ctx, lambda: ctx.collision_step(), args.steps, args.warmup)
    t_max = t
    if ws > 1:
        tt = torch.tensor([t], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_max = float(tt.item())
    value = ws * cells * args.steps / t_max

    # End to end through the C ABI's host-buffer entry (lp_collision_step_host):
    # every step copies the whole state from pinned host memory to the device,
    # collides every cell and copies the state back into pinned host memory.
    # The K steps are queued back to back (LP_HOST_ASYNC on all but the last),
    # so one step's copies overlap the neighbouring steps' collisions, and
    # timed as one region with CUDA events on the context's stream (its
    # working set -- two 49.5 MB staging states and the collision scratch --
    # is larger than L2).  The chunk count per step is picked outside the
    # timed region from {1, 2, 4}.
    U_host = torch.from_numpy(ctx.get_state()).pin_memory()
    U_out = torch.empty_like(U_host).pin_memory()
    nbytes = U_host.numel() * 8
    e2e_k = max(3, args.steps)

    def e2e_region(k, ch):
        with torch.cuda.stream(stream):
            for _ in range(2):
                ctx.collision_step_host(U_host, U_out, ch)
            ctx.synchronize()
            torch.cuda.synchronize()
            flush.zero_()
            torch.cuda.synchronize()  # no copy of the region starts before its first event
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for i in range(k):
                ctx.collision_step_host(U_host, U_out, ch, asynchronous=(i < k - 1))
            e1.record(stream)
            ctx.synchronize()
            torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    e2e_try = {ch: e2e_region(3, ch) / 3 for ch in (1, 2, 4)}
    e2e_chunks = min(e2e_try, key=e2e_try.get)
    t_e2e = e2e_region(e2e_k, e2e_chunks)
    e2e_value = ws * cells * e2e_k / t_e2e

    # Dominant kernel: the weighted contraction of ComputeQ for the 64 cells,
    # timed alone with CUDA events on the context's stream; in the
    # convolution form each of its four kernels is timed alone too.
    extra = {}
    with torch.cuda.stream(stream):
        flush.zero_()
        t_contract_ms = ctx.time_kernel(0, reps=max(5, args.steps))
        fq_ms = {}
        if schedule[1] == 0:
            for name, code in fq_kernels(ctx.convolution_form()):
                flush.zero_()
                fq_ms[name] = ctx.time_kernel(code, reps=max(5, args.steps))
    n = WORKLOAD["n"]
    h = n // 2
    win = [i + h + 1 if i < h else 3 * h - 1 - i for i in range(n)]
    npairs = sum((a * b * c + 1) // 2 for a in win for b in win for c in win)
    # FP32 work per pair and cell: complex product (6 flops), weight (2), accumulate (2)
    contract_flops = 10.0 * npairs * cells
    # bytes the contraction must move: F read once (complex float), q written
    # (complex double), and its weight table (one float per pair) read once
    n3 = n ** 3
    contract_bytes = n3 * cells * 8 + n3 * cells * 16 + npairs * 4
    fp32_peak, fp64_peak = lp.measure_fp_peaks()
    # Full time step (advection + collision) through the captured graph.
    with torch.cuda.stream(stream):
        ctx.step(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.step(3)
        e1.record(stream)
        torch.cuda.synchronize()
        extra["full_step_ms"] = e0.elapsed_time(e1) / 3
    extra["schedule"] = {"cells_per_pass": schedule[0], "line_warps": schedule[1],
                         "convolution_form": ctx.convolution_form()}
    if rank == 0:
        t_fp64 = None
        if args.precision == "mixed" and args.fp64_steps > 0:
            ctx64 = make("fp64")
            t64 = timed(ctx64, lambda: ctx64.collision_step(), args.fp64_steps, 1)
            t_fp64 = cells * args.fp64_steps / t64
            ctx64.close()
            if args.accuracy_steps > 0:
                extra["accuracy"] = accuracy_report(lp, make, schedule, args.accuracy_steps, stream)
                extra["finite"] = extra["accuracy"]["finite"]
        extra["fp64_value"] = t_fp64
        extra["mixed_over_fp64"] = (value / ws / t_fp64) if t_fp64 else None

    if rank == 0:
        peak, peak_kind = _peaks()
        cb = None
        if not args.no_cpu_baseline and ws == 1:
            v, secs = cpu_baseline(1)
            cb = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                  "sample": f"1 spatial cell of the 64-cell step ({secs:.1f} s of CPU work)"}
        if fq_ms:
            model = fq_kernel_model(n, cells)
            kern = []
            for name, ms in fq_ms.items():
                b, fl = model[name]
                kern.append({"kernel": name, "ms_per_launch": ms, "algorithmic_bytes": b,
                             "gbs": b / (ms * 1e-3) / 1e9,
                             "tflops": (fl / (ms * 1e-3) / 1e12) if fl else None})
            extra["contraction_kernels"] = kern
            dom = max(kern, key=lambda k: k["ms_per_launch"])
            hbm_frac = dom["gbs"] / peak
            traffic, traffic_src = profiled_traffic(dom["kernel"])
            roof = {"bound": "hbm", "achieved": dom["gbs"], "peak": peak, "unit": "GB/s", "frac": hbm_frac,
                    "traffic": traffic, "traffic_source": traffic_src,
                    "algorithmic_bytes": dom["algorithmic_bytes"], "peak_kind": peak_kind,
                    "kernel": dom["kernel"] + " (the largest kernel of the convolution form)",
                    "ms_per_launch": dom["ms_per_launch"]}
            fma_busy, fma_src = profiled_fma_pipe(dom["kernel"])
            comp = {"pipe": "fp32 FMA (packed f32x2, CUDA cores)", "kernel": dom["kernel"],
                    "achieved_tflops": dom["tflops"], "peak_tflops": fp32_peak,
                    "frac": (dom["tflops"] / fp32_peak) if (dom["tflops"] and fp32_peak) else None,
                    "flops_counted": "the direct axis-1 sums only (7 pairs x 432 (i, l) pairs x 8 x M^2 per cell)",
                    "fma_pipe_busy_ncu": fma_busy, "fma_pipe_source": fma_src,
                    "peak_kind": "measured (FMA-chain microbenchmark)", "fp64_peak_tflops": fp64_peak}
        else:
            achieved = contract_bytes / (t_contract_ms * 1e-3) / 1e9
            contract_tflops = contract_flops / (t_contract_ms * 1e-3) / 1e12
            roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "traffic": CONTRACT_TRAFFIC_BYTES if args.precision == "mixed" else None,
                    "algorithmic_bytes": contract_bytes, "peak_kind": peak_kind,
                    "kernel": "k_cq_lines (weighted contraction of ComputeQ, all tiles)",
                    "ms_per_launch": t_contract_ms,
                    "note": "the contraction is bound by the FP32 FMA pipe, see compute_roofline"}
            comp = {"pipe": "fp32 FMA (packed f32x2, CUDA cores)",
                    "achieved_tflops": contract_tflops, "peak_tflops": fp32_peak,
                    "frac": contract_tflops / fp32_peak if fp32_peak else None,
                    "peak_kind": "measured (FMA-chain microbenchmark)", "fp64_peak_tflops": fp64_peak}
        extra["contraction_ms"] = t_contract_ms
        # the step against the per-cell-step figures of the workload's
        # algorithmic counts: HBM bytes Nv^3 (7 + 5) 8 (read the records,
        # write the 5 collided coefficients) and the FFT form's FLOP
        # 4 [15 * 5 m log2 m + 7 * 8 m] with m = (2N)^3, plus the separable
        # projection 8 * 5 (Nv N^3 + Nv^2 N^2 + Nv^3 N)
        nv_, n_ = WORKLOAD["nv"], WORKLOAD["n"]
        m_ = (2 * n_) ** 3
        flop_cs = 4 * (15 * 5 * m_ * np.log2(m_) + 7 * 8 * m_) + 8 * 5 * (nv_ * n_ ** 3 + nv_ ** 2 * n_ ** 2 + nv_ ** 3 * n_)
        bytes_cs = nv_ ** 3 * 12 * 8
        step_s = t_max / args.steps
        extra["step_roofline_per_cell_step_counts"] = {
            "bytes_per_cell_step": bytes_cs, "flop_per_cell_step": float(flop_cs),
            "hbm_gbs": bytes_cs * cells / step_s / 1e9, "hbm_frac": bytes_cs * cells / step_s / 1e9 / peak,
            "tflops": flop_cs * cells / step_s / 1e12,
            "fp32_frac": (flop_cs * cells / step_s / 1e12) / fp32_peak if fp32_peak else None,
            "note": "whole collision step; the step moves its intermediates through HBM and L2, so the per-step "
                    "HBM figure is far below the copy peak while the FLOP figure is near the FP32 FMA peak"}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64" if args.precision == "mixed" else "f64",
                "data": "synthetic (seeded analytic initial state)",
                "config": _config({"precision": args.precision}),
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes,
                        "d2h_bytes_per_step": nbytes, "api": "lp_collision_step_host (pinned host buffers)",
                        "chunks": e2e_chunks, "steps": e2e_k, "ms_per_step": 1e3 * t_e2e / e2e_k,
                        "ms_per_step_by_chunks": {str(k): 1e3 * v for k, v in e2e_try.items()}},
                "roofline": roof, "compute_roofline": comp,
                "cpu_baseline": cb, "clocks": clk.summary(),
                "gpu_launches": ctx.collision_graph_kernels() * args.steps,
                "graph": {"kernels": ctx.collision_graph_kernels(),
                          "programmatic_edges": ctx.collision_graph_edges()}}
        line.update(extra)
        if ws == 1 and not args.no_secondary and args.precision == "mixed":
            line["secondary"] = secondary_lines(args)
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
