"""Batches of independent runs (lp_batch_*): every run of a batch, stepped
through the batch's captured per-step graph, matches the same run stepped
alone through its own context; the autotuner keeps the state and only picks
among schedules that give the same results."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def _runs(lp, precision):
    P = lambda **kw: lp.Params(lv=5.25, fixes=lp.FIX_DEFAULT, precision=precision, **kw)
    return [
        P(nx1=8, nx2=1, nv=8, n=8, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5),
        P(nx1=6, nx2=1, nv=8, n=8, lx=2 * np.pi / 0.4, nu=0.02, dt=0.005, a_amp=0.1, k_wave=0.4),
        P(nx1=4, nx2=3, nv=8, n=16, lx=4 * np.pi, nu=0.1, dt=0.01, a_amp=0.2, k_wave=0.5),
        P(nx1=5, nx2=1, nv=8, n=16, lx=2 * np.pi / 0.3, nu=0.0, dt=0.01, a_amp=0.01, k_wave=0.3),
    ]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_matches_single_runs(gpu_lib, prec):
    lp = gpu_lib
    precision = lp.PREC_FP64 if prec == "fp64" else lp.PREC_MIXED
    runs = _runs(lp, precision)
    b = lp.Batch(runs)
    cls = b.classes()
    assert [(c[0], c[1], c[2], c[3]) for c in cls] == [(8, 8, 2, 14), (16, 8, 2, 17)]
    singles = []
    for r, P in enumerate(runs):
        b.set_init(r, 1)
        ctx = lp.Context(P)
        ctx.set_init(1)
        singles.append(ctx)
    b.step(3)
    for r, ctx in enumerate(singles):
        ctx.step(3)
        assert rel(b.get_state(r), ctx.get_state()) < 1e-12, r
        m_b, m_s = b.moments(r), ctx.moments()
        assert abs(m_b[0] - m_s[0]) <= 1e-12 * abs(m_s[0])
        assert abs(m_b[5] - m_s[5]) <= 1e-10 * abs(m_s[5]) + 1e-300


def test_batch_graph_equals_eager_steps(gpu_lib):
    lp = gpu_lib
    runs = _runs(lp, lp.PREC_MIXED)
    b1, b2 = lp.Batch(runs), lp.Batch(runs)
    for r in range(len(runs)):
        b1.set_init(r, 1)
        b2.set_init(r, 1)
    b1.step(2)
    for _ in range(2):
        b2.advect_step()
        b2.collision_step()
    for r in range(len(runs)):
        assert np.array_equal(b1.get_state(r), b2.get_state(r)), r


def test_autotune_keeps_state_and_caches(gpu_lib, tmp_path):
    lp = gpu_lib
    runs = _runs(lp, lp.PREC_MIXED)
    b = lp.Batch(runs)
    for r in range(len(runs)):
        b.set_init(r, 1)
    before = [b.get_state(r) for r in range(len(runs))]
    cache = str(tmp_path / "tune.txt")
    b.autotune(reps=2, cache_path=cache)
    for r in range(len(runs)):
        assert np.array_equal(b.get_state(r), before[r]), r
    cls = b.classes()
    for c in cls:
        assert c[4] % 32 == 0 and c[4] >= 32 and c[5] in (0, 2, 4) and c[6] > 0
    assert os.path.exists(cache) and len(open(cache).read().splitlines()) == len(cls)
    b.step(2)
    ref = lp.Batch(runs)  # default schedule
    for r in range(len(runs)):
        ref.set_init(r, 1)
    ref.step(2)
    for r in range(len(runs)):
        assert rel(b.get_state(r), ref.get_state(r)) < 1e-6, r
    # a second batch reads the cached schedules instead of timing again
    b2 = lp.Batch(runs)
    for r in range(len(runs)):
        b2.set_init(r, 1)
    b2.autotune(reps=2, cache_path=cache)
    assert [c[4:6] for c in b2.classes()] == [c[4:6] for c in cls]


def test_batch_rejects_mixed_settings(gpu_lib):
    lp = gpu_lib
    runs = _runs(lp, lp.PREC_MIXED)
    runs[1].precision = lp.PREC_FP64
    with pytest.raises(lp.LPError):
        lp.Batch(runs)
    runs = _runs(lp, lp.PREC_MIXED)
    runs[0].fixes = lp.FIX_F2 | lp.FIX_F3  # collisions in passes need F1 fixed
    with pytest.raises(lp.LPError):
        lp.Batch(runs)


def test_context_autotune(gpu_lib, tmp_path):
    lp = gpu_lib
    P = lp.Params(nx1=8, nx2=1, nv=8, n=16, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.2, k_wave=0.5,
                  fixes=lp.FIX_DEFAULT, precision=lp.PREC_MIXED)
    a, b = lp.Context(P), lp.Context(P)
    a.set_init(1)
    b.set_init(1)
    U0 = a.get_state()
    cache = str(tmp_path / "t.txt")
    bp, lw = a.autotune(reps=2, cache_path=cache)
    assert bp % 32 == 0 and lw in (0, 2, 4)
    assert np.array_equal(a.get_state(), U0)
    # the cache line records the kernel form of the convolution form too
    fields = open(cache).read().split()
    assert len(fields) == 5 and int(fields[4]) == a.convolution_form() in (0, 1)
    b.set_convolution_form(1 - a.convolution_form())
    assert b.autotune(reps=2, cache_path=cache) == (bp, lw)  # from the cache
    assert b.convolution_form() == a.convolution_form()
    # a line without the form (an older cache) sets the schedule and keeps the form
    old_cache = str(tmp_path / "old.txt")
    with open(old_cache, "w") as f:
        f.write(" ".join(fields[:4]) + "\n")
    d = lp.Context(P)
    d.set_init(1)
    d.set_convolution_form(0)
    assert d.autotune(reps=2, cache_path=old_cache) == (bp, lw)
    assert d.convolution_form() == 0
    a.step(2)
    c = lp.Context(P)
    c.set_init(1)
    c.step(2)
    assert rel(a.get_state(), c.get_state()) < 1e-6
