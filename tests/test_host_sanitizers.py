"""The host-side code under AddressSanitizer and UndefinedBehaviorSanitizer:
the library's table builders (landau-poisson-solver-2d_gb300/csrc/
lp_tables.cpp: grids, weight factors, conservation rows, DFT factors, the
LDG band matrix, its LU factors and dense inverse) and the CPU oracle
(oracle/lp_oracle.c), each driven on small cases by a driver in
tests/sanitize/.  A sanitizer report makes the driver exit non-zero
(-fno-sanitize-recover), and the test fails."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAN = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-g", "-O1"]


def _build_and_run(tmp_path, compiler, sources, includes, extra, name):
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not available")
    exe = str(tmp_path / name)
    cmd = [compiler] + SAN + [f"-I{i}" for i in includes] + sources + extra + ["-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ok" in r.stdout
    assert "runtime error" not in r.stderr and "ERROR: AddressSanitizer" not in r.stderr, r.stderr


def test_host_tables_sanitized(tmp_path):
    csrc = os.path.join(ROOT, "landau-poisson-solver-2d_gb300", "csrc")
    _build_and_run(tmp_path, "g++", [os.path.join(ROOT, "tests", "sanitize", "tables_driver.cpp"),
                                     os.path.join(csrc, "lp_tables.cpp")],
                   [os.path.join(ROOT, "include"), csrc], ["-std=c++17", "-ffp-contract=off"], "tables_driver")


def test_oracle_sanitized(tmp_path):
    odir = os.path.join(ROOT, "oracle")
    _build_and_run(tmp_path, "gcc", [os.path.join(ROOT, "tests", "sanitize", "oracle_driver.c"),
                                     os.path.join(odir, "lp_oracle.c")],
                   [odir], ["-ffp-contract=off", "-lm"], "oracle_driver")
