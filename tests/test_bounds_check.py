"""The bounds-check build (libkillingfusion_bc.so, -DKF_BOUNDS_CHECK).

compute-sanitizer is not available on the GPU pool, so the kernels of the
hot path check every index they take from data in this build (band lists
and their append positions, the dense passes' queues and run tables, the
in-place write-back, side lists, marching-cubes block lists) and record the
first one outside its bound instead of using it.  tests/bounds_workload.py
runs every hot-path kernel on 8^3-32^3 grids through that build, in a child
process:
* as built, no check fails and the results agree as they must (band-only =
  dense, batch = single solves, trust region band = dense);
* with every bound lowered to 40 entries (kf_bounds_reset(40)), the checks
  fire -- each flagged access is skipped, so nothing leaves its buffer --
  and the record names a site, an index and the bound 40.
The normal build reports the mode as disabled.
"""
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def run_checked(*args):
    env = dict(os.environ, KF_LIBRARY="bounds_check")
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_workload.py"), *args], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.gpu
def test_checked_build_runs_clean(gpu):
    st = run_checked()
    assert st["enabled"] == 1
    assert st["failures"] == []
    assert st["violations"] == 0, st


@pytest.mark.gpu
def test_checked_build_reports_lowered_bounds(gpu):
    st = run_checked("--limit", "40")
    assert st["enabled"] == 1
    assert st["violations"] > 0
    assert 1 <= st["site"] <= 10 and st["bound"] == 40 and st["index"] >= 40, st


def test_normal_build_reports_disabled():
    from killingfusion_gb300 import _build, capi
    if not os.path.exists(_build.LIB):
        _build.build()
    st = capi.bounds_status()  # host-side only: reads no device record
    assert st["enabled"] == 0 and st["violations"] == 0
