"""Per-iteration statistics of a solve (kf_psi_solve_history).

The monitored energy, max |dpsi| and band count of every executed iteration,
as the solvers record them on the device: the first and last entries equal
the solve's own statistics, the dense and band-only solvers give the same
band counts and steps, an early-exit solve reports the iterations it ran,
and the per-voxel schedule (which keeps no per-iteration record) and a field
without a solve are refused.
"""
import numpy as np
import pytest

from helpers import small_pair

pytestmark = pytest.mark.gpu


def setup(capi, P, n=32, seed=80):
    can, live = small_pair(n, P.voxel_size, 5.0, seed=seed)
    dims = (n, n, n)
    gl = capi.Grid(dims, P.voxel_size, (0, 0, 0), P.unknown_clip, P)
    gc = capi.Grid(dims, P.voxel_size, (0, 0, 0), P.unknown_clip, P)
    gl.upload(live, (live <= P.max_surface).astype(np.int32))
    gc.upload(can, (can <= P.max_surface).astype(np.int32))
    return gl, gc, dims


def test_history_matches_statistics(gpu):
    capi = gpu
    P = capi.Params.reference(0.004, 5.0)
    gl, gc, dims = setup(capi, P)
    hist = {}
    for solver in ("fused", "band"):
        f = capi.Field(dims, capi.KF_F32)
        st = capi.psi_solve(gl, gc, f, P, 30, solver)
        h = capi.solve_history(f)
        assert len(h["energy"]) == 30
        assert h["active"][0] == st["active_first"] and h["active"][-1] == st["active_last"]
        assert h["energy"][0] == st["energy_first"] and h["energy"][-1] == st["energy_last"]
        assert h["max_delta"][-1] == st["max_delta_last"]
        assert np.all(h["max_delta"] > 0) and np.all(h["active"] > 0)
        hist[solver] = h
        f.close()
    np.testing.assert_array_equal(hist["fused"]["active"], hist["band"]["active"])
    np.testing.assert_array_equal(hist["fused"]["max_delta"], hist["band"]["max_delta"])
    np.testing.assert_allclose(hist["fused"]["energy"], hist["band"]["energy"], rtol=1e-9)


def test_history_of_early_exit_and_refusals(gpu):
    capi = gpu
    # this pair's steps start at 7.3e-5 voxel and fall below 5e-5 after about 95
    # iterations (FP64 oracle)
    P = capi.Params.reference(0.004, 5.0).with_(early_exit=True, threshold=5e-5)
    gl, gc, dims = setup(capi, P, seed=81)
    f = capi.Field(dims, capi.KF_F32)
    with pytest.raises(capi.KFError):
        capi.solve_history(f)  # no solve yet
    st = capi.psi_solve(gl, gc, f, P, 400, "fused")
    h = capi.solve_history(f)
    assert 1 < len(h["max_delta"]) == st["iterations_run"] < 400
    assert h["max_delta"][-1] <= np.float32(5e-5) < h["max_delta"][0]
    capi.psi_solve(gl, gc, f, P, 5, "pervoxel")
    with pytest.raises(capi.KFError):
        capi.solve_history(f)
    f.close()
