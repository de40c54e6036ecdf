"""The non-waiting entry points: kf_psi_solve_async / kf_psi_solve_wait and
kf_marching_cubes_async give what their waiting forms give, bit for bit, and
work queued behind them sees their results; the frame pipeline, which uses
them, leaves the canonical SDF untouched when a solve diverges."""
import ctypes as C

import numpy as np
import pytest

from helpers import small_pair

pytestmark = pytest.mark.gpu

VOXEL = 0.004
STATS = ("iterations_run", "converged", "diverged", "active_first", "active_last", "max_delta_last")


def grid(gpu, phi, P):
    nz, ny, nx = phi.shape
    g = gpu.Grid((nx, ny, nz), VOXEL, (0.0, 0.0, 0.0), P.unknown_clip, P)
    g.upload(phi.astype(np.float32), (phi <= P.max_surface).astype(np.int32))
    return g


@pytest.mark.parametrize("solver,iters", [("fused", 37), ("band", 37), ("band", 20), ("plain", 21),
                                          ("exact", 21), ("pervoxel", 50)])
def test_async_solve_equals_solve(gpu, solver, iters):
    P = gpu.Params.paper(VOXEL)
    can, live = small_pair(24, VOXEL, 5.0, seed=41)
    gl, gc = grid(gpu, live, P), grid(gpu, can, P)
    prec = gpu.KF_F64 if solver == "exact" else gpu.KF_F32
    a, b = gpu.Field(gl.dims, prec), gpu.Field(gl.dims, prec)
    want = gpu.psi_solve(gl, gc, a, P, iters, solver)
    gpu.psi_solve_async(gl, gc, b, P, iters, solver)
    # work queued behind the solve reads its result: warp + fuse on copies
    c1, c2 = grid(gpu, can, P), grid(gpu, can, P)
    l1, l2 = grid(gpu, live, P), grid(gpu, live, P)
    gpu.warp_fuse(c2, l2, b, P)
    got = gpu.psi_solve_wait(b)
    gpu.warp_fuse(c1, l1, a, P)
    np.testing.assert_array_equal(b.download(), a.download())
    for k in STATS:
        assert got[k] == want[k], k
    for x, y in ((c1, c2), (l1, l2)):
        np.testing.assert_array_equal(x.download()[0], y.download()[0])
        np.testing.assert_array_equal(x.download()[1], y.download()[1])


def test_async_solve_rules(gpu):
    P = gpu.Params.paper(VOXEL)
    can, live = small_pair(24, VOXEL, 5.0, seed=42)
    gl, gc = grid(gpu, live, P), grid(gpu, can, P)
    f = gpu.Field(gl.dims, gpu.KF_F32)
    with pytest.raises(gpu.KFError) as e:  # nothing queued
        gpu.psi_solve_wait(f)
    assert e.value.status == gpu.KF_ERR_INVALID
    gpu.psi_solve_async(gl, gc, f, P, 5, "fused")
    gpu.psi_solve_wait(f)
    with pytest.raises(gpu.KFError) as e:  # already read
        gpu.psi_solve_wait(f)
    assert e.value.status == gpu.KF_ERR_INVALID
    Pe = P.with_(early_exit=True, threshold=1e-4)
    with pytest.raises(gpu.KFError) as e:  # two buffers: where psi ends depends on the iterations run
        gpu.psi_solve_async(gl, gc, f, Pe, 50, "band")
    assert e.value.status == gpu.KF_ERR_INVALID
    a, b = gpu.Field(gl.dims, gpu.KF_F32), gpu.Field(gl.dims, gpu.KF_F32)
    Pr = gpu.Params.reference(VOXEL, 5.0).with_(early_exit=True, threshold=1e-4)
    want = gpu.psi_solve(gl, gc, a, Pr, 400, "fused")
    gpu.psi_solve_async(gl, gc, b, Pr, 400, "fused")
    got = gpu.psi_solve_wait(b)
    assert got["converged"] == want["converged"] == 1
    assert got["iterations_run"] == want["iterations_run"] < 400
    np.testing.assert_array_equal(b.download(), a.download())


def test_async_divergence_reported_at_wait(gpu):
    P = gpu.Params.reference(VOXEL, 5.0)
    can, live = small_pair(24, VOXEL, 5.0, seed=1)
    gl, gc = grid(gpu, live, P), grid(gpu, can, P)
    for solver in ("fused", "band"):
        f = gpu.Field(gl.dims, gpu.KF_F32)
        psi = np.zeros(live.shape + (3,))
        z, y, x = np.argwhere((live > -0.01) & (live < 0.01))[0]
        psi[z, y, x, 0] = np.nan
        f.upload(psi)
        gpu.psi_solve_async(gl, gc, f, P, 6, solver)
        with pytest.raises(gpu.DivergedError):
            gpu.psi_solve_wait(f)


def test_marching_cubes_async(gpu):
    import torch
    P = gpu.Params.paper(VOXEL)
    can, _ = small_pair(24, VOXEL, 5.0, seed=43)
    g = grid(gpu, can, P)
    want = gpu.marching_cubes(g, P)
    n = len(want)
    assert n > 100
    L = gpu.load()
    buf = torch.full((n + 10, 9), -7.0, dtype=torch.float32, device="cuda")
    for where in ("cuda", "pinned"):
        cnt = torch.zeros(1, dtype=torch.int64, device="cuda") if where == "cuda" else \
            torch.zeros(1, dtype=torch.int64).pin_memory()
        gpu.check(L.kf_marching_cubes_async(g.h, C.byref(P.c()), buf.data_ptr(), n + 10, cnt.data_ptr(), None))
        torch.cuda.synchronize()
        assert int(cnt.item()) == n
        np.testing.assert_array_equal(buf[:n].cpu().numpy().reshape(-1, 3, 3), want)
        assert (buf[n:] == -7.0).all()
    # a buffer smaller than the mesh: the first triangles, the full count
    small = torch.zeros((50, 9), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    gpu.check(L.kf_marching_cubes_async(g.h, C.byref(P.c()), small.data_ptr(), 50, cnt.data_ptr(), None))
    torch.cuda.synchronize()
    assert int(cnt.item()) == n
    np.testing.assert_array_equal(small.cpu().numpy().reshape(-1, 3, 3), want[:50])
    # the count must land where the device can write it
    pageable = np.zeros(1, np.int64)
    st = L.kf_marching_cubes_async(g.h, C.byref(P.c()), buf.data_ptr(), n, pageable.ctypes.data, None)
    assert st == gpu.KF_ERR_INVALID


def test_pipeline_keeps_canonical_when_solve_diverges(gpu):
    """kf_fusion_process_frame reads the solve's status before warp + fuse:
    a diverging frame returns KF_ERR_DIVERGED and the canonical SDF is as it
    was."""
    from killingfusion_gb300 import synth
    grid_, frames = synth.sphere_pair()
    P = gpu.Params.paper(grid_.voxel)
    # NaN depth on the object passes the reference's range test
    # (SDF.cpp:178) and integrates NaN distances: psi turns non-finite
    bad = frames[1].copy()
    bad[230:250, 310:330] = np.nan
    fu = gpu.Fusion(grid_.dims, grid_.voxel, grid_.origin, P, iterations=20, solver="fused")
    fu.process_frame(frames[0])
    can, _, _ = fu.state()
    shape = tuple(grid_.dims[::-1])

    def download():
        phi, w = np.empty(shape, np.float32), np.empty(shape, np.int32)
        gpu.check(gpu.load().kf_grid_download(can, phi.ctypes.data, w.ctypes.data, None))
        return phi, w

    before = download()
    with pytest.raises(gpu.DivergedError):
        fu.process_frame(bad)
    after = download()
    assert np.any(before[1] > 0)
    np.testing.assert_array_equal(before[0], after[0])
    np.testing.assert_array_equal(before[1], after[1])
