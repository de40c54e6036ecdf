"""The dense fused solver's split schedule, on grids of at least 512 runs of
2048 voxels (about 1 M voxels and up).

After the first iteration the runs that listed no band voxel are streamed on
a second stream, beside the band pass, while the runs that did keep the
stream -> band order.  Whatever the grid's shape, the starting psi, the
iteration count or the way the loop ends (fixed count, convergence,
divergence), psi, the band counts and the statistics must equal the
band-only solver's bit for bit.  The band-only solver is pinned to the dense
two-pass schedule and, through it, to the oracle by the small-grid tests
(test_gpu_parity.py, test_edge_cases.py)."""
import numpy as np
import pytest

from killingfusion_gb300 import synth

pytestmark = pytest.mark.gpu

KEYS = ("iterations_run", "active_first", "active_last", "max_delta_last", "converged", "diverged")


def ellipsoid_pair(capi, n, params="paper"):
    """Frames 0 and 3 of the ellipsoid sequence on an n^3 grid."""
    seq = synth.EllipsoidSequence(seed=2, frames=30, n=n)
    g = seq.grid
    P = capi.Params.paper(g.voxel) if params == "paper" else capi.Params.reference(g.voxel, 5.0)
    can = capi.Grid(g.dims, g.voxel, g.origin, P.unknown_clip, P)
    live = capi.Grid(g.dims, g.voxel, g.origin, P.unknown_clip, P)
    can.integrate(seq.frame(0), max_depth=1.6)
    live.integrate(seq.frame(3), max_depth=1.6)
    return can, live, P


def solve_both(capi, live, can, P, iters, psi0=None):
    out, st = {}, {}
    for solver in ("fused", "band"):
        f = capi.Field(live.dims, capi.KF_F32)
        if psi0 is not None:
            f.upload(psi0)
        st[solver] = capi.psi_solve(live, can, f, P, iters, solver)
        out[solver] = f.download()
    return out, st


def assert_same(out, st):
    np.testing.assert_array_equal(out["fused"], out["band"])
    for k in KEYS:
        assert st["fused"][k] == st["band"][k], k


@pytest.mark.parametrize("n,iters", [(128, 1), (128, 2), (128, 37), (128, 200), (256, 40)])
def test_split_schedule_equals_band_solver(gpu, n, iters):
    can, live, P = ellipsoid_pair(gpu, n)
    out, st = solve_both(gpu, live, can, P, iters)
    assert_same(out, st)
    assert st["fused"]["active_first"] > 1000
    if iters > 1:
        assert np.abs(out["fused"]).max() > 0.05  # the field moved


def ellipsoid_sdf(dims, centre, axes, voxel, trunc):
    """Approximate truncated SDF (metres, float32) of an axis-aligned
    ellipsoid on a (nx, ny, nz) grid, voxel centres at i + 0.5."""
    nx, ny, nz = dims
    Z, Y, X = np.meshgrid(np.arange(nz) + 0.5, np.arange(ny) + 0.5, np.arange(nx) + 0.5, indexing="ij")
    q = np.sqrt(((X - centre[0]) / axes[0]) ** 2 + ((Y - centre[1]) / axes[1]) ** 2 +
                ((Z - centre[2]) / axes[2]) ** 2)
    d = (q - 1.0) * min(axes) * voxel
    return np.where(d > trunc, trunc + 1e-5, d).astype(np.float32)


def test_split_schedule_ragged_grid_moved_start(gpu):
    """A non-cubic grid whose voxel count is not a multiple of 4 (the last
    voxels are taken by run 0 outside the 16-byte groups), started from a
    psi that is non-zero everywhere, so every voxel of every run -- hot and
    cold -- takes the moved-voxel path of the band test."""
    dims = (161, 163, 165)
    assert (dims[0] * dims[1] * dims[2]) % 4 == 3
    voxel = 0.004
    P = gpu.Params.paper(voxel)
    trunc = voxel * 5.0
    can = ellipsoid_sdf(dims, (80.3, 81.7, 82.1), (40.0, 34.0, 45.0), voxel, trunc)
    live = ellipsoid_sdf(dims, (81.1, 80.9, 83.0), (41.5, 33.0, 44.0), voxel, trunc)
    gc = gpu.Grid(dims, voxel, (0.0, 0.0, 0.0), P.unknown_clip, P)
    gl = gpu.Grid(dims, voxel, (0.0, 0.0, 0.0), P.unknown_clip, P)
    gc.upload(can, (can <= P.max_surface).astype(np.int32))
    gl.upload(live, (live <= P.max_surface).astype(np.int32))
    nx, ny, nz = dims
    Z, Y, X = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    psi0 = np.stack([0.3 * np.sin(X / 17.0 + 0.4), 0.2 * np.cos(Y / 23.0), 0.25 * np.sin(Z / 11.0 - 1.0)],
                    axis=-1).astype(np.float32)
    assert (psi0 != 0).all(axis=-1).mean() > 0.99
    out, st = solve_both(gpu, gl, gc, P, 30, psi0)
    assert_same(out, st)
    assert st["fused"]["active_first"] > 1000


def test_split_schedule_early_exit(gpu):
    """The loop stops once max |dpsi| <= threshold; the cold passes queued
    after convergence change nothing."""
    can, live, P = ellipsoid_pair(gpu, 128, "reference")
    f = gpu.Field(live.dims, gpu.KF_F32)
    probe = gpu.psi_solve(live, can, f, P, 60, "band")
    # at most the last step of the 60-iteration probe: the loop must stop by iteration 61
    Q = P.with_(early_exit=True, threshold=float(probe["max_delta_last"]) * 1.0001)
    out, st = solve_both(gpu, live, can, Q, 400, None)
    assert_same(out, st)
    assert st["fused"]["converged"] == 1 and st["fused"]["iterations_run"] <= 61


def test_split_schedule_divergence(gpu):
    """A non-finite psi inside the band stops the solve with KF_ERR_DIVERGED."""
    can, live, P = ellipsoid_pair(gpu, 128)
    phi, _ = live.download()
    z, y, x = np.argwhere((phi > -0.005) & (phi < 0.005))[0]
    psi = np.zeros(phi.shape + (3,), np.float32)
    psi[z, y, x, 1] = np.nan
    f = gpu.Field(live.dims, gpu.KF_F32)
    f.upload(psi)
    with pytest.raises(gpu.DivergedError):
        gpu.psi_solve(live, can, f, P, 20, "fused")
