"""kf_fusion_process_frame (KillingFusion::processNextFrame,
KillingFusion.cpp:109-175) against the oracle replaying the same frames:
integration, the psi solve (float64 exact solver: bit-identical), warp +
fuse and the three meshes of every frame."""

import numpy as np
import pytest

from killingfusion_gb300 import synth
from oracle.oracle import Params as OParams

pytestmark = pytest.mark.gpu


def oparams(p):
    d = {k: getattr(p, k) for k in OParams.__dataclass_fields__}
    return OParams(**d)


def f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def download(capi, grid_handle, field_handle, shape):
    L = capi.load()
    phi = np.empty(shape, np.float32)
    w = np.empty(shape, np.int32)
    capi.check(L.kf_grid_download(grid_handle, phi.ctypes.data, w.ctypes.data, None))
    psi = None
    if field_handle is not None:
        psi = np.empty(shape + (3,), np.float64)
        capi.check(L.kf_field_download(field_handle, psi.ctypes.data, None))
    return phi, w, psi


def assert_soup(got, want, voxel_tol):
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=0, atol=voxel_tol)


@pytest.mark.parametrize("iters", [10])
def test_pipeline_matches_oracle(gpu, oracle, iters):
    grid, frames = synth.sphere_pair()
    frames = frames + [synth.sphere_pair(seed=9)[1][1]]
    P = gpu.Params.paper(grid.voxel)
    OP = oparams(P)
    fu = gpu.Fusion(grid.dims, grid.voxel, grid.origin, P, iterations=iters, solver="exact")
    shape = grid.dims[::-1]
    init = f32(np.full(shape, OP.max_surface + OP.epsilon))
    # mesh vertices are float32 in [-1, 1]: compare to 1e-5 of the half-extent
    tol = 1e-5

    def integrate(frame):
        phi, w = oracle.integrate(init, np.zeros(shape, np.int64), grid.voxel, grid.origin,
                                  OP.unknown_clip, frame.astype(np.float64), np.eye(4), synth.K,
                                  0.05, 1.2)
        return f32(phi), w

    r = fu.process_frame(frames[0])
    assert r["frame"] == 1 and r["solve"]["iterations_run"] == 0
    can, cw = integrate(frames[0])
    assert_soup(r["live"], oracle.mesh(can, OP), tol)
    reg, _ = oracle.fuse_psi(init, np.zeros(shape, np.int64), can, cw, np.zeros(shape + (3,)), OP)
    assert_soup(r["registered"], oracle.mesh(f32(reg), OP), tol)
    assert_soup(r["canonical"], oracle.mesh(can, OP), tol)
    hc, hl, hf = fu.state()
    phi, w, _ = download(gpu, hc, None, shape)
    np.testing.assert_array_equal(phi, can.astype(np.float32))
    np.testing.assert_array_equal(w, cw)
    for k in (1, 2):
        r = fu.process_frame(frames[k])
        assert r["frame"] == k + 1 and r["solve"]["iterations_run"] == iters
        live, lw = integrate(frames[k])
        st, psi = oracle.solve(live, can, np.zeros(shape + (3,)), iters, OP)
        assert st == 0
        _, _, gpsi = download(gpu, hl, hf, shape)
        np.testing.assert_array_equal(gpsi, psi)
        assert_soup(r["live"], oracle.mesh(live, OP), tol)
        uphi, uw = oracle.update(live, lw, psi, OP)
        uphi = f32(uphi)
        fphi, cw = oracle.fuse(can, cw, uphi, uw)
        can = f32(fphi)
        assert_soup(r["registered"], oracle.mesh(uphi, OP), tol)
        assert_soup(r["canonical"], oracle.mesh(can, OP), tol)
        phi, w, _ = download(gpu, hc, None, shape)
        np.testing.assert_array_equal(w, cw)
        np.testing.assert_array_equal(phi, can.astype(np.float32))
    fu.close()


def test_pipeline_solvers_agree(gpu):
    """The float32 solvers through the pipeline: band-only equals dense
    fused bit for bit, frame after frame."""
    grid, frames = synth.sphere_pair()
    P = gpu.Params.paper(grid.voxel)
    out = {}
    for solver in ("fused", "band"):
        fu = gpu.Fusion(grid.dims, grid.voxel, grid.origin, P, iterations=50, solver=solver)
        res = [fu.process_frame(f) for f in frames + frames[:1]]
        hc, _, _ = fu.state()
        out[solver] = (download(gpu, hc, None, grid.dims[::-1])[:2], [r["ntri"] for r in res])
        fu.close()
    np.testing.assert_array_equal(out["fused"][0][0], out["band"][0][0])
    np.testing.assert_array_equal(out["fused"][0][1], out["band"][0][1])
    assert out["fused"][1] == out["band"][1]
