"""Parity at the benchmark workloads' full sizes.

256^3 ellipsoid sequence (5 mm voxels, 200 Jacobi iterations at the paper
weights: the grid and frame of the bench line), against the FP64 oracle on
the same inputs:
* integration of two frames (SDF::integrateDepthFrame, SDF.cpp:137-197):
  weights exact, SDF values the oracle's doubles rounded to float32;
* the float64 exact solver, 5 iterations (KillingFusion.cpp:248-352): psi
  bit-identical;
* the float32 dense fused solver over the frame's 200 iterations: psi and
  statistics bit-identical to the band-only solver, psi zero wherever the
  first iteration's band test failed (a voxel outside the band keeps psi),
  the band never growing;
* warp + fuse (SDF::update + SDF::fuse, SDF.cpp:199-241, 300-328) with that
  psi: weights exact, values the oracle's doubles rounded;
* marching cubes (SDF::getMesh, SDF.cpp:396-414) of the live, registered
  and canonical SDFs: triangle counts exact, vertices within 1e-4 voxel.

512^3 capsule sequence (2 mm voxels, 300 iterations, the large-grid
workload): integration and marching cubes against the oracle, the dense
fused solve against the band-only solve.
"""
import numpy as np
import pytest

from killingfusion_gb300 import synth
from oracle.oracle import Params as OParams

pytestmark = pytest.mark.gpu

VERTEX_TOL = 1e-4  # voxel


def oparams(p):
    return OParams(**{k: getattr(p, k) for k in OParams.__dataclass_fields__})


def f32(a):
    return np.asarray(a).astype(np.float32).astype(np.float64)


def integrate_both(capi, oracle, seq, P, frame, max_depth):
    g = seq.grid
    grid = capi.Grid(g.dims, g.voxel, g.origin, P.unknown_clip, P)
    depth = seq.frame(frame)
    grid.integrate(depth, min_depth=0.05, max_depth=max_depth)
    phi, w = grid.download()
    OP = oparams(P)
    shape = g.dims[::-1]
    ophi, ow = oracle.integrate(np.full(shape, OP.max_surface + OP.epsilon), np.zeros(shape, np.int64),
                                g.voxel, g.origin, OP.unknown_clip, depth.astype(np.float64), np.eye(4),
                                synth.K, 0.05, max_depth)
    np.testing.assert_array_equal(w, ow)
    np.testing.assert_array_equal(phi, ophi.astype(np.float32))
    assert (w > 0).sum() > 10000
    return grid, phi, w


def assert_mesh(capi, oracle, grid, phi64, P):
    tris = capi.marching_cubes(grid, P)
    otris = oracle.mesh(phi64, oparams(P))
    assert tris.shape == otris.shape and len(tris) > 1000
    err_vox = np.abs(tris - otris).max() / (2.0 / max(grid.dims))
    assert err_vox <= VERTEX_TOL, err_vox
    return len(tris)


def solve_pair(capi, live, can, P, iters):
    out, st = {}, {}
    for solver in ("fused", "band"):
        f = capi.Field(live.dims, capi.KF_F32)
        st[solver] = capi.psi_solve(live, can, f, P, iters, solver)
        out[solver] = f.download()
        f.close()
    np.testing.assert_array_equal(out["fused"], out["band"])
    for k in ("iterations_run", "active_first", "active_last", "max_delta_last", "converged", "diverged"):
        assert st["fused"][k] == st["band"][k], k
    return out["fused"], st["fused"]


def band_mask(live, P):
    """Voxels whose first band test passes: psi = 0, so the warped value is
    the voxel's own (KillingFusion.cpp:272-274), compared in double."""
    live = live.astype(np.float64)
    return (live <= P.max_surface - P.epsilon) & (live >= -P.unknown_clip)


def test_ellipsoid_256_frame(gpu, oracle):
    seq = synth.EllipsoidSequence(seed=2, frames=30, n=256)
    P = gpu.Params.paper(seq.grid.voxel)
    OP = oparams(P)
    can, cphi, cw = integrate_both(gpu, oracle, seq, P, 0, 1.6)
    live, lphi, lw = integrate_both(gpu, oracle, seq, P, 3, 1.6)
    shape = seq.grid.dims[::-1]

    # float64 exact solver: bit-identical to the oracle
    f64 = gpu.Field(live.dims, gpu.KF_F64)
    st = gpu.psi_solve(live, can, f64, P, 5, "exact")
    ost, opsi = oracle.solve(lphi.astype(np.float64), cphi.astype(np.float64), np.zeros(shape + (3,)), 5, OP)
    assert ost == 0 and st["iterations_run"] == 5
    np.testing.assert_array_equal(f64.download(), opsi)
    f64.close()
    del opsi

    # float32 dense fused solve over the frame's 200 iterations
    psi, st = solve_pair(gpu, live, can, P, 200)
    band = band_mask(lphi, P)
    assert st["active_first"] == int(band.sum()) > 10000
    assert 0 < st["active_last"] <= st["active_first"]
    assert not np.any(psi[~band]), "a voxel outside the first band moved"
    assert np.abs(psi).max() > 0.05

    # the live mesh, then warp + fuse with the solved psi, then both meshes
    ntri_live = assert_mesh(gpu, oracle, live, lphi.astype(np.float64), P)
    f = gpu.Field(live.dims, gpu.KF_F32)
    f.upload(psi)
    gpu.warp_fuse(can, live, f, P)
    uphi, uw = oracle.update(lphi.astype(np.float64), lw.astype(np.int64), psi.astype(np.float64), OP)
    gphi, gw = live.download()
    np.testing.assert_array_equal(gw, uw)
    np.testing.assert_array_equal(gphi, uphi.astype(np.float32))
    fphi, fw = oracle.fuse(cphi.astype(np.float64), cw.astype(np.int64), f32(uphi), uw)
    gphi, gw = can.download()
    np.testing.assert_array_equal(gw, fw)
    np.testing.assert_array_equal(gphi, fphi.astype(np.float32))
    assert assert_mesh(gpu, oracle, live, f32(uphi), P) > 0
    assert assert_mesh(gpu, oracle, can, f32(fphi), P) >= ntri_live // 2
    for g in (f, live, can):
        g.close()


def test_capsules_512_frame(gpu, oracle):
    seq = synth.CapsuleSequence(seed=5, frames=100, n=512)
    P = gpu.Params.paper(seq.grid.voxel)
    can, cphi, _ = integrate_both(gpu, oracle, seq, P, 0, 1.6)
    live, lphi, _ = integrate_both(gpu, oracle, seq, P, 10, 1.6)
    assert_mesh(gpu, oracle, live, lphi.astype(np.float64), P)
    del cphi
    psi, st = solve_pair(gpu, live, can, P, 300)
    band = band_mask(lphi, P)
    assert st["active_first"] == int(band.sum()) > 10000
    assert 0 < st["active_last"] <= st["active_first"]
    assert not np.any(psi[~band])
    for g in (live, can):
        g.close()
