"""The per-iteration energy statistic is accumulated in float64 end to end.

Each band voxel's monitored energy is a float32 value; the per-thread
partials, the block sums and the grid sum are float64.  With the data term
alone and psi = 0, a voxel's energy is 0.5 * ((phi_live - phi_can) / v)^2
evaluated in float32 with one rounding per operation (the warped value at
psi = 0 is phi_live itself), which numpy reproduces bit for bit.  The exact
sum of those values then pins the GPU's total to within float64 summation
error (1e-11 relative here), on a grid where every voxel is in the band and
each thread of the band pass takes dozens of voxels; float32 partials would
be off by about 1e-7.  The batched solver's per-problem totals are checked
the same way.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-11


def band_fields(n, voxel, trunc, seed):
    """Two smooth fields strictly inside the band (every voxel active)."""
    rng = np.random.default_rng(seed)
    ax = (np.arange(n) + 0.5) / n
    Z, Y, X = np.meshgrid(ax, ax, ax, indexing="ij")
    k = rng.uniform(1.0, 4.0, (2, 3))
    ph = rng.uniform(0, 2 * np.pi, (2, 3))
    f = [0.3 * trunc * (np.sin(2 * np.pi * (k[j, 0] * X + ph[j, 0])) + np.sin(2 * np.pi * (k[j, 1] * Y + ph[j, 1]))
                        + np.sin(2 * np.pi * (k[j, 2] * Z + ph[j, 2]))) for j in range(2)]
    return f[0].astype(np.float32), f[1].astype(np.float32)


def float_data_energy(live, can, voxel):
    r = (live - can) / np.float32(voxel)              # float32, one rounding each
    e = (np.float32(0.5) * r).astype(np.float64) * r.astype(np.float64)
    return e.astype(np.float32).astype(np.float64)    # the fused multiply-add's single rounding


def data_only(capi, voxel):
    return capi.Params.reference(voxel, 5.0).with_(use_levelset=False, use_killing=False)


def test_band_solver_energy_sum(gpu):
    capi = gpu
    n, voxel = 160, 0.005
    P = data_only(capi, voxel)
    live, can = band_fields(n, voxel, P.max_surface, seed=7)
    assert np.all(np.abs(live) < P.max_surface - P.epsilon) and np.all(np.abs(can) < P.max_surface)
    dims = (n, n, n)
    gl = capi.Grid(dims, voxel, (0, 0, 0), P.unknown_clip, P)
    gc = capi.Grid(dims, voxel, (0, 0, 0), P.unknown_clip, P)
    gl.upload(live, np.ones(live.shape, np.int32))
    gc.upload(can, np.ones(can.shape, np.int32))
    expect = math.fsum(float_data_energy(live, can, voxel).ravel())
    for solver in ("band", "fused"):
        f = capi.Field(dims, capi.KF_F32)
        st = capi.psi_solve(gl, gc, f, P, 1, solver)
        assert st["active_first"] == n ** 3  # ~54 voxels per band-pass thread
        rel = abs(st["energy_first"] - expect) / expect
        assert rel <= REL_TOL, (solver, st["energy_first"], expect, rel)
        f.close()


def test_batch_energy_sums(gpu):
    capi = gpu
    probs, expect = [], []
    for k, n in enumerate((96, 120)):
        voxel = 0.004 + 0.001 * k
        P = data_only(capi, voxel)
        live, can = band_fields(n, voxel, P.max_surface, seed=20 + k)
        dims = (n, n, n)
        gl = capi.Grid(dims, voxel, (0, 0, 0), P.unknown_clip, P)
        gc = capi.Grid(dims, voxel, (0, 0, 0), P.unknown_clip, P)
        gl.upload(live, np.ones(live.shape, np.int32))
        gc.upload(can, np.ones(can.shape, np.int32))
        probs.append((gl, gc, capi.Field(dims, capi.KF_F32), P))
        expect.append(math.fsum(float_data_energy(live, can, voxel).ravel()))
    batch = capi.Batch(probs, 1)
    stats = batch.run()
    for st, e, (gl, _, _, _) in zip(stats, expect, probs):
        assert st["active_first"] == int(np.prod(gl.dims))
        assert abs(st["energy_first"] - e) / e <= REL_TOL, (st["energy_first"], e)
    batch.close()
