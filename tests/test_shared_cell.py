"""The band pass's shared corner cell against its per-sample gathers.

For an interior band voxel the 25 cell-centre samples of the gradient and
Hessian usually fall into one cell of phi_live, whose eight corners the
band pass then loads once; when the samples straddle a cell face each one
gathers its own corners.  A rough psi (a few voxels with per-voxel noise)
sends a large share of the band through each form.  One Jacobi iteration
of every float32 solver must then agree with the FP64 oracle run from the
same psi (the derivative samples are the reference's, SDF.cpp:726-744 and
842-886), and the solvers with one another bit for bit.
"""
import numpy as np
import pytest

from oracle.oracle import Params as OParams
from helpers import small_pair

pytestmark = pytest.mark.gpu

PSI_TOL = 1e-4  # voxel


def oparams(p):
    return OParams(**{k: getattr(p, k) for k in OParams.__dataclass_fields__})


def rough_psi(shape, seed):
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    smooth = np.stack([np.sin(0.31 * x + 0.17 * z), np.cos(0.23 * y - 0.29 * x), np.sin(0.19 * z + 0.41 * y)], -1)
    return (1.4 * smooth + rng.normal(0.0, 0.35, shape + (3,))).astype(np.float32)


def shared_fraction(psi, band, h):
    """Share of the interior band voxels whose samples keep one cell (the
    band pass's test, without its rounding margin)."""
    nz, ny, nx = band.shape
    inner = np.zeros_like(band)
    inner[1:-1, 1:-1, 1:-1] = True
    z, y, x = np.nonzero(band & inner)
    ok = np.ones(len(x), bool)
    for c, coord in enumerate((x, y, z)):
        p = psi[..., c].astype(np.float64)

        def k(dx, dy, dz):
            return p[z + dz, y + dy, x + dx]
        k000, k100, k010, k110 = k(0, 0, 0), k(1, 0, 0), k(0, 1, 0), k(1, 1, 0)
        k001, k101, k011, k111 = k(0, 0, 1), k(1, 0, 1), k(0, 1, 1), k(1, 1, 1)
        sx0, sx1 = k000 + k010 + k001 + k011, k100 + k110 + k101 + k111
        sy0, sy1 = k000 + k100 + k001 + k101, k010 + k110 + k011 + k111
        sz0, sz1 = k000 + k100 + k010 + k110, k001 + k101 + k011 + k111
        m0 = 0.125 * (sx0 + sx1)
        m1 = 0.25 * (np.abs(sx1 - sx0) + np.abs(sy1 - sy0) + np.abs(sz1 - sz0))
        m4 = 0.5 * np.abs((k110 - k010) - (k100 - k000) + (k111 - k011) - (k101 - k001))
        m5 = 0.5 * np.abs((k101 - k001) - (k100 - k000) + (k111 - k011) - (k110 - k010))
        m6 = 0.5 * np.abs((k011 - k001) - (k010 - k000) + (k111 - k101) - (k110 - k100))
        r = h * (2 + 2 * m1 + h * (m4 + m5 + m6))
        ctr = coord + 0.5 + m0
        ok &= (np.floor(ctr - r) == np.floor(ctr + r)) & (ctr - r >= 0)
        ok &= (np.floor(ctr - r) <= band.shape[2 - c] - 2)
    return ok.mean(), len(x)


@pytest.mark.parametrize("weights", ["reference", "paper"])
def test_one_iteration_from_rough_psi(gpu, oracle, weights):
    voxel = 0.004
    P = gpu.Params.reference(voxel, 5.0) if weights == "reference" else gpu.Params.paper(voxel)
    OP = oparams(P)
    can, live = small_pair(40, voxel, 5.0, seed=41)
    nz, ny, nx = live.shape
    psi0 = rough_psi(live.shape, 7)
    l64 = live.astype(np.float64)
    # both forms run: measured over the voxels near the surface
    frac, nnear = shared_fraction(psi0, np.abs(l64) < P.unknown_clip, P.delta_size)
    assert nnear > 2000 and 0.1 < frac < 0.9, (frac, nnear)

    def grid(phi):
        g = gpu.Grid((nx, ny, nz), voxel, (0.0, 0.0, 0.0), P.unknown_clip, P)
        g.upload(phi, (phi <= P.max_surface).astype(np.int32))
        return g

    gl, gc = grid(live), grid(can)
    _, opsi = oracle.solve(l64, can.astype(np.float64), psi0.astype(np.float64), 1, OP)
    moved = np.any(opsi != psi0, axis=-1)
    assert moved.sum() > 1000
    out = {}
    for solver in ("fused", "band"):
        f = gpu.Field(gl.dims, gpu.KF_F32)
        f.upload(psi0)
        gpu.psi_solve(gl, gc, f, P, 1, solver)
        out[solver] = f.download()
        err = np.abs(out[solver] - opsi).max()
        assert err <= PSI_TOL, (solver, err)
    np.testing.assert_array_equal(out["fused"], out["band"])
    # the batched band pass (its own kernel and launch shapes) gives the same bits
    fb = gpu.Field(gl.dims, gpu.KF_F32)
    fb.upload(psi0)
    batch = gpu.Batch([(gl, gc, fb, P)], 1)
    batch.autotune()
    fb.upload(psi0)
    batch.run()
    batch.close()
    np.testing.assert_array_equal(fb.download(), out["band"])
    # the float64 solver replays the oracle exactly
    f = gpu.Field(gl.dims, gpu.KF_F64)
    f.upload(psi0.astype(np.float64))
    gpu.psi_solve(gl, gc, f, P, 1, "exact")
    np.testing.assert_array_equal(f.download(), opsi)
