"""The trust-region step of the Jacobi schedule on the GPU (UseTrustStrategy,
KillingFusion.cpp:288-314; kf_params.use_trust): taken with the data term
alone, it divides the step size by 1.5 while the step does not bring the
warped live value closer to the canonical one, and when the step size falls
below 1e-7 the reference breaks out of the row's x loop, leaving that voxel
and the rest of its row unchanged for the iteration.

* float64 solver: bit-identical to the oracle, which is pinned to the
  reference (tests/golden/trust_region.npz, test_oracle_ref.py);
* float32 solvers: the dense and band-only forms agree bit for bit; their
  step-size search runs in float64 (a float32 position cannot resolve the
  smallest trial steps), so against the oracle psi agrees within 1e-4 voxel
  after 1 and after 60 iterations; a decision at an exact tie could still
  flip, and a flipped break moves a whole row, so the bar leaves 1 % of the
  voxels to that and also compares the registration's data residual;
* the step is skipped with the level-set or Killing term, as the reference
  skips it; the per-term solver and batches reject it.
"""
import os

import numpy as np
import pytest

from oracle.oracle import Params as OParams
from helpers import sphere_frames

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def oparams(p):
    d = {k: getattr(p, k) for k in OParams.__dataclass_fields__}
    return OParams(**d)


def trust_params(gpu, voxel, alpha=0.1):
    return gpu.Params.paper(voxel).with_(use_levelset=False, use_killing=False, use_trust=True,
                                         alpha=alpha)


def grid_of(gpu, phi, voxel, P):
    nz, ny, nx = phi.shape
    g = gpu.Grid((nx, ny, nz), voxel, (0.0, 0.0, 0.0), P.unknown_clip, P)
    g.upload(phi.astype(np.float32), (phi <= P.max_surface).astype(np.int32))
    return g


def sphere_pair(gpu, oracle, P):
    """The 64^3 sphere pair integrated by the GPU, and its values for the
    oracle (integration is bit-exact, test_gpu_parity.py)."""
    grid, frames = sphere_frames()
    out = []
    for f in frames:
        g = gpu.Grid(grid.dims, grid.voxel, grid.origin, P.unknown_clip, P)
        g.integrate(f, min_depth=0.05, max_depth=1.2)
        out.append(g)
    can, live = out
    return can, live, can.download()[0].astype(np.float64), live.download()[0].astype(np.float64)


def test_exact_trust_matches_reference_fixture(gpu):
    """The reference's own psi (tests/golden/trust_region.npz) from the
    float64 solver, bit for bit, row break included."""
    g = np.load(os.path.join(GOLD, "trust_region.npz"))
    live, can = g["live"], g["can"]
    assert np.array_equal(live.astype(np.float32).astype(np.float64), live)
    voxel = 0.004
    P = trust_params(gpu, voxel)
    gl, gc = grid_of(gpu, live, voxel, P), grid_of(gpu, can, voxel, P)
    f = gpu.Field(gl.dims, gpu.KF_F64)
    st = gpu.psi_solve(gl, gc, f, P, int(g["iterations"]), "exact")
    assert st["iterations_run"] == int(g["iterations"])
    np.testing.assert_array_equal(f.download(), g["psi"])


@pytest.mark.parametrize("alpha", [0.1, 0.5])
def test_exact_trust_bitexact_64cubed(gpu, oracle, alpha):
    voxel = 0.004
    P = trust_params(gpu, voxel, alpha)
    can, live, ocan, olive = sphere_pair(gpu, oracle, P)
    f = gpu.Field(live.dims, gpu.KF_F64)
    st = gpu.psi_solve(live, can, f, P, 60, "exact")
    ost, opsi, counts = oracle.solve(olive, ocan, np.zeros(olive.shape + (3,)), 60, oparams(P),
                                     active_counts=True)
    assert ost == 0
    assert st["active_first"] == counts[0] and st["active_last"] == counts[-1]
    np.testing.assert_array_equal(f.download(), opsi)
    # the row breaks took effect: the plain step moves voxels that stay put here
    _, plain = oracle.solve(olive, ocan, np.zeros(olive.shape + (3,)), 60,
                            oparams(P.with_(use_trust=False)))
    assert np.abs(plain - opsi).max() > 0.1


def data_residual(oracle, olive, ocan, psi, P, band):
    """Sum over the band voxels of (phi_live(i + psi(i)) - phi_can(i))^2."""
    w = oracle.voxel_query("warped", olive, ocan, psi.astype(np.float64), band, oparams(P))[:, 0]
    return float(np.sum((w - ocan[band[:, 2], band[:, 1], band[:, 0]]) ** 2))


@pytest.mark.parametrize("alpha", [0.1, 0.5])
def test_fp32_trust_solvers(gpu, oracle, alpha):
    """Float32 dense and band-only forms agree bit for bit and follow the
    oracle within 1e-4 voxel (1 and 60 iterations)."""
    voxel = 0.004
    P = trust_params(gpu, voxel, alpha)
    can, live, ocan, olive = sphere_pair(gpu, oracle, P)
    zero = np.zeros(olive.shape + (3,))
    band = np.argwhere(np.ones(olive.shape, bool))[:, ::-1].astype(np.int32)
    act = oracle.voxel_query("active", olive, ocan, zero, band, oparams(P))[:, 0] > 0
    band = band[act]
    for iters in (1, 60):
        out, st = {}, {}
        for solver in ("fused", "band"):
            f = gpu.Field(live.dims, gpu.KF_F32)
            st[solver] = gpu.psi_solve(live, can, f, P, iters, solver)
            out[solver] = f.download()
        np.testing.assert_array_equal(out["band"], out["fused"])
        assert st["band"]["active_last"] == st["fused"]["active_last"]
        _, opsi, counts = oracle.solve(olive, ocan, zero, iters, oparams(P), active_counts=True)
        assert st["fused"]["active_first"] == counts[0] == len(band)
        err = np.abs(out["fused"].astype(np.float64) - opsi).max(axis=-1)
        close = (err <= 1e-4)[band[:, 2], band[:, 1], band[:, 0]].sum()
        r0 = data_residual(oracle, olive, ocan, zero, P, band)
        rg = data_residual(oracle, olive, ocan, out["fused"], P, band)
        ro = data_residual(oracle, olive, ocan, opsi, P, band)
        print("alpha %g, %d iterations: %d of %d band voxels within 1e-4 voxel; data residual "
              "%.4g -> gpu %.4g, oracle %.4g" % (alpha, iters, close, len(band), r0, rg, ro))
        assert close >= 0.99 * len(band)
        assert ro < r0 and rg < r0
        assert abs(rg - ro) <= 0.01 * (r0 - ro)


def test_trust_skipped_with_other_terms(gpu):
    """With the Killing term on, use_trust changes nothing (the reference's
    condition, KillingFusion.cpp:289)."""
    voxel = 0.004
    P = gpu.Params.paper(voxel)
    g = np.load(os.path.join(GOLD, "trust_region.npz"))
    gl, gc = grid_of(gpu, g["live"], voxel, P), grid_of(gpu, g["can"], voxel, P)
    out = []
    for trust in (False, True):
        f = gpu.Field(gl.dims, gpu.KF_F32)
        gpu.psi_solve(gl, gc, f, P.with_(use_trust=trust), 20, "fused")
        out.append(f.download())
    np.testing.assert_array_equal(out[0], out[1])


def test_trust_rejected_where_not_run(gpu):
    voxel = 0.004
    P = trust_params(gpu, voxel)
    g = np.load(os.path.join(GOLD, "trust_region.npz"))
    gl, gc = grid_of(gpu, g["live"], voxel, P), grid_of(gpu, g["can"], voxel, P)
    f = gpu.Field(gl.dims, gpu.KF_F32)
    with pytest.raises(gpu.KFError) as e:
        gpu.psi_solve(gl, gc, f, P, 5, "plain")
    assert e.value.status == gpu.KF_ERR_INVALID
    with pytest.raises(gpu.KFError) as e:
        gpu.Batch([(gl, gc, f, P)], 5)
    assert e.value.status == gpu.KF_ERR_INVALID
    # the per-voxel schedule has no trust-region step: use_trust is ignored
    a, b = gpu.Field(gl.dims, gpu.KF_F32), gpu.Field(gl.dims, gpu.KF_F32)
    gpu.psi_solve(gl, gc, a, P, 50, "pervoxel")
    gpu.psi_solve(gl, gc, b, P.with_(use_trust=False), 50, "pervoxel")
    np.testing.assert_array_equal(a.download(), b.download())
