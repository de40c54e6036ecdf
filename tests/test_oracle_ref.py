"""The FP64 restatement against the reference's own code on fresh seeded
inputs (needs the reference checkout; oracle/_ref is built from it)."""
import numpy as np
import pytest

from oracle import build as obuild
from oracle.oracle import Params, RefLib
from helpers import small_pair

pytestmark = pytest.mark.skipif(not obuild.reference_available(), reason="reference checkout absent")

PARAMS = {
    "reference": Params(voxel_size=0.004, unknown_clip=0.02, max_surface=0.02),
    "paper": Params.paper(0.004),
    "gamma0": Params.paper(0.004).with_(gamma_k=0.0),
    "no_levelset": Params.paper(0.004).with_(use_levelset=False),
}


@pytest.mark.parametrize("name", sorted(PARAMS))
def test_voxel_queries_bitexact(oracle, name):
    P = PARAMS[name]
    R = RefLib(P, 1)
    can, live = small_pair(20, P.voxel_size, 5.0, seed=3)
    rng = np.random.default_rng(4)
    psi = rng.normal(0.0, 0.6, live.shape + (3,))
    # a few large displacements that leave the grid (wrap / outside values)
    psi.reshape(-1, 3)[rng.integers(0, psi.size // 3, 50)] *= 20
    z, y, x = np.meshgrid(*[np.arange(20)] * 3, indexing="ij")
    xyz = np.stack([x, y, z], -1).reshape(-1, 3)
    for what in ("grad", "dgrad", "hess", "killing", "warped", "active"):
        a = oracle.voxel_query(what, live, can, psi, xyz, P)
        b = R.voxel_query(what, live, can, psi, xyz)
        np.testing.assert_array_equal(a, b, err_msg=what)


@pytest.mark.parametrize("name", ["reference", "paper"])
def test_solve_bitexact(oracle, name):
    P = PARAMS[name]
    iters = 15
    R = RefLib(P, iters)
    can, live = small_pair(22, P.voxel_size, 5.0, seed=9)
    st1, p1 = oracle.solve(live, can, np.zeros(live.shape + (3,)), iters, P)
    st2, p2 = R.solve(live, can, np.zeros(live.shape + (3,)))
    assert st1 == st2 == 0
    np.testing.assert_array_equal(p1, p2)


@pytest.mark.parametrize("alpha", [0.1, 0.5, 2.0])
def test_solve_trust_region_bitexact(oracle, alpha):
    """UseTrustStrategy with the data term alone (KillingFusion.cpp:288-314),
    including the break out of a row's x loop when the step size underflows."""
    P = Params.paper(0.004).with_(use_levelset=False, use_killing=False, use_trust=True, alpha=alpha)
    iters = 5
    R = RefLib(P, iters)
    can, live = small_pair(22, P.voxel_size, 5.0, seed=9)
    st1, p1 = oracle.solve(live, can, np.zeros(live.shape + (3,)), iters, P)
    st2, p2 = R.solve(live, can, np.zeros(live.shape + (3,)))
    assert st1 == st2 == 0
    np.testing.assert_array_equal(p1, p2)
    # with the level-set or Killing term the reference skips the strategy
    Pk = P.with_(use_killing=True)
    st3, p3 = oracle.solve(live, can, np.zeros(live.shape + (3,)), 2, Pk)
    st4, p4 = RefLib(Pk, 2).solve(live, can, np.zeros(live.shape + (3,)))
    assert st3 == st4 == 0
    np.testing.assert_array_equal(p3, p4)


def test_warp_fuse_mesh_bitexact(oracle):
    P = PARAMS["paper"]
    R = RefLib(P, 1)
    can, live = small_pair(20, P.voxel_size, 5.0, seed=13)
    rng = np.random.default_rng(2)
    psi = rng.normal(0.0, 0.4, live.shape + (3,))
    wl = rng.integers(0, 3, live.shape).astype(np.int64)
    wc = rng.integers(0, 3, live.shape).astype(np.int64)
    a = oracle.update(live, wl, psi, P)
    b = R.update(live, wl, psi)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(oracle.fuse(can, wc, *a)[0], R.fuse(can, wc, *b)[0])
    c = oracle.fuse_psi(can, wc, live, wl, psi, P)
    d = R.fuse_psi(can, wc, live, wl, psi)
    np.testing.assert_array_equal(c[0], d[0])
    np.testing.assert_array_equal(c[1], d[1])
    for phi in (can, live, a[0], c[0]):
        np.testing.assert_array_equal(oracle.mesh(phi, P), R.mesh(phi))


def test_integrate_bitexact_sphere_frames(oracle):
    from killingfusion_gb300 import synth
    P = Params.paper(0.004)
    R = RefLib(P, 1)
    grid, frames = synth.sphere_pair()
    n = grid.dims[::-1]
    for f in frames:
        phi = np.full(n, P.max_surface + P.epsilon)
        w = np.zeros(n, np.int64)
        a = oracle.integrate(phi, w, grid.voxel, grid.origin, P.unknown_clip, f.astype(np.float64),
                             np.eye(4), synth.K, 0.05, 1.2)
        b = R.integrate(phi, w, grid.voxel, grid.origin, P.unknown_clip, f.astype(np.float64),
                        np.eye(4), synth.K, 0.05, 1.2)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
        assert (a[1] > 0).sum() > 1000


def test_grid_size_rule():
    """SDF::computeVoxelGridSize: int(bound / voxel) + 1 (SDF.cpp:117-124);
    the synthetic grids pick bounds that give their sizes exactly."""
    from killingfusion_gb300 import synth
    R = RefLib(Params(), 1)
    for g in (synth.sphere_pair()[0], synth.EllipsoidSequence(n=64).grid):
        bound = g.max3d - g.origin
        np.testing.assert_array_equal(R.grid_size(bound, g.voxel), g.dims)
