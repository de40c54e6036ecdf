"""Edge cases of the GPU path against the oracle: grids whose voxel count is
not a multiple of the 4-voxel vectors or of the dense pass's 2048-voxel runs,
non-cubic grids, grids one voxel thick, single-voxel grids, a band with no
voxel in it and one holding every voxel, frames with no valid depth, and
batches that mix such problems."""
import numpy as np
import pytest

from oracle.oracle import Params as OParams

pytestmark = pytest.mark.gpu

VOXEL = 0.004


def oparams(p):
    d = {k: getattr(p, k) for k in OParams.__dataclass_fields__}
    return OParams(**d)


def blob_pair(shape, seed, trunc_voxels=5.0):
    """Canonical and live SDFs (float32, metres) of a sphere and a moved,
    stretched sphere on a grid of shape (nz, ny, nx)."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    c = np.array([nx, ny, nz]) / 2.0 + rng.uniform(-0.5, 0.5, 3)
    r = 0.3 * min(shape)
    trunc = VOXEL * trunc_voxels
    z, y, x = np.meshgrid(np.arange(nz) + 0.5, np.arange(ny) + 0.5, np.arange(nx) + 0.5, indexing="ij")

    def sdf(centre, scale):
        q = np.sqrt(((x - centre[0]) / scale[0]) ** 2 + ((y - centre[1]) / scale[1]) ** 2 +
                    ((z - centre[2]) / scale[2]) ** 2)
        d = (q - r) * VOXEL
        return np.where(d > trunc, trunc + 1e-5, d).astype(np.float32)

    return sdf(c, (1, 1, 1)), sdf(c + rng.uniform(-0.8, 0.8, 3), (1.05, 1.0, 0.97))


def in_band_field(shape, P, seed):
    """Values spread over the whole band: every voxel is active."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.9 * P.unknown_clip, 0.9 * P.max_surface, shape).astype(np.float32)


def grid(gpu, phi, P, weight=None):
    nz, ny, nx = phi.shape
    g = gpu.Grid((nx, ny, nz), VOXEL, (0.0, 0.0, 0.0), P.unknown_clip, P)
    w = weight if weight is not None else (phi <= P.max_surface).astype(np.int32)
    g.upload(phi.astype(np.float32), w.astype(np.int32))
    return g


def solve(gpu, gl, gc, P, iters, solver):
    f = gpu.Field(gl.dims, gpu.KF_F64 if solver == "exact" else gpu.KF_F32)
    st = gpu.psi_solve(gl, gc, f, P, iters, solver)
    return f.download(), st


def check_all_solvers(gpu, oracle, live, can, iters_exact=20, iters_f32=60):
    """Exact solver bit-exact at the paper weights; float32 solvers within
    1e-4 voxel at the reference's weights; band-only = dense bit for bit."""
    Pp = gpu.Params.paper(VOXEL)
    gl, gc = grid(gpu, live, Pp), grid(gpu, can, Pp)
    psi, st = solve(gpu, gl, gc, Pp, iters_exact, "exact")
    ost, opsi, counts = oracle.solve(live.astype(np.float64), can.astype(np.float64),
                                     np.zeros(live.shape + (3,)), iters_exact, oparams(Pp), active_counts=True)
    assert ost == 0
    np.testing.assert_array_equal(psi, opsi)
    assert st["active_first"] == counts[0] and st["active_last"] == counts[-1]
    Pr = gpu.Params.reference(VOXEL, 5.0)
    gl, gc = grid(gpu, live, Pr), grid(gpu, can, Pr)
    _, opsi = oracle.solve(live.astype(np.float64), can.astype(np.float64), np.zeros(live.shape + (3,)),
                           iters_f32, oparams(Pr))
    out = {}
    for solver in ("fused", "band", "plain"):
        out[solver], st = solve(gpu, gl, gc, Pr, iters_f32, solver)
        err = np.abs(out[solver].astype(np.float64) - opsi).max()
        assert err <= 1e-4, (solver, err)
    np.testing.assert_array_equal(out["band"], out["fused"])
    return counts[0]


def check_warp_fuse_mesh(gpu, oracle, live, can, seed):
    P = gpu.Params.paper(VOXEL)
    OP = oparams(P)
    rng = np.random.default_rng(seed)
    psi = rng.normal(0, 0.4, live.shape + (3,)).astype(np.float32)
    psi[rng.random(live.shape) < 0.3] = 0.0
    wl = rng.integers(0, 3, live.shape).astype(np.int32)
    wc = rng.integers(0, 3, live.shape).astype(np.int32)
    gl, gc = grid(gpu, live, P, wl), grid(gpu, can, P, wc)
    f = gpu.Field(gl.dims, gpu.KF_F32)
    f.upload(psi)
    gpu.warp_fuse(gc, gl, f, P)
    lphi, lw = gl.download()
    cphi, cw = gc.download()
    uphi, uw = oracle.update(live.astype(np.float64), wl.astype(np.int64), psi.astype(np.float64), OP)
    np.testing.assert_array_equal(lw, uw)
    np.testing.assert_array_equal(lphi, uphi.astype(np.float32))
    fphi, fw = oracle.fuse(can.astype(np.float64), wc.astype(np.int64),
                           uphi.astype(np.float32).astype(np.float64), uw)
    np.testing.assert_array_equal(cw, fw)
    np.testing.assert_array_equal(cphi, fphi.astype(np.float32))
    for g, phi in ((gl, lphi), (gc, cphi)):
        tris = gpu.marching_cubes(g, P)
        otris = oracle.mesh(phi.astype(np.float64), OP)
        assert tris.shape == otris.shape
        if len(otris):
            assert np.abs(tris - otris).max() / (2.0 / max(g.dims)) <= 1e-4


@pytest.mark.parametrize("shape", [(23, 19, 17), (7, 45, 33), (9, 10, 61)])
def test_ragged_noncubic_grids(gpu, oracle, shape):
    """Voxel counts 7429, 10395 and 5490: not multiples of 4 (7429, 10395)
    nor of the 2048-voxel dense runs, so the tails of the vector loads and of
    the last run are exercised; the grids are not cubes."""
    can, live = blob_pair(shape, seed=sum(shape))
    assert check_all_solvers(gpu, oracle, live, can) > 50
    check_warp_fuse_mesh(gpu, oracle, live, can, seed=1)


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 1, 2), (1, 1, 5), (2, 3, 1), (5, 2, 3), (1, 7, 9)])
def test_tiny_grids_every_voxel_in_band(gpu, oracle, shape):
    """Grids a voxel or a few thick, every voxel inside the band: all voxels
    take the reference-order path of the outer shell, and the reference's
    linear-index check on psi (DisplacementField.cpp:25-34) wraps rows."""
    P = gpu.Params.paper(VOXEL)
    live, can = in_band_field(shape, P, 3), in_band_field(shape, P, 4)
    n = check_all_solvers(gpu, oracle, live, can, iters_exact=8, iters_f32=20)
    assert n == live.size
    check_warp_fuse_mesh(gpu, oracle, live, can, seed=2)


def test_every_voxel_in_band_32(gpu, oracle):
    """A 32^3 grid whose every voxel is in the band: the band list holds the
    whole grid (the dense pass's lists and the band pass's rounds at their
    largest)."""
    P = gpu.Params.paper(VOXEL)
    shape = (32, 32, 32)
    live, can = in_band_field(shape, P, 5), in_band_field(shape, P, 6)
    assert check_all_solvers(gpu, oracle, live, can, iters_exact=4, iters_f32=10) == live.size


def test_empty_band(gpu, oracle):
    """No voxel of the live SDF is observed: every solver leaves psi at zero,
    counts no band voxel and meshes nothing."""
    P = gpu.Params.paper(VOXEL)
    shape = (21, 22, 23)
    live = np.full(shape, P.max_surface + P.epsilon, np.float32)
    can, _ = blob_pair(shape, seed=9)
    gl, gc = grid(gpu, live, P, np.zeros(shape, np.int32)), grid(gpu, can, P)
    for solver in ("fused", "band", "plain", "exact", "pervoxel"):
        psi, st = solve(gpu, gl, gc, P, 12, solver)
        assert not np.any(psi), solver
        assert st["active_first"] == 0 and st["diverged"] == 0, solver
    assert len(gpu.marching_cubes(gl, P)) == 0
    f = gpu.Field(gl.dims, gpu.KF_F32)
    before = gc.download()
    gpu.warp_fuse(gc, gl, f, P)  # live weights are all zero: nothing fuses
    after = gc.download()
    np.testing.assert_array_equal(before[0], after[0])
    np.testing.assert_array_equal(before[1], after[1])


def test_integrate_frames_without_valid_depth(gpu):
    """All-zero depth, and depth beyond maxDepth everywhere: no voxel is
    touched (SDF.cpp:178)."""
    from killingfusion_gb300 import synth
    P = gpu.Params.paper(VOXEL)
    grid_, frames = synth.sphere_pair()
    for depth in (np.zeros_like(frames[0]), np.full_like(frames[0], 5.0)):
        g = gpu.Grid(grid_.dims, grid_.voxel, grid_.origin, P.unknown_clip, P)
        g.integrate(depth, min_depth=0.05, max_depth=1.2)
        phi, w = g.download()
        assert not np.any(w)
        assert np.all(phi == np.float32(P.max_surface + P.epsilon))


def test_batch_mixes_tiny_ragged_and_empty_problems(gpu):
    """A batch of a single voxel, a one-voxel-thick grid, a ragged grid, an
    empty band and a 32^3 sphere pair: each psi equals its own band solve bit
    for bit."""
    P = gpu.Params.paper(VOXEL)
    probs = []
    for shape, kind in (((1, 1, 1), "band"), ((1, 7, 9), "band"), ((23, 19, 17), "blob"),
                        ((21, 22, 23), "empty"), ((32, 32, 32), "blob")):
        if kind == "band":
            live, can = in_band_field(shape, P, 7), in_band_field(shape, P, 8)
        elif kind == "empty":
            live = np.full(shape, P.max_surface + P.epsilon, np.float32)
            can, _ = blob_pair(shape, seed=10)
        else:
            can, live = blob_pair(shape, seed=11)
        probs.append((grid(gpu, live, P), grid(gpu, can, P)))
    iters = 25
    fields = [gpu.Field(gl.dims, gpu.KF_F32) for gl, _ in probs]
    b = gpu.Batch([(gl, gc, f, P) for (gl, gc), f in zip(probs, fields)], iters)
    stats = b.run()
    for (gl, gc), f, st in zip(probs, fields, stats):
        ref, rst = solve(gpu, gl, gc, P, iters, "band")
        np.testing.assert_array_equal(f.download(), ref)
        assert st["active_first"] == rst["active_first"]
    b.close()
