"""GPU parity: the CUDA path, called through the C ABI, against the FP64
oracle (which tests/test_oracle_golden.py pins to the reference).

Tolerances
* integer/index results (weights, band flags, triangle counts, topology):
  exact;
* float64 "exact" solver: bit-identical to the oracle given the same float32
  SDFs;
* float32 solvers: |psi - psi_oracle| <= 1e-4 voxel where the reference's
  iteration is stable (its own default weights), see test_fp32_* below;
* float32 SDF values written by float64 arithmetic: equal to the oracle's
  double rounded to float32.
"""
import numpy as np
import pytest

from killingfusion_gb300 import synth
from oracle.oracle import Params as OParams
from helpers import small_pair, integrate_oracle

pytestmark = pytest.mark.gpu

PSI_TOL = 1e-4  # voxel


def oparams(p):
    """capi.Params -> oracle.Params (same fields, minus early_exit)."""
    d = {k: getattr(p, k) for k in OParams.__dataclass_fields__}
    return OParams(**d)


def make_grid(capi, phi, voxel, params, origin=(0.0, 0.0, 0.0), weight=None):
    nz, ny, nx = phi.shape
    g = capi.Grid((nx, ny, nz), voxel, origin, params.unknown_clip, params)
    w = weight if weight is not None else (phi <= params.max_surface).astype(np.int32)
    g.upload(phi.astype(np.float32), w.astype(np.int32))
    return g


# ---------------------------------------------------------------------------
# integration
# ---------------------------------------------------------------------------

def test_integrate_sphere_frames(gpu, oracle):
    grid, frames = synth.sphere_pair()
    P = gpu.Params.paper(grid.voxel)
    for f in frames:
        g = gpu.Grid(grid.dims, grid.voxel, grid.origin, P.unknown_clip, P)
        g.integrate(f, min_depth=0.05, max_depth=1.2)
        phi, w = g.download()
        ophi, ow = integrate_oracle(oracle, grid, f, oparams(P))
        np.testing.assert_array_equal(w, ow)
        np.testing.assert_array_equal(phi, ophi.astype(np.float32))
        assert (w > 0).sum() > 1000


def test_integrate_pose_and_running_mean(gpu, oracle):
    """A rotated camera and a second frame into the same grid (weights 2)."""
    import os
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "integrate_small.npz"))
    P = gpu.Params.paper(0.01)
    g = gpu.Grid((20, 20, 20), 0.01, gold["origin"], P.unknown_clip, P)
    g.integrate(gold["depth"].astype(np.float32), gold["c2w"], gold["K"], 0.05, 1.2)
    phi, w = g.download()
    np.testing.assert_array_equal(w, gold["w_pose"])
    np.testing.assert_array_equal(phi, gold["phi_pose"].astype(np.float32))
    # second frame: the running mean starts from the float32 value on the GPU
    g.integrate((gold["depth"] * 1.01).astype(np.float32), gold["c2w"], gold["K"], 0.05, 1.2)
    phi2, w2 = g.download()
    np.testing.assert_array_equal(w2, gold["w2_pose"])
    ref = gold["phi2_pose"]
    m = w2 > 0
    assert np.abs(phi2[m] - ref[m]).max() <= 2e-7 * np.abs(ref[m]).max() + 1e-9


@pytest.mark.parametrize("shift", [(0.0, 0.0, 0.0), (3.0, -2.0, 1.5), (120.0, -75.0, 300.0)])
def test_integrate_far_from_origin(gpu, oracle, shift):
    """Grid and camera moved together away from the world origin, the camera
    turned by 4 degrees.  The camera coordinates are then differences of
    world coordinates of up to hundreds of metres, whose float rounding is
    hundreds of times that of the unshifted grid: the float projection's
    per-voxel error bound grows with them (at the largest shift more than a
    third of the voxels lie within it of a pixel edge and take the float64
    path, past the side list's capacity some in place), and every pixel,
    weight and distance stays the reference's.  A fixed margin of 1/128
    pixel would misplace about 1.4 k voxels at the largest shift."""
    grid, frames = synth.sphere_pair()
    P = gpu.Params.paper(grid.voxel)
    t = np.asarray(shift, dtype=np.float64)
    a = np.deg2rad(4.0)
    c2w = np.eye(4)
    c2w[:3, :3] = [[np.cos(a), 0.0, np.sin(a)], [0.0, 1.0, 0.0], [-np.sin(a), 0.0, np.cos(a)]]
    c2w[:3, 3] = t
    origin = np.asarray(grid.origin, dtype=np.float64) + t
    w2c = oracle.invert4(c2w)
    n = grid.dims[::-1]
    for f in frames:
        g = gpu.Grid(grid.dims, grid.voxel, origin, P.unknown_clip, P)
        g.integrate(f, c2w, synth.K, 0.05, 1.2)
        phi, w = g.download()
        g.close()
        ophi, ow = oracle.integrate(np.full(n, P.max_surface + P.epsilon), np.zeros(n, np.int64), grid.voxel,
                                    origin, P.unknown_clip, f.astype(np.float64), w2c, synth.K, 0.05, 1.2)
        np.testing.assert_array_equal(w, ow)
        np.testing.assert_array_equal(phi, ophi.astype(np.float32))
        assert (w > 0).sum() > 1000


@pytest.mark.parametrize("case", ["float", "float_far", "u16"])
def test_compute_sdf_equals_reset_then_integrate(gpu, case):
    """kf_compute_sdf (KillingFusion::computeSDF in one pass) leaves the grid
    bit for bit as kf_grid_reset followed by kf_integrate_depth does, also
    when the grid held other values before (every voxel is written)."""
    grid, frames = synth.sphere_pair()
    P = gpu.Params.paper(grid.voxel)
    c2w, origin = None, grid.origin
    if case == "float_far":
        c2w = np.eye(4)
        c2w[:3, 3] = (120.0, -75.0, 300.0)
        origin = np.asarray(grid.origin) + c2w[:3, 3]
    rng = np.random.default_rng(51)
    for f in frames:
        a = gpu.Grid(grid.dims, grid.voxel, origin, P.unknown_clip, P)
        b = gpu.Grid(grid.dims, grid.voxel, origin, P.unknown_clip, P)
        shape = grid.dims[::-1]
        b.upload(rng.normal(0, 1, shape).astype(np.float32), rng.integers(0, 9, shape).astype(np.int32))
        if case == "u16":
            d16 = np.where(np.isfinite(f), np.round(f * 1000.0), 0).astype(np.uint16)
            a.reset(P)
            a.integrate_u16(d16, 0.001, c2w, min_depth=0.05, max_depth=1.2)
            b.compute_sdf(P, d16, c2w, min_depth=0.05, max_depth=1.2, u16_scale=0.001)
        else:
            a.reset(P)
            a.integrate(f, c2w, min_depth=0.05, max_depth=1.2)
            b.compute_sdf(P, f, c2w, min_depth=0.05, max_depth=1.2)
        pa, wa = a.download()
        pb, wb = b.download()
        a.close()
        b.close()
        np.testing.assert_array_equal(wb, wa)
        np.testing.assert_array_equal(pb.view(np.int32), pa.view(np.int32))
        assert (wa > 0).sum() > 1000


# ---------------------------------------------------------------------------
# reference gradient at single voxels
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("weights", ["reference", "paper"])
def test_gradient_ref_f64_bitexact(gpu, oracle, weights):
    """KillingFusion::computeEnergyGradient at every voxel of a 20^3 pair,
    including the outer shell and displacements that leave the grid."""
    voxel = 0.004
    P = gpu.Params.reference(voxel, 5.0) if weights == "reference" else gpu.Params.paper(voxel)
    can, live = small_pair(20, voxel, 5.0, seed=3)
    rng = np.random.default_rng(4)
    psi = rng.normal(0.0, 0.6, live.shape + (3,))
    psi.reshape(-1, 3)[rng.integers(0, psi.size // 3, 50)] *= 20
    gl, gc = make_grid(gpu, live, voxel, P), make_grid(gpu, can, voxel, P)
    f = gpu.Field(gl.dims, gpu.KF_F64)
    f.upload(psi)
    z, y, x = np.meshgrid(*[np.arange(20)] * 3, indexing="ij")
    xyz = np.stack([x, y, z], -1).reshape(-1, 3)
    g, act = gpu.psi_gradient_ref(gl, gc, f, P, xyz)
    OP = oparams(P)
    og = oracle.voxel_query("grad", live, can, psi, xyz, OP)
    oa = oracle.voxel_query("active", live, can, psi, xyz, OP)[:, 0]
    np.testing.assert_array_equal(g, og)
    np.testing.assert_array_equal(act, oa.astype(np.uint8))


def test_gradient_ref_f32_close(gpu, oracle):
    voxel = 0.004
    P = gpu.Params.paper(voxel)
    can, live = small_pair(20, voxel, 5.0, seed=5)
    rng = np.random.default_rng(6)
    psi = rng.normal(0.0, 0.3, live.shape + (3,)).astype(np.float32)
    gl, gc = make_grid(gpu, live, voxel, P), make_grid(gpu, can, voxel, P)
    f = gpu.Field(gl.dims, gpu.KF_F32)
    f.upload(psi)
    xyz = np.argwhere(np.ones(live.shape, bool))[:, ::-1]
    g, _ = gpu.psi_gradient_ref(gl, gc, f, P, xyz)
    og = oracle.voxel_query("grad", live, can, psi.astype(np.float64), xyz, oparams(P))
    scale = np.abs(og).max()
    assert np.abs(g - og).max() <= 1e-3 * scale


# ---------------------------------------------------------------------------
# psi solve
# ---------------------------------------------------------------------------

def sphere_sdfs(gpu, P):
    """GPU-integrated canonical and live SDFs of the 64^3 sphere pair, and
    their float32 values as float64 for the oracle."""
    grid, frames = synth.sphere_pair()
    grids = []
    for f in frames:
        g = gpu.Grid(grid.dims, grid.voxel, grid.origin, P.unknown_clip, P)
        g.integrate(f, min_depth=0.05, max_depth=1.2)
        grids.append(g)
    can, live = grids
    return can, live, can.download()[0].astype(np.float64), live.download()[0].astype(np.float64)


@pytest.mark.parametrize("weights", ["paper", "reference"])
def test_exact_solver_bitexact_64cubed(gpu, oracle, weights):
    """100 float64 iterations at 64^3 replay the reference bit for bit, with
    the paper weights as well (where any other rounding diverges)."""
    voxel = 0.004
    P = gpu.Params.paper(voxel) if weights == "paper" else gpu.Params.reference(voxel, 5.0)
    can, live, ocan, olive = sphere_sdfs(gpu, P)
    f = gpu.Field(live.dims, gpu.KF_F64)
    st = gpu.psi_solve(live, can, f, P, 100, "exact")
    psi = f.download()
    ost, opsi, counts = oracle.solve(olive, ocan, np.zeros(olive.shape + (3,)), 100, oparams(P),
                                     active_counts=True)
    assert ost == 0 and st["iterations_run"] == 100
    assert st["active_first"] == counts[0] and st["active_last"] == counts[-1]
    np.testing.assert_array_equal(psi, opsi)


@pytest.mark.parametrize("solver", ["fused", "plain", "band"])
def test_fp32_solvers_match_oracle_stable_weights(gpu, oracle, solver):
    """Float32 solvers within 1e-4 voxel of the FP64 oracle after 100
    iterations with the reference's own weights (config.cpp:45-54)."""
    voxel = 0.004
    P = gpu.Params.reference(voxel, 5.0)
    can, live, ocan, olive = sphere_sdfs(gpu, P)
    f = gpu.Field(live.dims, gpu.KF_F32)
    st = gpu.psi_solve(live, can, f, P, 100, solver)
    psi = f.download().astype(np.float64)
    _, opsi, counts = oracle.solve(olive, ocan, np.zeros(olive.shape + (3,)), 100, oparams(P),
                                   active_counts=True)
    err = np.abs(psi - opsi).max()
    assert err <= PSI_TOL, err
    assert np.abs(opsi).max() > 0.05  # the field did move
    assert st["active_first"] == counts[0]


def test_fused_and_plain_agree(gpu):
    voxel = 0.004
    P = gpu.Params.reference(voxel, 5.0)
    can, live, _, _ = sphere_sdfs(gpu, P)
    out = {}
    for solver in ("fused", "plain"):
        f = gpu.Field(live.dims, gpu.KF_F32)
        gpu.psi_solve(live, can, f, P, 50, solver)
        out[solver] = f.download()
    assert np.abs(out["fused"] - out["plain"]).max() <= 1e-5


@pytest.mark.parametrize("weights,iters", [("paper", 200), ("paper", 37), ("reference", 100)])
def test_band_solver_equals_fused(gpu, weights, iters):
    """The band-only solver visits only the shrinking band after the first
    dense pass; psi, band counts and statistics equal the dense fused
    solver's bit for bit -- at the paper weights too, over the full
    iteration count, where any difference would be amplified."""
    voxel = 0.004
    P = gpu.Params.paper(voxel) if weights == "paper" else gpu.Params.reference(voxel, 5.0)
    can, live, _, _ = sphere_sdfs(gpu, P)
    out, st = {}, {}
    for solver in ("fused", "band"):
        f = gpu.Field(live.dims, gpu.KF_F32)
        st[solver] = gpu.psi_solve(live, can, f, P, iters, solver)
        out[solver] = f.download()
    np.testing.assert_array_equal(out["band"], out["fused"])
    for k in ("iterations_run", "active_first", "active_last", "max_delta_last"):
        assert st["band"][k] == st["fused"][k], k
    assert st["band"]["active_last"] <= st["band"]["active_first"]


def test_fp32_paper_weights_short_horizon(gpu, oracle):
    """With the paper weights the reference's iteration amplifies rounding
    (about 10x per iteration once the Killing term is active), so float32
    tracks the FP64 oracle only over the first iterations."""
    voxel = 0.004
    P = gpu.Params.paper(voxel)
    can, live, ocan, olive = sphere_sdfs(gpu, P)
    for solver in ("fused", "plain"):
        f = gpu.Field(live.dims, gpu.KF_F32)
        gpu.psi_solve(live, can, f, P, 3, solver)
        _, opsi = oracle.solve(olive, ocan, np.zeros(olive.shape + (3,)), 3, oparams(P))
        assert np.abs(f.download() - opsi).max() <= PSI_TOL


def test_solve_is_repeatable_and_graph_reuse(gpu):
    """A second solve reuses the captured graph and gives the same field."""
    voxel = 0.004
    P = gpu.Params.reference(voxel, 5.0)
    can, live, _, _ = sphere_sdfs(gpu, P)
    f = gpu.Field(live.dims, gpu.KF_F32)
    gpu.psi_solve(live, can, f, P, 20, "fused")
    a = f.download()
    f.zero()
    gpu.psi_solve(live, can, f, P, 20, "fused")
    np.testing.assert_array_equal(a, f.download())
    f.zero()
    gpu.psi_solve(live, can, f, P, 21, "fused")  # odd count: result in the other buffer
    b = f.download()
    assert np.abs(b - a).max() > 0


def test_divergence_is_reported(gpu):
    """A non-finite psi inside the band stops the solve with KF_ERR_DIVERGED
    (the reference throws -1, KillingFusion.cpp:328-332)."""
    voxel = 0.004
    P = gpu.Params.reference(voxel, 5.0)
    can, live = small_pair(24, voxel, 5.0, seed=1)
    gl, gc = make_grid(gpu, live, voxel, P), make_grid(gpu, can, voxel, P)
    for prec, solver in ((gpu.KF_F32, "fused"), (gpu.KF_F32, "plain"), (gpu.KF_F32, "band"),
                         (gpu.KF_F64, "exact")):
        f = gpu.Field(gl.dims, prec)
        psi = np.zeros(live.shape + (3,))
        z, y, x = np.argwhere((live > -0.01) & (live < 0.01))[0]
        psi[z, y, x, 0] = np.nan
        f.upload(psi)
        with pytest.raises(gpu.DivergedError):
            gpu.psi_solve(gl, gc, f, P, 5, solver)


def test_early_exit_convergence_flag(gpu):
    """With early_exit the loop stops once max |dpsi| <= threshold."""
    voxel = 0.004
    P = gpu.Params.reference(voxel, 5.0).with_(early_exit=True, threshold=1e-4)
    can, live, _, _ = sphere_sdfs(gpu, P)
    res = {}
    for solver in ("fused", "band"):
        f = gpu.Field(live.dims, gpu.KF_F32)
        st = gpu.psi_solve(live, can, f, P, 400, solver)
        assert st["converged"] == 1 and st["iterations_run"] < 400
        assert st["max_delta_last"] <= 1e-4
        res[solver] = (st["iterations_run"], f.download())
    assert res["fused"][0] == res["band"][0]
    np.testing.assert_array_equal(res["fused"][1], res["band"][1])


# ---------------------------------------------------------------------------
# warp / fuse / marching cubes
# ---------------------------------------------------------------------------

def test_warp_fuse_exact(gpu, oracle):
    """SDF::update + SDF::fuse on the same psi: integer weights exact (the
    truncation of an interpolated double), SDF values the oracle's doubles
    rounded to float32."""
    voxel = 0.004
    P = gpu.Params.paper(voxel)
    can, live = small_pair(24, voxel, 5.0, seed=21)
    rng = np.random.default_rng(3)
    psi = rng.normal(0, 0.4, live.shape + (3,)).astype(np.float32)
    psi[rng.random(live.shape) < 0.5] = 0.0
    wl = rng.integers(0, 3, live.shape).astype(np.int32)
    wc = rng.integers(0, 3, live.shape).astype(np.int32)
    gl, gc = make_grid(gpu, live, voxel, P, weight=wl), make_grid(gpu, can, voxel, P, weight=wc)
    f = gpu.Field(gl.dims, gpu.KF_F32)
    f.upload(psi)
    gpu.warp_fuse(gc, gl, f, P)
    lphi, lw = gl.download()
    cphi, cw = gc.download()
    OP = oparams(P)
    uphi, uw = oracle.update(live.astype(np.float64), wl.astype(np.int64), psi.astype(np.float64), OP)
    np.testing.assert_array_equal(lw, uw)
    np.testing.assert_array_equal(lphi, uphi.astype(np.float32))
    fphi, fw = oracle.fuse(can.astype(np.float64), wc.astype(np.int64), uphi.astype(np.float32).astype(np.float64), uw)
    np.testing.assert_array_equal(cw, fw)
    np.testing.assert_array_equal(cphi, fphi.astype(np.float32))


def test_fuse_and_fuse_warped(gpu, oracle):
    voxel = 0.004
    P = gpu.Params.paper(voxel)
    can, live = small_pair(24, voxel, 5.0, seed=22)
    rng = np.random.default_rng(8)
    psi = rng.normal(0, 0.5, live.shape + (3,)).astype(np.float32)
    wl = rng.integers(0, 3, live.shape).astype(np.int32)
    wc = rng.integers(0, 3, live.shape).astype(np.int32)
    OP = oparams(P)
    gl, gc = make_grid(gpu, live, voxel, P, weight=wl), make_grid(gpu, can, voxel, P, weight=wc)
    gpu.fuse(gc, gl)
    cphi, cw = gc.download()
    ophi, ow = oracle.fuse(can.astype(np.float64), wc.astype(np.int64), live.astype(np.float64), wl.astype(np.int64))
    np.testing.assert_array_equal(cw, ow)
    np.testing.assert_array_equal(cphi, ophi.astype(np.float32))
    gl, gc = make_grid(gpu, live, voxel, P, weight=wl), make_grid(gpu, can, voxel, P, weight=wc)
    f = gpu.Field(gl.dims, gpu.KF_F32)
    f.upload(psi)
    gpu.fuse_warped(gc, gl, f, P)
    cphi, cw = gc.download()
    ophi, ow = oracle.fuse_psi(can.astype(np.float64), wc.astype(np.int64), live.astype(np.float64),
                               wl.astype(np.int64), psi.astype(np.float64), OP)
    np.testing.assert_array_equal(cw, ow)
    np.testing.assert_array_equal(cphi, ophi.astype(np.float32))


@pytest.mark.parametrize("which", ["sphere64", "pair24"])
def test_marching_cubes_counts_exact(gpu, oracle, which):
    """Triangle counts and order bit-exact, vertices within 1e-4 voxel."""
    if which == "sphere64":
        P = gpu.Params.paper(0.004)
        can, live, ocan, olive = sphere_sdfs(gpu, P)
        grids = [(can, ocan), (live, olive)]
    else:
        P = gpu.Params.paper(0.004)
        c, l = small_pair(24, 0.004, 5.0, seed=30)
        grids = [(make_grid(gpu, c, 0.004, P), c.astype(np.float64)),
                 (make_grid(gpu, l, 0.004, P), l.astype(np.float64))]
    for g, ophi in grids:
        tris = gpu.marching_cubes(g, P)
        otris = oracle.mesh(ophi, oparams(P))
        assert tris.shape == otris.shape and len(tris) > 100
        # vertices lie in [-1, 1]; one voxel is 2/n of that range
        n = max(g.dims)
        err_vox = np.abs(tris - otris).max() / (2.0 / n)
        assert err_vox <= 1e-4, err_vox


def mesh_against_oracle(gpu, oracle, phi, P, min_tris):
    nz, ny, nx = phi.shape
    g = make_grid(gpu, phi, 0.004, P)
    tris = gpu.marching_cubes(g, P)
    g.close()
    otris = oracle.mesh(phi.astype(np.float64), oparams(P))
    assert tris.shape == otris.shape and len(tris) >= min_tris, (tris.shape, otris.shape)
    # vertex coordinates are (index / half size - 1): one voxel is 2/n of the range
    err_vox = (np.abs(tris - otris).reshape(-1, 3, 3) / (2.0 / np.array([nx, ny, nz]))).max()
    assert err_vox <= 1e-4, err_vox


def test_marching_cubes_ragged_dims(gpu, oracle):
    """A grid whose sizes are not multiples of anything the passes use
    (37 x 29 x 23): rows end inside a thread's run of cells and the last
    block is partial."""
    P = gpu.Params.paper(0.004)
    dims = (37, 29, 23)
    Z, Y, X = np.meshgrid(*[np.arange(n) + 0.5 for n in dims[::-1]], indexing="ij")
    d = (np.sqrt((X - 17.3) ** 2 + ((Y - 14.1) / 0.9) ** 2 + (Z - 11.6) ** 2) - 8.2) * 0.004
    phi = np.where(d > P.max_surface, P.max_surface + 1e-5, d).astype(np.float32)
    mesh_against_oracle(gpu, oracle, phi, P, 200)


def test_marching_cubes_list_overflow(gpu, oracle):
    """More cells with triangles than the marching cubes' cell list holds
    (count / 16 entries at 200^3): a noise box of 112 x 96 x 72 cells, all
    in the band with random signs, inside an otherwise empty grid.  The emit
    pass then re-classifies every block with triangles, and the mesh is
    still the reference's, triangle for triangle."""
    P = gpu.Params.paper(0.004)
    n = 200
    rng = np.random.default_rng(41)
    phi = np.full((n, n, n), P.max_surface + 1e-5, np.float32)
    box = rng.uniform(0.2, 0.8, (72, 96, 112)) * np.where(rng.random((72, 96, 112)) < 0.5, -P.unknown_clip,
                                                            P.max_surface)
    phi[60:132, 50:146, 40:152] = box.astype(np.float32)
    # all but 1/128 of the box's cells (those with eight equal signs) have
    # triangles, each at least one
    min_cells = int(0.9 * box.size)
    assert min_cells > n ** 3 // 16
    mesh_against_oracle(gpu, oracle, phi, P, min_cells)


def test_mesh_capacity_error(gpu):
    import ctypes as C
    import torch
    P = gpu.Params.paper(0.004)
    c, _ = small_pair(24, 0.004, 5.0, seed=31)
    g = make_grid(gpu, c, 0.004, P)
    L = gpu.load()
    n = C.c_int64(0)
    buf = torch.empty((4, 9), dtype=torch.float32, device="cuda")
    st = L.kf_marching_cubes(g.h, C.byref(P.c()), buf.data_ptr(), 4, C.byref(n), None)
    assert st == gpu.KF_ERR_CAPACITY and n.value > 4
