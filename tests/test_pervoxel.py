"""KF_SOLVER_PERVOXEL, the reference's default per-voxel schedule
(KillingFusion.cpp:353-396), against the oracle's single-thread runs of the
same schedule.  The GPU takes the voxels colour by colour (parity of x, y, z:
no two voxels of one colour share a neighbourhood, so each iterates with its
neighbours fixed, as in the reference's loop); the oracle runs that order in
float64 (psi within float32 rounding) and the reference's z, y, x order
(same voxels, same convergence, registration residual within a few per cent
of its improvement)."""
import numpy as np
import pytest

from helpers import small_pair
from oracle.oracle import Params as OParams

pytestmark = pytest.mark.gpu


def oparams(p):
    d = {k: getattr(p, k) for k in OParams.__dataclass_fields__}
    return OParams(**d)


def grid(gpu, phi, voxel, P):
    n = phi.shape[0]
    g = gpu.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
    g.upload(phi, (phi <= P.max_surface).astype(np.int32))
    return g


def residual(oracle, live, can, psi, P, voxels):
    """Mean |phi_live(i + psi(i)) - phi_can(i)| over voxels (in voxel units)."""
    w = oracle.voxel_query("warped", live, None, psi, voxels, P)[:, 0]
    c = can[voxels[:, 2], voxels[:, 1], voxels[:, 0]]
    return float(np.mean(np.abs(w - c))) / P.voxel_size


def test_pervoxel_matches_oracle_statistically(gpu, oracle):
    voxel = 0.004
    P = gpu.Params.reference(voxel, 5.0)
    OP = oparams(P)
    can, live = small_pair(24, voxel, 5.0, seed=3)
    gl, gc = grid(gpu, live, voxel, P), grid(gpu, can, voxel, P)
    f = gpu.Field(gl.dims, gpu.KF_F32)
    st = gpu.psi_solve(gl, gc, f, P, 1024, "pervoxel")
    psi = f.download().astype(np.float64)
    l64, c64 = live.astype(np.float64), can.astype(np.float64)
    ost, opsi, (visited, steps, capped) = oracle.solve_pervoxel(l64, c64, np.zeros(psi.shape), 1024, OP)
    cst, cpsi, (cvisited, csteps, ccapped) = oracle.solve_pervoxel(l64, c64, np.zeros(psi.shape), 1024, OP,
                                                                   colored=True)
    assert ost == 0 and cst == 0
    print("gpu: visited %d, capped %d, most steps %d; oracle: visited %d, capped %d, steps %d"
          % (st["active_first"], st["capped"], st["iterations_run"], visited, capped, steps))
    assert st["active_first"] == visited == cvisited > 1000
    assert capped == ccapped == st["capped"] == 0 and st["converged"] == 1
    assert 1 <= st["iterations_run"] <= 1024
    # the GPU's order, in float64: float32 rounding apart
    print("psi: max |gpu - oracle (colour order)| %.2e voxel, max |psi| %.2e"
          % (np.abs(psi - cpsi).max(), np.abs(cpsi).max()))
    assert np.abs(psi - cpsi).max() <= 2e-5
    # the voxels visited: symmetric band of the zero field
    lo = -(OP.max_surface - OP.epsilon)
    z, y, x = np.nonzero((l64 <= OP.max_surface - OP.epsilon) & (l64 >= lo))
    vox = np.stack([x, y, z], 1)
    assert len(vox) == visited
    # psi moved only at visited voxels
    moved = np.abs(psi).sum(-1) > 0
    assert not moved[~((l64 <= OP.max_surface - OP.epsilon) & (l64 >= lo))].any()
    r0 = residual(oracle, l64, c64, np.zeros(psi.shape), OP, vox)
    r_gpu = residual(oracle, l64, c64, psi, OP, vox)
    r_orc = residual(oracle, l64, c64, opsi, OP, vox)
    r_col = residual(oracle, l64, c64, cpsi, OP, vox)
    print("residual: start %.6f  reference order %.6f  colour order %.6f  gpu %.6f" % (r0, r_orc, r_col, r_gpu))
    assert r_orc < r0 and r_col < r0 and r_gpu < r0
    # the GPU is the colour order; the two orders improve the residual alike
    assert abs(r_gpu - r_col) <= 1e-6 * r_col
    assert abs(r_col - r_orc) <= 0.25 * (r0 - r_orc)


def test_pervoxel_cap_and_paper_weights(gpu, oracle):
    """At the paper weights the per-voxel iteration does not settle: every
    voxel runs to the cap, on the GPU as in the oracle, and psi stays finite."""
    voxel = 0.004
    P = gpu.Params.paper(voxel)
    OP = oparams(P)
    can, live = small_pair(16, voxel, 5.0, seed=5)
    gl, gc = grid(gpu, live, voxel, P), grid(gpu, can, voxel, P)
    f = gpu.Field(gl.dims, gpu.KF_F32)
    cap = 64
    st = gpu.psi_solve(gl, gc, f, P, cap, "pervoxel")
    _, _, (visited, steps, capped) = oracle.solve_pervoxel(live.astype(np.float64), can.astype(np.float64),
                                                           np.zeros(live.shape + (3,)), cap, OP, colored=True)
    print("paper weights: gpu capped %d of %d, oracle capped %d" % (st["capped"], st["active_first"], capped))
    assert st["active_first"] == visited
    assert st["iterations_run"] <= cap
    assert capped == visited and st["capped"] >= 0.9 * visited
    assert np.isfinite(f.download()).all()
