"""The oracle's project energy (oracle/kf_oracle.c) is consistent with its
own exact gradient: central differences of the windowed energy match the
scattered gradient.  This energy has no counterpart in the reference (its
solver never evaluates one), so it is pinned by this self-consistency and by
the reference-form gradient checks elsewhere."""
import numpy as np

from killingfusion_gb300 import synth
from oracle.oracle import Params


def problem(n=14, seed=3):
    """The blob workload shrunk to a small grid (coarser voxels, same
    shapes); psi stretched so it crosses cells."""
    voxel = 3.584 / (16 * n)
    can, live, psi = synth.blob_fields(seed=seed, n=n, voxel=voxel)
    psi = (psi * 3.0).astype(np.float64)
    P = Params.paper(voxel)
    active = (np.abs(live) < P.unknown_clip).astype(np.uint8)
    return can.astype(np.float64), live.astype(np.float64), psi, active, P


def test_project_energy_gradient_matches_central_differences(oracle):
    can, live, psi, active, P = problem()
    assert active.sum() > 50
    E = oracle.project_energy(live, can, psi, active, P)
    assert np.isfinite(E) and E > 0
    g = oracle.project_energy_grad(live, can, psi, active, P)
    rng = np.random.default_rng(0)
    n = live.shape[0]
    h = 1e-4
    checked = 0
    for _ in range(60):
        x, y, z = (int(v) for v in rng.integers(0, n, 3))
        for a in range(3):
            t = (x, y, z)[a] + psi[z, y, x, a]
            if min(t % 1.0, 1.0 - t % 1.0) < 4 * h:
                continue  # a cell boundary of the trilinear sample
            pp, pm = psi.copy(), psi.copy()
            pp[z, y, x, a] += h
            pm[z, y, x, a] -= h
            ep = oracle.project_energy_local(live, can, pp, active, (x, y, z), 1, P)
            em = oracle.project_energy_local(live, can, pm, active, (x, y, z), 1, P)
            fd = (ep - em) / (2 * h)
            assert abs(fd - g[z, y, x, a]) <= 1e-6 * (1 + abs(g[z, y, x, a])), (x, y, z, a, fd, g[z, y, x, a])
            checked += 1
    assert checked > 120


def test_local_energy_sums_to_global(oracle):
    can, live, psi, active, P = problem(n=10, seed=5)
    E = oracle.project_energy(live, can, psi, active, P)
    n = live.shape[0]
    # a window covering the whole grid equals the global energy
    El = oracle.project_energy_local(live, can, psi, active, (n // 2,) * 3, n, P)
    assert abs(E - El) <= 1e-12 * abs(E)
