"""Project energy, its adjoint and finite differences on the GPU
(kf_energy, kf_energy_adjoint, kf_energy_fd) against the oracle
(orc_project_energy*, tests/test_oracle_energy.py pins its gradient), and the
differentiation workload: 128^3 random-blob SDFs, psi of 8 Gaussian RBFs,
10^4 voxels drawn from the band.

Tolerances
* float64 energy terms: per-voxel arithmetic as the oracle's; sums in a
  different order, so relative 1e-12;
* float64 adjoint: a gather where the oracle scatters, relative 1e-11 of the
  largest component;
* float32 energy: relative 1e-4 of the float64 one;
* adjoint vs central differences (h = 1e-3 voxel): relative 1e-6, skipping
  samples within 2h of a trilinear cell boundary (where the energy is not
  differentiable);
* reference-form gradient (KillingFusion::computeEnergyGradient) in float64:
  bit-identical to the oracle.
"""
import numpy as np
import pytest

from killingfusion_gb300 import synth
from oracle.oracle import Params as OParams

pytestmark = pytest.mark.gpu


def oparams(p):
    d = {k: getattr(p, k) for k in OParams.__dataclass_fields__}
    return OParams(**d)


def setup(gpu, n, voxel, seed=3, psi_scale=1.0, prec="f32"):
    can, live, psi = synth.blob_fields(seed=seed, n=n, voxel=voxel)
    psi = (psi * psi_scale).astype(np.float32)
    P = gpu.Params.paper(voxel)
    gl = gpu.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
    gc = gpu.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
    gl.upload(live, (np.abs(live) < P.unknown_clip).astype(np.int32))
    gc.upload(can, (np.abs(can) < P.unknown_clip).astype(np.int32))
    f = gpu.Field((n, n, n), gpu.KF_F32 if prec == "f32" else gpu.KF_F64)
    f.upload(psi if prec == "f32" else psi.astype(np.float64))
    active = (np.abs(live) < P.unknown_clip).astype(np.uint8)
    return gl, gc, f, P, can, live, psi, active


def test_energy_and_adjoint_match_oracle(gpu, oracle):
    n, voxel = 24, 3.584 / (16 * 24)
    gl, gc, f, P, can, live, psi, active = setup(gpu, n, voxel, psi_scale=3.0)
    OP = oparams(P)
    c64, l64, p64 = can.astype(np.float64), live.astype(np.float64), psi.astype(np.float64)
    E = oracle.project_energy(l64, c64, p64, active, OP)
    terms = gpu.energy(gl, gc, f, P, active)
    assert terms.min() > 0
    assert abs(terms.sum() - E) <= 1e-12 * abs(E)
    t32 = gpu.energy(gl, gc, f, P, active, arith="f32")
    np.testing.assert_allclose(t32, terms, rtol=1e-4)
    # each term alone
    for k, name in enumerate(("use_data", "use_levelset", "use_killing")):
        only = P.with_(**{m: (m == name) for m in ("use_data", "use_levelset", "use_killing")})
        Ek = oracle.project_energy(l64, c64, p64, active, oparams(only))
        tk = gpu.energy(gl, gc, f, only, active)
        assert abs(tk.sum() - Ek) <= 1e-12 * abs(Ek), name
        assert abs(tk[k] - terms[k]) <= 1e-12 * abs(terms[k]), name
    # a window
    box = (3, 5, 7, 17, 19, 21)
    El = 0.0
    tb = gpu.energy(gl, gc, f, P, active, box=box)
    mask = np.zeros_like(active)
    mask[box[2]:box[5], box[1]:box[4], box[0]:box[3]] = active[box[2]:box[5], box[1]:box[4], box[0]:box[3]]
    El = oracle.project_energy(l64, c64, p64, mask, OP)
    assert abs(tb.sum() - El) <= 1e-12 * abs(El)
    # the adjoint, and with every voxel active
    g = gpu.energy_adjoint(gl, gc, f, P, active)
    go = oracle.project_energy_grad(l64, c64, p64, active, OP)
    assert np.abs(g - go).max() <= 1e-11 * np.abs(go).max()
    g = gpu.energy_adjoint(gl, gc, f, P, None)
    go = oracle.project_energy_grad(l64, c64, p64, np.ones_like(active), OP)
    assert np.abs(g - go).max() <= 1e-11 * np.abs(go).max()


def test_float64_field(gpu, oracle):
    n, voxel = 16, 3.584 / (16 * 16)
    gl, gc, f, P, can, live, psi, active = setup(gpu, n, voxel, psi_scale=3.0, prec="f64")
    OP = oparams(P)
    E = oracle.project_energy(live.astype(np.float64), can.astype(np.float64), psi.astype(np.float64),
                              active, OP)
    assert abs(gpu.energy(gl, gc, f, P, active).sum() - E) <= 1e-12 * abs(E)


def boundary_free(psi, xyz, h):
    """Samples whose warped position is at least 2h away from a cell face."""
    t = xyz.astype(np.float64) + psi[xyz[:, 2], xyz[:, 1], xyz[:, 0]].astype(np.float64)
    fr = t - np.trunc(t)
    fr = np.where(fr < 0, fr + 1.0, fr)
    return np.minimum(fr, 1.0 - fr) > 2 * h


def test_adjoint_against_central_differences_128(gpu, oracle):
    """The differentiation workload: adjoint vs float64 central differences
    at 10^4 band voxels, and the reference-form gradient at the same voxels
    against the oracle's computeEnergyGradient."""
    n, voxel, h = 128, 0.004, 1e-3
    gl, gc, f, P, can, live, psi, active = setup(gpu, n, voxel)
    z, y, x = np.nonzero(active)
    rng = np.random.default_rng(17)
    pick = rng.choice(len(x), size=10000, replace=False)
    xyz = np.stack([x[pick], y[pick], z[pick]], 1).astype(np.int32)
    g = gpu.energy_adjoint(gl, gc, f, P, active)
    fd = gpu.energy_fd(gl, gc, f, P, xyz, h, active)
    ga = g[xyz[:, 2], xyz[:, 1], xyz[:, 0]]
    # where psi is (near) zero the warped position sits on a cell face, where
    # the trilinear sample has no derivative: those samples are left out
    ok = boundary_free(psi, xyz, h)
    assert ok.sum() > 15000
    scale = np.abs(ga).max()
    err = np.abs(fd - ga)[ok]
    assert err.max() <= 1e-6 * scale, (err.max(), scale)
    # the oracle's own central differences at a few voxels
    OP = oparams(P)
    c64, l64, p64 = can.astype(np.float64), live.astype(np.float64), psi.astype(np.float64)
    for i in range(8):
        vx, vy, vz = (int(v) for v in xyz[i])
        for a in range(3):
            pp, pm = p64.copy(), p64.copy()
            pp[vz, vy, vx, a] += h
            pm[vz, vy, vx, a] -= h
            ep = oracle.project_energy_local(l64, c64, pp, active, (vx, vy, vz), 1, OP)
            em = oracle.project_energy_local(l64, c64, pm, active, (vx, vy, vz), 1, OP)
            assert abs((ep - em) / (2 * h) - fd[i, a]) <= 1e-9 * (1 + abs(fd[i, a]))
    # Check B: the reference-form gradient, float64 field
    f64 = gpu.Field((n, n, n), gpu.KF_F64)
    f64.upload(psi.astype(np.float64))
    gref, act = gpu.psi_gradient_ref(gl, gc, f64, P, xyz[:2000])
    gora = oracle.voxel_query("grad", l64, c64, p64, xyz[:2000], OP)
    aora = oracle.voxel_query("active", l64, c64, p64, xyz[:2000], OP)[:, 0]
    np.testing.assert_array_equal(act, aora.astype(np.uint8))
    np.testing.assert_array_equal(gref[act == 1], gora[act == 1])
