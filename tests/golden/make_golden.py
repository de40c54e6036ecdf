"""Generate the golden fixtures of tests/golden from the reference itself.

Runs the reference's own SDF / DisplacementField / KillingFusion code (built
from the reference checkout into oracle/_ref by oracle/build.py) on small
seeded inputs and stores inputs and outputs as .npz files.  The oracle
restatement (oracle/kf_oracle.c) must reproduce every stored output bit for
bit (tests/test_oracle_golden.py); the fixtures travel where the reference
checkout does not.

Usage:  python tests/golden/make_golden.py [fixture ...]   (default: all)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle.oracle import Params, RefLib  # noqa: E402
from helpers import small_pair  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("wrote", path, sum(a.nbytes for a in arrays.values()), "bytes raw")


def linear_selftests():
    """SDF::testGetDistance / testGetWeight / testComputeDistanceGradient /
    testComputeDistanceHessian (SDF.cpp:526-568, 606-648, 681-724, 797-840):
    f = x + y - z on the 17^3 grid of voxel 0.5 over [0, 8]."""
    P = Params()  # the reference's defaults (epsilon 1e-5, deltaSize 0.05)
    R = RefLib(P, 1)
    n = R.grid_size(np.array([8.0, 8.0, 8.0]), 0.5)
    nz, ny, nx = int(n[2]), int(n[1]), int(n[0])
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    f = (x + y - z).astype(np.float64)
    pts, pts_h, expect = [], [], []
    for zz in range(2, nz - 2):
        for yy in range(2, ny - 2):
            for xx in range(2, nx - 2):
                for i in range(10):
                    d = i / 10.0
                    pts.append((xx + 0.5 + d, yy + 0.5 - d, zz + 0.5 - d))
                    expect.append(xx + d + yy - d - zz + d)
                    dh = i * 0.5 / 10.0  # testComputeDistanceHessian's delta (SDF.cpp:829)
                    pts_h.append((xx + 0.5 + dh, yy + 0.5 - dh, zz + 0.5 - dh))
    pts = np.array(pts)
    pts_h = np.array(pts_h)
    save("linear_selftests", grid_size=n, field=f, points=pts, points_hessian=pts_h,
         expect=np.array(expect), distance=R.phi_sample(f, pts),
         weight=R.weight_sample(f.astype(np.int64), pts),
         gradient=R.distance_gradient_at(f, pts), hessian=R.distance_hessian_at(f, pts_h))


def jacobian_killing():
    """DisplacementField::testJacobian / testKillingEnergy (DisplacementField.cpp:142-272)."""
    P = Params()
    R = RefLib(P, 1)
    psi1 = np.zeros((8, 8, 8, 3))
    for x in range(5):
        for y in range(5):
            for z in range(5):
                psi1[z, y, x] = (x + y + z, x + z, y + z)
    jac = R.jacobian(psi1, 2.0, 2.0, 2.0)
    psi2 = np.zeros((8, 8, 8, 3))
    for x in range(8):
        for y in range(8):
            for z in range(8):
                psi2[z, y, x] = (x + y + z, x + z, y)
    pts = [(x, y, z) for x in range(7) for y in range(1, 7) for z in range(1, 7)]
    ke = np.array([R.killing_energy(psi2, *map(float, p)) for p in pts])
    jacs = np.array([R.jacobian(psi2, *map(float, p)) for p in pts])
    psi3 = np.zeros((8, 8, 8, 3))
    for x in range(8):
        psi3[:, :, x, 0] = x * x
    pts3 = [(x, y, z) for x in range(1, 7) for y in range(1, 7) for z in range(1, 7)]
    g_fd = np.array([R.killing_energy_gradient_fd(psi3, *p) for p in pts3])
    g_el = R.voxel_query("killing", np.zeros((8, 8, 8)), None, psi3, np.array(pts3))
    save("jacobian_killing", psi_linear=psi1, jacobian_222=jac, psi_killing=psi2,
         points=np.array(pts, dtype=np.float64), killing_energy=ke, jacobians=jacs,
         psi_square=psi3, points_square=np.array(pts3), grad_fd=g_fd, grad_clamped=g_el)


def two_spheres():
    """SDF::getDataEnergyTestSample + KillingFusion::processTest(3)
    (SDF.cpp:64-115, KillingFusion.cpp:177-207) with the Jacobi schedule."""
    P = Params()  # VoxelSize 0.012, clip 4 voxels (config.cpp:4-6)
    iters = 40
    R = RefLib(P, iters)
    phi0, w0, phi1, w1 = R.two_spheres(P.voxel_size, P.unknown_clip)
    st, psi = R.solve(phi1, phi0, np.zeros(phi0.shape + (3,)))
    assert st == 0
    fphi, fw = R.fuse_psi(phi0, w0, phi1, w1, psi)
    cphi, cw = R.fuse_psi(np.full_like(phi1, P.max_surface + P.epsilon), np.zeros_like(w1),
                          phi1, w1, psi)
    save("two_spheres", phi0=phi0, w0=w0, phi1=phi1, w1=w1, iterations=np.array(iters), psi=psi,
         fused_phi=fphi, fused_w=fw, deformed_phi=cphi, deformed_w=cw,
         mesh0=R.mesh(phi0), mesh_fused=R.mesh(fphi))


def sphere_pair_small():
    """24^3 sphere pair, paper weights: per-voxel gradient terms at a random
    psi, a 12-iteration Jacobi solve, warp + fuse and the meshes."""
    P = Params.paper(0.004)
    iters = 12
    R = RefLib(P, iters)
    can, live = small_pair(24, 0.004, 5.0, seed=7)
    can, live = can.astype(np.float64), live.astype(np.float64)
    rng = np.random.default_rng(11)
    psi_r = rng.normal(0.0, 0.3, can.shape + (3,)).astype(np.float32).astype(np.float64)
    z, y, x = np.meshgrid(*[np.arange(24)] * 3, indexing="ij")
    xyz = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.int32)
    # every voxel in the band, every voxel of the outer shell, and a sample of the rest
    flat = live.reshape(-1)
    band = (flat <= P.max_surface) & (flat >= -P.unknown_clip)
    shell = ((xyz == 0) | (xyz == 23)).any(axis=1)
    pick = band | shell | (rng.random(len(flat)) < 0.05)
    xyz = xyz[pick]
    grad = R.voxel_query("grad", live, can, psi_r, xyz)
    dgrad = R.voxel_query("dgrad", live, can, psi_r, xyz)
    hess = R.voxel_query("hess", live, can, psi_r, xyz)
    kill = R.voxel_query("killing", live, can, psi_r, xyz)
    warped = R.voxel_query("warped", live, can, psi_r, xyz)
    active = R.voxel_query("active", live, can, psi_r, xyz)
    st, psi = R.solve(live, can, np.zeros(can.shape + (3,)))
    assert st == 0
    wl = (live <= P.max_surface).astype(np.int64)
    wc = (can <= P.max_surface).astype(np.int64)
    uphi, uw = R.update(live, wl, psi)
    fphi, fw = R.fuse(can, wc, uphi, uw)
    save("sphere_pair_small", can=can, live=live, psi_random=psi_r, grad=grad, dgrad=dgrad,
         hess=hess, killing=kill, warped=warped, active=active, iterations=np.array(iters),
         psi=psi, w_live=wl, w_can=wc, warped_phi=uphi, warped_w=uw, fused_phi=fphi,
         fused_w=fw, mesh_can=R.mesh(can), mesh_fused=R.mesh(fphi))


def integrate_small():
    """SDF::integrateDepthFrame on a 20^3 grid from a 64x48 frame, identity and
    a rotated/translated camera pose."""
    P = Params.paper(0.01)
    R = RefLib(P, 1)
    rng = np.random.default_rng(5)
    h, w = 48, 64
    K = np.array([[50.0, 0.0, 31.5], [0.0, 50.0, 23.5], [0.0, 0.0, 1.0]])
    u, v = np.meshgrid(np.arange(w), np.arange(h))
    depth = 0.5 + 0.05 * np.sin(u / 7.0) * np.cos(v / 5.0) + rng.normal(0, 0.002, (h, w))
    depth[rng.random((h, w)) < 0.05] = 0.0
    depth = depth.astype(np.float32).astype(np.float64)
    n = (20, 20, 20)
    origin = np.array([-0.1, -0.1, 0.4])
    a = np.deg2rad(4.0)
    c2w = np.array([[np.cos(a), 0, np.sin(a), 0.01], [0, 1, 0, -0.005],
                    [-np.sin(a), 0, np.cos(a), 0.02], [0, 0, 0, 1.0]])
    out = {"depth": depth, "K": K, "origin": origin, "c2w": c2w}
    for tag, pose in (("eye", np.eye(4)), ("pose", c2w)):
        phi = np.full(n, P.max_surface + P.epsilon)
        wt = np.zeros(n, np.int64)
        phi, wt = R.integrate(phi, wt, 0.01, origin, P.unknown_clip, depth, pose, K, 0.05, 1.2)
        phi2, wt2 = R.integrate(phi, wt, 0.01, origin, P.unknown_clip, depth * 1.01, pose, K,
                                0.05, 1.2)
        out["phi_" + tag], out["w_" + tag] = phi, wt
        out["phi2_" + tag], out["w2_" + tag] = phi2, wt2
    save("integrate_small", **out)


def trust_region():
    """The Jacobi schedule with the trust-region step (UseTrustStrategy,
    KillingFusion.cpp:288-314), data term alone: 22^3 sphere pair, alpha 0.1,
    8 iterations.  At the sphere centre's row the step size underflows and
    the reference breaks out of the row's x loop."""
    P = Params.paper(0.004).with_(use_levelset=False, use_killing=False, use_trust=True)
    iters = 8
    R = RefLib(P, iters)
    can, live = small_pair(22, P.voxel_size, 5.0, seed=9)
    can, live = can.astype(np.float64), live.astype(np.float64)
    st, psi = R.solve(live, can, np.zeros(can.shape + (3,)))
    assert st == 0
    save("trust_region", can=can, live=live, iterations=np.array(iters), psi=psi)


FIXTURES = {f.__name__: f for f in (linear_selftests, jacobian_killing, two_spheres,
                                    sphere_pair_small, integrate_small, trust_region)}

if __name__ == "__main__":
    for name in sys.argv[1:] or list(FIXTURES):
        FIXTURES[name]()
