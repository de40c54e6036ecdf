"""The C++ class layer (SDF, DisplacementField, KillingFusion, DatasetReader,
SimpleMesh over the C ABI) against the oracle: a small C++ driver
(tests/cpp/host_driver.cpp) runs the reference's call shapes and writes the
reference's file formats; these tests read them back.

Tolerances as in test_gpu_parity: float64 "exact" solver bit-identical to the
oracle, SDF values equal to the oracle's doubles rounded to float32, weights
and triangle counts exact; OFF vertices to the writer's 6 significant digits.
"""
import os
import subprocess

import numpy as np
import pytest

from killingfusion_gb300 import synth
from oracle.oracle import Params as OParams

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def driver(gpu, tmp_path_factory):
    from killingfusion_gb300 import _build
    _build.build()
    lib = os.path.join(ROOT, "killingfusion_gb300", "_lib")
    exe = str(tmp_path_factory.mktemp("driver") / "host_driver")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "killingfusion_gb300", "csrc", "host"),
                    os.path.join(HERE, "cpp", "host_driver.cpp"), "-L", lib, "-lkf_host",
                    "-lkillingfusion", "-Wl,-rpath," + lib, "-o", exe], check=True)

    def run(*args):
        r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        return r.stdout

    return run


def read_sdf_bin(path):
    """SDF::dumpToBinFile: int32 dims[3], f64 min[3], f64 voxel, f64 trunc,
    f64 phi[N] (SDF.cpp:432-446)."""
    raw = open(path, "rb").read()
    dims = np.frombuffer(raw, np.int32, 3)
    head = np.frombuffer(raw, np.float64, 5, offset=12)
    phi = np.frombuffer(raw, np.float64, offset=12 + 40).reshape(dims[::-1])
    return dims, head, phi


def read_psi_bin(path):
    """DisplacementField::dumpToBinFile: int32 dims[3], f64 voxel, f64 xyz[N][3]
    (DisplacementField.cpp:349-366)."""
    raw = open(path, "rb").read()
    dims = np.frombuffer(raw, np.int32, 3)
    psi = np.frombuffer(raw, np.float64, offset=20).reshape(tuple(dims[::-1]) + (3,))
    return dims, psi


def read_off(path):
    with open(path) as f:
        assert f.readline().strip() == "OFF"
        nv, nt, _ = (int(v) for v in f.readline().split())
        v = np.array([[float(t) for t in f.readline().split()] for _ in range(nv)])
        t = np.array([[int(t) for t in f.readline().split()] for _ in range(nt)])
    return v.reshape(-1, 3), t.reshape(-1, 4)


def assert_mesh(path, soup):
    """An OFF written by SimpleMesh::WriteMesh against the oracle's soup."""
    v, t = read_off(path)
    assert len(t) == len(soup)
    if len(t):
        assert (t[:, 0] == 3).all()
        np.testing.assert_array_equal(t[:, 1:], np.arange(3 * len(t)).reshape(-1, 3))
        np.testing.assert_allclose(v, soup.reshape(-1, 3), rtol=1e-5, atol=1e-6)


def f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def test_process_test_spheres(driver, oracle, tmp_path):
    """KillingFusion::processTest(1..3) on SDF::getDataEnergyTestSample
    (KillingFusion.cpp:177-207, SDF.cpp:64-115) with the exact solver."""
    gold = np.load(os.path.join(HERE, "golden", "two_spheres.npz"))
    iters = int(gold["iterations"])
    K = np.array(synth.K)
    synth.write_dataset(str(tmp_path / "dataset"), [np.zeros((48, 64), np.float32)], K, 0.3, 0.5)
    out = driver("spheres", tmp_path, "exact", iters)
    assert "solve iterations %d" % iters in out
    P = OParams()  # the reference's config.cpp values
    phi0, w0 = f32(gold["phi0"]), gold["w0"]
    phi1, w1 = f32(gold["phi1"]), gold["w1"]
    dims, head, s0 = read_sdf_bin(tmp_path / "testType-1-outputSphere0.bin")
    assert tuple(dims) == (10, 10, 10)
    np.testing.assert_array_equal(head, [0, 0, 0, P.voxel_size, P.unknown_clip])
    np.testing.assert_array_equal(s0, phi0)
    np.testing.assert_array_equal(read_sdf_bin(tmp_path / "testType-1-outputSphere1.bin")[2], phi1)
    # processTest(1): fuse into itself; (2): sphere 1 into sphere 0
    ophi, _ = oracle.fuse(phi0, w0, phi0, w0)
    np.testing.assert_array_equal(read_sdf_bin(tmp_path / "testType-1-outputSphere0MergedTo0.bin")[2],
                                  f32(ophi))
    ophi, _ = oracle.fuse(phi0, w0, phi1, w1)
    np.testing.assert_array_equal(read_sdf_bin(tmp_path / "testType-1-outputSphere1MergedTo0.bin")[2],
                                  f32(ophi))
    # processTest(3): register sphere 1 onto sphere 0, fuse along psi
    st, psi = oracle.solve(phi1, phi0, np.zeros(phi0.shape + (3,)), iters, P)
    assert st == 0
    fphi, _ = oracle.fuse_psi(phi0, w0, phi1, w1, psi, P)
    init = np.full_like(phi1, f32(P.max_surface + P.epsilon))
    dphi, _ = oracle.fuse_psi(init, np.zeros_like(w1), phi1, w1, psi, P)
    merged = read_sdf_bin(tmp_path / "testType-2-outputSphere1MergedTo0UsingKilling.bin")[2]
    deformed = read_sdf_bin(tmp_path / "testType-2-outputSphere1Deformed.bin")[2]
    np.testing.assert_array_equal(merged, f32(fphi))
    np.testing.assert_array_equal(deformed, f32(dphi))
    # and the reference's own float64 run, through float32 storage
    np.testing.assert_allclose(psi, gold["psi"], atol=1e-5)
    np.testing.assert_allclose(merged, gold["fused_phi"], atol=1e-6)


def test_process_test_spheres_trust_region(driver, oracle, tmp_path):
    """kf::Config's UseTrustStrategy with the data term alone reaches the
    solver: processTest(3) registers with the trust-region step
    (KillingFusion.cpp:288-314), bit for bit with the oracle, and differs
    from the plain data-term step."""
    gold = np.load(os.path.join(HERE, "golden", "two_spheres.npz"))
    iters, alpha = 40, 0.5
    K = np.array(synth.K)
    synth.write_dataset(str(tmp_path / "dataset"), [np.zeros((48, 64), np.float32)], K, 0.3, 0.5)
    driver("spheres", tmp_path, "exact", iters, "trust", alpha)
    P = OParams().with_(use_levelset=False, use_killing=False, use_trust=True, alpha=alpha)
    phi0, w0 = f32(gold["phi0"]), gold["w0"]
    phi1, w1 = f32(gold["phi1"]), gold["w1"]
    st, psi = oracle.solve(phi1, phi0, np.zeros(phi0.shape + (3,)), iters, P)
    assert st == 0
    fphi, _ = oracle.fuse_psi(phi0, w0, phi1, w1, psi, P)
    merged = read_sdf_bin(tmp_path / "testType-2-outputSphere1MergedTo0UsingKilling.bin")[2]
    np.testing.assert_array_equal(merged, f32(fphi))
    _, plain = oracle.solve(phi1, phi0, np.zeros(phi0.shape + (3,)), iters, P.with_(use_trust=False))
    pphi, _ = oracle.fuse_psi(phi0, w0, phi1, w1, plain, P)
    assert np.any(f32(pphi) != merged)


def test_reference_selftests_on_the_classes(driver):
    """SDF::testGetDistance/testGetWeight/testComputeDistanceGradient/
    testComputeDistanceHessian and DisplacementField::testJacobian/
    testKillingEnergy (public static methods of the reference's classes,
    SDF.cpp:526-840, DisplacementField.cpp:142-272) pass on the drop-in
    classes; the Jacobian at (2,2,2) is the analytical one."""
    out = driver("selftests")
    assert "selftests ok" in out
    lines = out.splitlines()
    k = lines.index("numericalJacobian at 2,2,2 is ")
    J = np.array([[float(v) for v in lines[k + 1 + r].split()] for r in range(3)])
    np.testing.assert_allclose(J, [[1, 1, 1], [1, 0, 1], [0, 1, 1]], atol=1e-9)
    assert "Killing energy gradient forms differ at" in out


def small_camera_frames(n_frames=3, seed=4):
    """A 64x48 camera (f = 52.5 px) looking at a sphere that moves and
    stretches along x, float32 metres."""
    K = np.array([[52.5, 0.0, 31.5], [0.0, 52.5, 23.5], [0.0, 0.0, 1.0]])
    rays = synth.pixel_rays(64, 48, K)
    frames = []
    for f in range(n_frames):
        s = synth.Ellipsoid(np.array([0.004 * f, 0.0, 0.4]), np.array([0.06 * (1 + 0.03 * f), 0.06, 0.06]))
        frames.append(synth.to_frame(synth.render([s], rays), 0.001, seed, f))
    return K, frames


def test_dataset_pipeline(driver, oracle, tmp_path):
    """DatasetReader + KillingFusion::processNextFrame over three frames
    (KillingFusion.cpp:109-175, computeBounds :478-519): meshes, psi and the
    canonical SDF against the oracle replaying the same sequence."""
    K, frames = small_camera_frames(3)
    min_d, max_d, voxel, iters = 0.3, 0.5, 0.008, 20
    root = tmp_path / "data"
    synth.write_dataset(str(root), frames, K, min_d, max_d)
    out = tmp_path / "out"
    out.mkdir()
    log = driver("dataset", root, out, "exact", iters, len(frames), voxel)
    assert "frame index 3" in log
    lo, hi = synth.frustum_bounds(K, 64, 48, min_d, max_d)
    dims = synth.grid_from_bounds(lo, hi, voxel)
    P = OParams(voxel_size=voxel, unknown_clip=5 * voxel, max_surface=5 * voxel, alpha=0.1,
                omega_k=0.5, gamma_k=0.1, omega_s=0.2)
    shape = dims[::-1]
    init = f32(np.full(shape, P.max_surface + P.epsilon))

    def integrate(frame):
        phi, w = oracle.integrate(init, np.zeros(shape, np.int64), voxel, lo, P.unknown_clip,
                                  frame.astype(np.float64), np.eye(4), K, min_d, max_d)
        return f32(phi), w

    can, cw = integrate(frames[0])
    assert (cw > 0).sum() > 500
    assert_mesh(out / "live_000.off", oracle.mesh(can, P))
    reg0, _ = oracle.fuse_psi(init, np.zeros(shape, np.int64), can, cw, np.zeros(shape + (3,)), P)
    assert_mesh(out / "registered_000.off", oracle.mesh(f32(reg0), P))
    assert_mesh(out / "canonical_000.off", oracle.mesh(can, P))
    _, psi_dump = read_psi_bin(out / "psi_000.bin")
    assert not psi_dump.any()
    for f in (1, 2):
        live, lw = integrate(frames[f])
        st, psi = oracle.solve(live, can, np.zeros(shape + (3,)), iters, P)
        assert st == 0
        d, psi_dump = read_psi_bin(out / ("psi_%03d.bin" % f))
        assert tuple(d) == dims
        np.testing.assert_array_equal(psi_dump, psi)
        assert_mesh(out / ("live_%03d.off" % f), oracle.mesh(live, P))
        uphi, uw = oracle.update(live, lw, psi, P)
        uphi = f32(uphi)
        fphi, cw = oracle.fuse(can, cw, uphi, uw)
        can = f32(fphi)
        assert_mesh(out / ("registered_%03d.off" % f), oracle.mesh(uphi, P))
        assert_mesh(out / ("canonical_%03d.off" % f), oracle.mesh(can, P))
    d, head, phi = read_sdf_bin(out / "canonical.bin")
    assert tuple(d) == dims
    np.testing.assert_array_equal(head[:3], lo)
    np.testing.assert_array_equal(phi, can)


def test_point_queries(driver, oracle, tmp_path):
    """SDF and DisplacementField point accessors (SDF.cpp:475-886,
    DisplacementField.cpp:22-347) against the oracle's samplers."""
    from helpers import small_pair
    voxel = 0.004
    P = OParams(voxel_size=voxel, unknown_clip=0.02, max_surface=0.02)
    can, live = small_pair(16, voxel, 5.0, seed=31)
    nz, ny, nx = live.shape
    rng = np.random.default_rng(5)
    w = rng.integers(0, 4, live.shape).astype(np.int32)
    psi = rng.normal(0, 0.4, live.shape + (3,)).astype(np.float32)
    with open(tmp_path / "grid.f32", "wb") as f:
        np.array([nx, ny, nz], np.int32).tofile(f)
        live.astype(np.float32).tofile(f)
        w.tofile(f)
    with open(tmp_path / "psi.bin", "wb") as f:
        np.array([nx, ny, nz], np.int32).tofile(f)
        np.array([voxel], np.float64).tofile(f)
        psi.astype(np.float64).tofile(f)
    pts = rng.uniform(-1.0, 17.0, (60, 3))
    pts[:5] = [[0.5, 0.5, 0.5], [15.5, 15.5, 15.5], [0.0, 3.0, 4.0], [16.0, 2.0, 2.0], [7.25, 8.5, 9.75]]
    vox = rng.integers(0, 16, (60, 3)).astype(np.int32)
    vox[:4] = [[-1, 3, 3], [16, 3, 3], [0, 0, 0], [15, 15, 15]]
    with open(tmp_path / "points.f64", "wb") as f:
        np.array([len(pts)], np.int32).tofile(f)
        pts.tofile(f)
    with open(tmp_path / "voxels.i32", "wb") as f:
        np.array([len(vox)], np.int32).tofile(f)
        vox.tofile(f)
    driver("points", tmp_path)
    res = np.fromfile(tmp_path / "queries.f64", np.float64)
    per_p, per_v = 1 + 1 + 3 + 9 + 3 + 1 + 9 + 1, 1 + 1 + 1 + 1 + 3 + 9 + 3 + 3
    assert res.size == len(pts) * per_p + len(vox) * per_v
    phi64, w64, psi64 = live.astype(np.float64), w.astype(np.int64), psi.astype(np.float64)
    rp = res[:len(pts) * per_p].reshape(len(pts), per_p)
    for i, p in enumerate(pts):
        d = oracle.psi_sample(psi64, p)
        expect = np.concatenate([
            [oracle.phi_sample(phi64, p, P), oracle.weight_sample(w64, p)],
            oracle.distance_gradient_at(phi64, p, P), oracle.distance_hessian_at(phi64, p, P).ravel(),
            d, [oracle.phi_sample(phi64, (p + d) + 0.5, P)],
            oracle.jacobian(psi64, *p, P).ravel(), [oracle.killing_energy(psi64, *p, P)]])
        np.testing.assert_array_equal(rp[i], expect, err_msg="point %d %s" % (i, p))
    rv = res[len(pts) * per_p:].reshape(len(vox), per_v)
    oob = P.max_surface + P.epsilon
    for i, v in enumerate(vox):
        x, y, z = (int(t) for t in v)
        inside = 0 <= x < nx and 0 <= y < ny and 0 <= z < nz
        lin = z * nx * ny + y * nx + x
        dv = psi64.reshape(-1, 3)[lin] if 0 <= lin < nx * ny * nz else np.zeros(3)
        q = (v.astype(np.float64) + dv) + 0.5
        expect = np.concatenate([
            [phi64[z, y, x] if inside else oob, w64[z, y, x] if inside else 0],
            oracle.voxel_query("warped", phi64, None, psi64, [v], P)[0],
            [oracle.weight_sample(w64, q)],
            oracle.voxel_query("dgrad", phi64, None, psi64, [v], P)[0],
            oracle.voxel_query("hess", phi64, None, psi64, [v], P)[0],
            dv, oracle.voxel_query("killing", phi64, None, psi64, [v], P)[0]])
        np.testing.assert_array_equal(rv[i], expect, err_msg="voxel %d %s" % (i, v))


def test_reference_dataset_layout(driver, oracle, tmp_path):
    """DatasetReader on the reference's own layout (Snoopy/depth_%06d.png in
    millimetres, omask_%06d.png, intrinsics_kinect1.txt; DatasetReader.cpp:15-66)
    with the reference's default configuration: the masked 16-bit depth is
    integrated as the reference's double metres, bit for bit."""
    import pngio
    grid, frames = synth.sphere_pair()
    root = tmp_path / "data"
    (root / "Snoopy").mkdir(parents=True)
    with open(root / "intrinsics_kinect1.txt", "w") as f:
        f.write(" ".join(repr(float(v)) for v in synth.K.ravel()) + "\n")
    depth_m = []
    for k, fr in enumerate(frames):
        mm = np.round(fr.astype(np.float64) * 1000.0).astype(np.uint16)
        mask = (mm > 0).astype(np.uint8) * 255
        mask[:, :200] = 0  # the left of the frame is masked out
        pngio.write(root / "Snoopy" / ("depth_%06d.png" % k), mm)
        pngio.write(root / "Snoopy" / ("omask_%06d.png" % k), mask)
        depth_m.append(np.where(mask > 0, mm.astype(np.float64) * (1.0 / 1000), 0.0))
    out = tmp_path / "out"
    out.mkdir()
    log = driver("refdataset", root, out, "exact", 4, 2)
    assert "frames 630 depth 0.0495164 1.2" in log
    P = OParams()  # config.cpp values
    lo, hi = synth.frustum_bounds(synth.K, 640, 480, 0.0495164, 1.2)
    dims = synth.grid_from_bounds(lo, hi, P.voxel_size)
    shape = dims[::-1]
    init = f32(np.full(shape, P.max_surface + P.epsilon))

    def integrate(d):
        phi, w = oracle.integrate(init, np.zeros(shape, np.int64), P.voxel_size, lo, P.unknown_clip, d,
                                  np.eye(4), synth.K, 0.0495164, 1.2)
        return f32(phi), w

    can, cw = integrate(depth_m[0])
    assert (cw > 0).sum() > 100
    live, lw = integrate(depth_m[1])
    st, psi = oracle.solve(live, can, np.zeros(shape + (3,)), 4, P)
    assert st == 0
    np.testing.assert_array_equal(read_psi_bin(out / "psi_001.bin")[1], psi)
    uphi, uw = oracle.update(live, lw, psi, P)
    fphi, _ = oracle.fuse(can, cw, f32(uphi), uw)
    d, head, phi = read_sdf_bin(out / "canonical.bin")
    assert tuple(d) == dims
    np.testing.assert_array_equal(phi, f32(fphi))
    assert_mesh(out / "live_001.off", oracle.mesh(live, P))


def test_process_carries_psi_and_fuses_through_it(driver, oracle, tmp_path):
    """KillingFusion::process (KillingFusion.cpp:41-107): frames 4.. of the
    sequence, psi carried from frame to frame, SDF::fuse(other, psi) into the
    canonical SDF and the registered meshes through SDF::save_mesh(.., psi);
    FinalCanonicalModel.bin at the end."""
    K, frames = small_camera_frames(7)
    min_d, max_d, voxel, iters = 0.3, 0.5, 0.008, 6
    root = tmp_path / "data"
    synth.write_dataset(str(root), frames, K, min_d, max_d)
    out = tmp_path / "out"
    out.mkdir()
    driver("process", root, out, "exact", iters, voxel)
    lo, hi = synth.frustum_bounds(K, 64, 48, min_d, max_d)
    dims = synth.grid_from_bounds(lo, hi, voxel)
    P = OParams(voxel_size=voxel, unknown_clip=5 * voxel, max_surface=5 * voxel)
    shape = dims[::-1]
    init = f32(np.full(shape, P.max_surface + P.epsilon))
    zero_w = np.zeros(shape, np.int64)

    def integrate(frame):
        phi, w = oracle.integrate(init, zero_w, voxel, lo, P.unknown_clip, frame.astype(np.float64),
                                  np.eye(4), K, min_d, max_d)
        return f32(phi), w

    prev, pw = integrate(frames[4])
    can, cw = oracle.fuse(init, zero_w, prev, pw)
    can = f32(can)
    for name in ("InputFrameSDF", "RegisteredFrameSDF", "CanonicalSDF", "LiveCanonicalSdf"):
        assert_mesh(out / ("%s004.off" % name), oracle.mesh(prev, P))
    psi = np.zeros(shape + (3,))
    for i in (5, 6):
        cur, curw = integrate(frames[i])
        assert_mesh(out / ("InputFrameSDF%03d.off" % i), oracle.mesh(cur, P))
        st, psi = oracle.solve(cur, can, psi, iters, P)
        assert st == 0
        reg, _ = oracle.fuse_psi(init, zero_w, cur, curw, psi, P)
        assert_mesh(out / ("RegisteredFrameSDF%03d.off" % i), oracle.mesh(f32(reg), P))
        can, cw = oracle.fuse_psi(can, cw, cur, curw, psi, P)
        can = f32(can)
        assert_mesh(out / ("CanonicalSDF%03d.off" % i), oracle.mesh(can, P))
    d, head, phi = read_sdf_bin(out / "FinalCanonicalModel.bin")
    assert tuple(d) == dims
    np.testing.assert_array_equal(phi, can)
