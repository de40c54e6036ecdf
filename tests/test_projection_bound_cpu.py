"""The float projection of integration and its error bound, restated in numpy
float32 and checked against the float64 projection of SDF::integrateDepthFrame
(SDF.cpp:151-172) on random poses, intrinsics and grids, on the CPU.

k_integrate decides a voxel's pixel in float from per-axis tables when u and
v lie farther than a per-voxel bound from a pixel edge (project_float in
csrc/kf_exact.cu), and k_integrate_tiles drops a 32 x 8 tile when the
corners' float projections, widened by the same bounds, put every voxel off
the image or onto pixel blocks without a valid depth.  This test models that
arithmetic operation for operation (numpy float32 rounds each operation to
nearest; the approximate reciprocal is modelled as the rounded one moved by
up to two ulps at random) and checks both claims at every voxel:
* a voxel the float path decides gets the reference's pixel;
* no voxel of a dropped tile has a pixel in the image that passes the depth
  test.
The GPU tests check the kernels themselves against the oracle; this one
covers poses and grids far beyond theirs, cheaply.
"""
import numpy as np
import pytest

f32 = np.float32
TILE_X, TILE_Y, PIX = 32, 8, 16


def pixel_of(u):
    """roundf((float)(u + 0.5)), half away from zero; -1 when not finite."""
    f = (u + 0.5).astype(np.float32).astype(np.float64)
    r = np.floor(np.abs(f) + 0.5) * np.sign(f)
    return np.where(np.isfinite(f), r, -1).astype(np.int64)


def reference_pixels(W, K, ax):
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    c = [((W[4 * r] * X + W[4 * r + 1] * Y) + W[4 * r + 2] * Z) + W[4 * r + 3] * 1.0 for r in range(3)]
    with np.errstate(all="ignore"):
        pa, pb = c[0] / c[2], c[1] / c[2]
        u = (K[0] * pa + K[1] * pb) + K[2] * 1.0
        v = (K[3] * pa + K[4] * pb) + K[5] * 1.0
    return pixel_of(u), pixel_of(v)


class FloatProjection:
    """project_float of csrc/kf_exact.cu for all voxels of a grid."""

    def __init__(self, W, K, ax, rng):
        r0 = [W[0] * ax[0] + W[3], W[1] * ax[1], W[2] * ax[2]]
        r1 = [W[4] * ax[0] + W[7], W[5] * ax[1], W[6] * ax[2]]
        r2 = [W[8] * ax[0] + W[11], W[9] * ax[1], W[10] * ax[2]]
        self.tab = [[t.astype(f32) for t in r] for r in (r0, r1, r2)]
        T = [abs(W[3]), abs(W[7]), abs(W[11])]
        for c in range(3):
            lo, hi = ax[c][0], ax[c][-1]
            for r in range(3):
                T[r] += abs(W[4 * r + c]) * max(abs(lo), abs(hi))
        up = 1.0 + 2.0 ** -20
        self.e = [f32(3.0001 * T[r] * 2.0 ** -24 * up) for r in range(3)]
        self.ku0, self.ku1, self.kv0, self.kv1 = [f32(1.5 * abs(k) * up) for k in (K[0], K[1], K[3], K[4])]
        self.c2_min = f32(max(8.0 * float(self.e[2]), 2.0 ** -100))
        self.Kf = K[:6].astype(f32)
        self.rng = rng

    def at(self, x, y, z):
        t = self.tab
        c0 = (t[0][0][x] + t[0][1][y]) + t[0][2][z]
        c1 = (t[1][0][x] + t[1][1][y]) + t[1][2][z]
        c2 = (t[2][0][x] + t[2][1][y]) + t[2][2][z]
        with np.errstate(all="ignore"):
            rc = f32(1) / c2
            for _ in range(2):  # __fdividef: within two ulps
                step = self.rng.integers(-1, 2, rc.shape)
                rc = np.where(step > 0, np.nextafter(rc, f32(np.inf)),
                              np.where(step < 0, np.nextafter(rc, f32(-np.inf)), rc))
            pa, pb = c0 * rc, c1 * rc
            Kf = self.Kf
            ua, ub, va, vb = Kf[0] * pa, Kf[1] * pb, Kf[3] * pa, Kf[4] * pb
            uf = (ua + ub) + Kf[2]
            vf = (va + vb) + Kf[5]
            arc = np.abs(rc)
            ea = self.e[0] + np.abs(pa) * self.e[2]
            eb = self.e[1] + np.abs(pb) * self.e[2]
            s_u = np.abs(ua) + np.abs(ub) + (abs(Kf[2]) + f32(2))
            s_v = np.abs(va) + np.abs(vb) + (abs(Kf[5]) + f32(2))
            mu = (self.ku0 * ea + self.ku1 * eb) * arc + f32(2 ** -19) * s_u
            mv = (self.kv0 * ea + self.kv1 * eb) * arc + f32(2 ** -19) * s_v
        return c2, uf, vf, mu, mv


def random_case(rng, far):
    """A camera looking at a grid placed in front of it, anywhere in the
    world: world = c2w * camera, the grid's centre at depth 0.3-2 m."""
    a = rng.normal(size=3)
    a *= np.deg2rad(rng.uniform(0, 35)) / np.linalg.norm(a)
    th = np.linalg.norm(a)
    k = a / th
    Kx = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    R = np.eye(3) + np.sin(th) * Kx + (1 - np.cos(th)) * Kx @ Kx
    t = rng.uniform(-300, 300, 3) if far else rng.uniform(-2, 2, 3)
    c2w = np.eye(4)
    c2w[:3, :3], c2w[:3, 3] = R, t
    w2c = np.linalg.inv(c2w)
    dims = tuple(int(v) for v in rng.integers(33, 70, 3))
    voxel = rng.uniform(0.003, 0.012)
    centre_cam = np.array([rng.uniform(-0.2, 0.2), rng.uniform(-0.2, 0.2), rng.uniform(0.3, 2.0)])
    centre_world = R @ centre_cam + t
    origin = centre_world - voxel * np.array(dims) / 2
    f = rng.uniform(300, 1000)
    W_img, H_img = int(rng.integers(160, 800)), int(rng.integers(120, 600))
    K = np.array([f, 0.0, (W_img - 1) / 2, 0.0, f * rng.uniform(0.95, 1.05), (H_img - 1) / 2, 0, 0, 1])
    return w2c.ravel(), K, dims, voxel, origin, W_img, H_img


def check_case(seed):
    """Both claims on random case `seed`; returns the number of tiles dropped."""
    rng = np.random.default_rng(seed)
    W, K, dims, voxel, origin, w_img, h_img = random_case(rng, far=seed % 3 == 2)
    ax = [voxel * (np.arange(n) + 0.5) + origin[c] for c, n in enumerate(dims)]
    nx, ny, nz = dims
    col_ref, row_ref = reference_pixels(W, K, ax)
    P = FloatProjection(W, K, ax, rng)
    Z, Y, X = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    c2, uf, vf, mu, mv = P.at(X, Y, Z)
    with np.errstate(all="ignore"):
        sure = (np.abs(c2) > P.c2_min) & (np.abs(c2) < 2.0 ** 100) & np.isfinite(uf) & np.isfinite(vf) & \
            (np.abs(uf) < 1e7) & (np.abs(vf) < 1e7) & (np.abs(uf - np.rint(uf)) > mu) & (np.abs(vf - np.rint(vf)) > mv)
        col = np.where(uf < -1, -1, np.floor(uf + f32(1))).astype(np.int64)
        row = np.where(vf < -1, -1, np.floor(vf + f32(1))).astype(np.int64)
    inside_ref = (col_ref >= 0) & (col_ref < w_img) & (row_ref >= 0) & (row_ref < h_img)
    inside = (col >= 0) & (col < w_img) & (row >= 0) & (row < h_img)
    # a decided voxel: the same in-or-out verdict, and inside the same pixel
    assert np.all(inside[sure] == inside_ref[sure])
    both = sure & inside
    assert np.all(col[both] == col_ref[both]) and np.all(row[both] == row_ref[both])
    assert sure.mean() > 0.3

    # tile culling against a random depth-validity mask (some 16 x 16 blocks valid)
    valid = np.zeros((h_img, w_img), bool)
    bw, bh = (w_img + PIX - 1) // PIX, (h_img + PIX - 1) // PIX
    blocks = rng.random((bh, bw)) < 0.15
    for by, bx in zip(*np.nonzero(blocks)):
        r0, c0 = by * PIX, bx * PIX
        valid[r0 + rng.integers(0, PIX):r0 + PIX, c0 + rng.integers(0, PIX):c0 + PIX] = True
    flags = np.array([[valid[by * PIX:(by + 1) * PIX, bx * PIX:(bx + 1) * PIX].any() for bx in range(bw)]
                      for by in range(bh)])
    integrable = np.zeros(col_ref.shape, bool)
    integrable[inside_ref] = valid[row_ref[inside_ref], col_ref[inside_ref]]
    culled = 0
    for z in range(nz):
        for ty in range((ny + TILE_Y - 1) // TILE_Y):
            for tx in range((nx + TILE_X - 1) // TILE_X):
                x0, y0 = tx * TILE_X, ty * TILE_Y
                x1, y1 = min(x0 + TILE_X - 1, nx - 1), min(y0 + TILE_Y - 1, ny - 1)
                cx = np.array([x0, x1, x0, x1])
                cy = np.array([y0, y0, y1, y1])
                cc2, cu, cv, cmu, cmv = P.at(cx, cy, np.full(4, z))
                with np.errstate(all="ignore"):
                    ok = np.all((cc2 > P.c2_min) & np.isfinite(cu) & np.isfinite(cv) & (np.abs(cu) < 1e7) &
                                (np.abs(cv) < 1e7) & (cmu < 1e6) & (cmv < 1e6))
                if not ok:
                    continue
                ulo, uhi = np.min(cu - cmu), np.max(cu + cmu)
                vlo, vhi = np.min(cv - cmv), np.max(cv + cmv)
                drop = uhi < -1.001 or ulo > w_img - 0.999 or vhi < -1.001 or vlo > h_img - 0.999
                if not drop:
                    c_lo, c_hi = max(0, int(np.floor(ulo + 1)) - 1), min(w_img - 1, int(np.floor(uhi + 1)) + 1)
                    r_lo, r_hi = max(0, int(np.floor(vlo + 1)) - 1), min(h_img - 1, int(np.floor(vhi + 1)) + 1)
                    drop = not flags[r_lo // PIX:r_hi // PIX + 1, c_lo // PIX:c_hi // PIX + 1].any()
                if drop:
                    culled += 1
                    assert not integrable[z, y0:y1 + 1, x0:x1 + 1].any(), (z, ty, tx)
    return culled


@pytest.mark.parametrize("seed", range(12))
def test_float_projection_and_tile_culling(seed):
    check_case(seed)


def test_tile_culling_is_exercised():
    """The random cases drop tiles, both off the image and on empty blocks."""
    assert sum(check_case(seed) for seed in range(12, 16)) > 100
