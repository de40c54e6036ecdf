"""Seeded synthetic depth sequences and analytic SDF pairs.

The reference runs on the Slavcheva Duck/Snoopy captures (config.cpp:13-19),
which are not available here; these generators stand in for them with the
shapes, sizes and noise levels of the benchmark workloads:

* ``sphere_pair``        -- 64^3, 4 mm: a sphere (r=30 mm, 400 mm ahead) and the
  same sphere moved 2 mm along +x and stretched 1.05x along x;
* ``ellipsoid_sequence`` -- 256^3, 5 mm: a union of 5 ellipsoids (semi-axes
  20-80 mm) whose far part bends about a seeded hinge, the bend angle
  following a sinusoid that changes by at most 2 degrees per frame;
* ``capsule_sequence``   -- 512^3, 2 mm: 7 capsules (radii 15-40 mm) chained
  into an articulated figure with seeded sinusoidal joint angles (<= 30 deg);
* ``blob_fields`` / ``shape_problem`` -- analytic SDFs (Gaussian-RBF blobs,
  sphere/ellipsoid/torus) for the gradient check and the batched solve.

Depth frames are float32 metres, 640x480, 0 where the ray misses.  Pixel
(row, col) is cast through image point (col-0.5, row-0.5): the integrator maps
a voxel to ``col = roundf(u+0.5)`` (SDF.cpp:167), so that is the ray whose
depth it reads there.  Gaussian noise comes from a counter-based generator
(SplitMix64 of (seed, frame, pixel) + Box-Muller), so a frame is a pure
function of its seed and index.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

WIDTH, HEIGHT = 640, 480
FX = FY = 525.0
CX, CY = 319.5, 239.5
K = np.array([[FX, 0.0, CX], [0.0, FY, CY], [0.0, 0.0, 1.0]])

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return z ^ (z >> np.uint64(31))


def counter_normal(seed: int, stream: int, count: int) -> np.ndarray:
    """count standard normals, a pure function of (seed, stream, index)."""
    with np.errstate(over="ignore"):
        base = _splitmix64(np.uint64(seed & 0xFFFFFFFFFFFFFFFF) ^ _splitmix64(np.uint64(stream)))
        idx = np.arange(count, dtype=np.uint64)
        a = _splitmix64(base ^ (idx * np.uint64(2)))
        b = _splitmix64(base ^ (idx * np.uint64(2) + np.uint64(1)))
    u1 = ((a >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    u2 = ((b >> np.uint64(11)).astype(np.float64)) * (1.0 / 9007199254740992.0)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def pixel_rays(width: int = WIDTH, height: int = HEIGHT, K: np.ndarray | None = None) -> np.ndarray:
    """Unnormalised ray directions (z = 1) per pixel, float64[h, w, 3]."""
    fx, fy, cx, cy = (FX, FY, CX, CY) if K is None else (K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    col = np.arange(width, dtype=np.float64) - 0.5
    row = np.arange(height, dtype=np.float64) - 0.5
    u, v = np.meshgrid(col, row)
    d = np.empty((height, width, 3))
    d[..., 0] = (u - cx) / fx
    d[..., 1] = (v - cy) / fy
    d[..., 2] = 1.0
    return d


def rot(axis, angle: float) -> np.ndarray:
    """Rotation matrix about a unit axis (Rodrigues)."""
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    k = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(angle) * k + (1 - np.cos(angle)) * (k @ k)


# ---------------------------------------------------------------------------
# ray casting
# ---------------------------------------------------------------------------

@dataclass
class Ellipsoid:
    centre: np.ndarray
    axes: np.ndarray                 # semi-axes (m)
    R: np.ndarray = field(default_factory=lambda: np.eye(3))  # local -> world

    def hit(self, d: np.ndarray) -> np.ndarray:
        """Smallest t > 0 with t*d on the surface (rays from the origin)."""
        o = (-self.centre) @ self.R / self.axes
        dl = (d @ self.R) / self.axes
        a = np.einsum("...k,...k->...", dl, dl)
        b = 2.0 * np.einsum("...k,k->...", dl, o)
        c = o @ o - 1.0
        disc = b * b - 4 * a * c
        t = np.full(d.shape[:-1], np.inf)
        ok = disc >= 0
        sq = np.sqrt(np.where(ok, disc, 0.0))
        t0 = (-b - sq) / (2 * a)
        t1 = (-b + sq) / (2 * a)
        tt = np.where(t0 > 0, t0, t1)
        return np.where(ok & (tt > 0), tt, t)


@dataclass
class Capsule:
    a: np.ndarray
    b: np.ndarray
    radius: float

    def hit(self, d: np.ndarray) -> np.ndarray:
        r = self.radius
        ab = self.b - self.a
        L2 = ab @ ab
        oa = -self.a
        t = np.full(d.shape[:-1], np.inf)
        # cylinder part
        dab = d @ ab
        oab = oa @ ab
        dd = np.einsum("...k,...k->...", d, d)
        doa = d @ oa
        qa = L2 * dd - dab * dab
        qb = 2 * (L2 * doa - dab * oab)
        qc = L2 * (oa @ oa) - oab * oab - r * r * L2
        disc = qb * qb - 4 * qa * qc
        ok = (disc >= 0) & (qa > 1e-18)
        sq = np.sqrt(np.where(ok, disc, 0.0))
        tc = (-qb - sq) / (2 * np.where(qa > 1e-18, qa, 1.0))
        s = (oab + tc * dab) / L2
        good = ok & (tc > 0) & (s >= 0) & (s <= 1)
        t = np.where(good, tc, t)
        for c in (self.a, self.b):
            sp = Ellipsoid(c, np.array([r, r, r]))
            t = np.minimum(t, sp.hit(d))
        return t


def render(shapes, rays: np.ndarray | None = None) -> np.ndarray:
    """Z-depth (float64, inf on a miss) of the union of shapes."""
    if rays is None:
        rays = pixel_rays()
    t = np.full(rays.shape[:-1], np.inf)
    for s in shapes:
        t = np.minimum(t, s.hit(rays))
    return t  # rays have z = 1, so t is the z-depth


def to_frame(depth: np.ndarray, sigma: float, seed: int, frame: int) -> np.ndarray:
    """Add seeded Gaussian noise, zero the misses, return float32 metres."""
    noise = counter_normal(seed, 1000 + frame, depth.size).reshape(depth.shape)
    out = np.where(np.isfinite(depth), depth + sigma * noise, 0.0)
    return out.astype(np.float32)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

@dataclass
class Grid:
    dims: tuple            # (nx, ny, nz)
    voxel: float           # m
    origin: np.ndarray     # world position of the grid's min corner (m)
    trunc_voxels: float = 5.0

    @property
    def trunc(self) -> float:
        return self.voxel * self.trunc_voxels

    @property
    def max3d(self) -> np.ndarray:
        """A max corner for which the reference's int(bound/v)+1 rule
        (SDF.cpp:117-124) yields exactly ``dims``."""
        return self.origin + (np.asarray(self.dims, dtype=np.float64) - 0.5) * self.voxel


def sphere_pair(seed: int = 1, sigma: float = 0.001):
    """64^3 / 4 mm: canonical sphere frame and the moved + stretched frame."""
    v = 0.004
    grid = Grid((64, 64, 64), v, np.array([-32 * v, -32 * v, 0.4 - 32 * v]))
    rays = pixel_rays()
    s0 = Ellipsoid(np.array([0.0, 0.0, 0.4]), np.array([0.03, 0.03, 0.03]))
    s1 = Ellipsoid(np.array([0.002, 0.0, 0.4]), np.array([0.03 * 1.05, 0.03, 0.03]))
    f0 = to_frame(render([s0], rays), sigma, seed, 0)
    f1 = to_frame(render([s1], rays), sigma, seed, 1)
    return grid, [f0, f1]


class SpherePairSequence:
    """sphere_pair as a sequence: frame 0 is the canonical sphere, every
    later frame the moved and stretched one (the small two-frame workload)."""

    def __init__(self, seed: int = 1, sigma: float = 0.001):
        self.grid, self._frames = sphere_pair(seed, sigma)
        self.frames = 2

    def frame(self, f: int) -> np.ndarray:
        return self._frames[0 if f == 0 else 1]


class EllipsoidSequence:
    """256^3 / 5 mm: union of 5 ellipsoids bending about a seeded hinge."""

    voxel = 0.005

    def __init__(self, seed: int = 2, frames: int = 30, sigma: float = 0.0015, n: int = 256):
        self.seed, self.frames, self.sigma = seed, frames, sigma
        v = self.voxel * 256 / n
        self.grid = Grid((n, n, n), v, np.array([-0.64, -0.64, 0.30]))
        rng = np.random.default_rng(seed)
        self.centres = np.stack([rng.uniform(-0.12, 0.12, 5), rng.uniform(-0.10, 0.10, 5),
                                 rng.uniform(0.72, 0.90, 5)], axis=1)
        self.axes = rng.uniform(0.020, 0.080, (5, 3))
        self.orients = [rot(rng.normal(size=3), rng.uniform(0, np.pi)) for _ in range(5)]
        self.hinge_point = self.centres.mean(axis=0)
        self.hinge_axis = rng.normal(size=3)
        self.hinge_axis /= np.linalg.norm(self.hinge_axis)
        normal = np.cross(self.hinge_axis, rng.normal(size=3))
        self.side = ((self.centres - self.hinge_point) @ normal) > 0
        period = 30.0
        self.omega = 2 * np.pi / period
        self.amp = np.deg2rad(2.0) / self.omega  # |d angle / d frame| <= 2 deg
        self._rays = None

    def angle(self, f: int) -> float:
        return self.amp * np.sin(self.omega * f)

    def shapes(self, f: int):
        R = rot(self.hinge_axis, self.angle(f))
        out = []
        for i in range(5):
            c, O = self.centres[i], self.orients[i]
            if self.side[i]:
                c = self.hinge_point + R @ (c - self.hinge_point)
                O = R @ O
            out.append(Ellipsoid(c, self.axes[i], O))
        return out

    def frame(self, f: int) -> np.ndarray:
        if self._rays is None:
            self._rays = pixel_rays()
        return to_frame(render(self.shapes(f), self._rays), self.sigma, self.seed, f)


class CapsuleSequence:
    """512^3 / 2 mm: 7 capsules chained into an articulated figure."""

    voxel = 0.002

    def __init__(self, seed: int = 5, frames: int = 100, sigma: float = 0.002, n: int = 512):
        self.seed, self.frames, self.sigma = seed, frames, sigma
        v = self.voxel * 512 / n
        self.grid = Grid((n, n, n), v, np.array([-0.512, -0.512, 0.35]))
        rng = np.random.default_rng(seed)
        self.radii = rng.uniform(0.015, 0.040, 7)
        self.lengths = rng.uniform(0.06, 0.14, 7)
        self.amps = np.deg2rad(rng.uniform(5.0, 30.0, 7))
        self.freqs = rng.uniform(0.05, 0.2, 7)
        self.phases = rng.uniform(0, 2 * np.pi, 7)
        self.axes = [rng.normal(size=3) for _ in range(7)]
        self.root = np.array([0.0, -0.05, 0.85])
        self.dirs = [np.array([0.0, 1.0, 0.0]), np.array([1.0, 0.3, 0.0]), np.array([-1.0, 0.3, 0.0]),
                     np.array([0.6, -1.0, 0.0]), np.array([-0.6, -1.0, 0.0]),
                     np.array([0.2, 1.0, 0.1]), np.array([0.0, -1.0, 0.2])]
        self.parent = [-1, 0, 0, -1, -1, 1, 3]
        self._rays = None

    def shapes(self, f: int):
        caps, ends, frames_R = [], [], []
        for i in range(7):
            ang = self.amps[i] * np.sin(2 * np.pi * self.freqs[i] * f / 10.0 + self.phases[i])
            R = rot(self.axes[i], ang)
            p = self.parent[i]
            if p < 0:
                start, Rp = self.root, np.eye(3)
            else:
                start, Rp = ends[p], frames_R[p]
            Rw = Rp @ R
            d = self.dirs[i] / np.linalg.norm(self.dirs[i])
            end = start + Rw @ d * self.lengths[i]
            caps.append(Capsule(start, end, self.radii[i]))
            ends.append(end)
            frames_R.append(Rw)
        return caps

    def frame(self, f: int) -> np.ndarray:
        if self._rays is None:
            self._rays = pixel_rays()
        return to_frame(render(self.shapes(f), self._rays), self.sigma, self.seed, f)


def blob_fields(seed: int = 3, n: int = 128, voxel: float = 0.004, trunc_voxels: float = 5.0):
    """Canonical and live SDFs of random smooth blobs plus a smooth psi.

    Each SDF is a sum of 16 Gaussian RBFs (sigma 10-40 mm) minus a threshold,
    turned into approximate signed distance (f - tau)/|grad f| and clamped to
    the truncation band; psi is a sum of 8 Gaussian RBFs with amplitude <= 2
    voxels.  Returns float32 arrays [nz, ny, nx] (psi [nz, ny, nx, 3]).
    """
    rng = np.random.default_rng(seed)
    ax = (np.arange(n) + 0.5) * voxel
    Z, Y, X = np.meshgrid(ax, ax, ax, indexing="ij")
    L = n * voxel
    trunc = voxel * trunc_voxels

    def blob(rng):
        f = np.zeros((n, n, n))
        gx = np.zeros_like(f); gy = np.zeros_like(f); gz = np.zeros_like(f)
        for _ in range(16):
            c = rng.uniform(0.25 * L, 0.75 * L, 3)
            s = rng.uniform(0.010, 0.040)
            a = rng.uniform(0.5, 1.0)
            dx, dy, dz = X - c[0], Y - c[1], Z - c[2]
            g = a * np.exp(-(dx * dx + dy * dy + dz * dz) / (2 * s * s))
            f += g
            gx -= g * dx / (s * s); gy -= g * dy / (s * s); gz -= g * dz / (s * s)
        tau = 0.35
        gn = np.sqrt(gx * gx + gy * gy + gz * gz) + 1e-9
        d = -(f - tau) / gn  # outside (f < tau) positive
        return np.clip(d, -trunc, trunc)

    can = blob(rng)
    live = blob(np.random.default_rng(seed + 1000))
    psi = np.zeros((n, n, n, 3))
    for _ in range(8):
        c = rng.uniform(0.2 * L, 0.8 * L, 3)
        s = rng.uniform(0.02, 0.08)
        amp = rng.uniform(-2.0, 2.0, 3) / 8.0 * 2.0
        g = np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / (2 * s * s))
        psi += g[..., None] * amp
    m = np.abs(psi).max()
    if m > 2.0:
        psi *= 2.0 / m
    return can.astype(np.float32), live.astype(np.float32), psi.astype(np.float32)


def shape_problem(seed: int, n: int, trunc_voxels: float = 5.0):
    """One two-frame registration problem of the batched workload.

    A sphere, ellipsoid or torus filling about half of an n^3 grid (voxel size
    scaled to the object), and the same shape after a rigid offset of up to 3
    voxels plus a smooth bend.  Returns (can, live) float32 [n, n, n] truncated
    SDFs and the voxel size.
    """
    rng = np.random.default_rng(seed)
    kind = int(rng.integers(0, 3))
    size = 0.10  # object extent (m)
    voxel = 2.0 * size / n
    ax = (np.arange(n) + 0.5) * voxel - n * voxel / 2
    Z, Y, X = np.meshgrid(ax, ax, ax, indexing="ij")
    trunc = voxel * trunc_voxels
    offset = rng.uniform(-3.0, 3.0, 3) * voxel
    bend = rng.uniform(-0.15, 0.15)
    axes = rng.uniform(0.6, 1.0, 3) * size * 0.45

    def sdf(X, Y, Z):
        if kind == 0:
            return np.sqrt(X * X + Y * Y + Z * Z) - axes[0]
        if kind == 1:
            q = np.sqrt((X / axes[0]) ** 2 + (Y / axes[1]) ** 2 + (Z / axes[2]) ** 2)
            return (q - 1.0) * axes.min()
        R, r = axes[0], axes[0] * 0.35
        qx = np.sqrt(X * X + Z * Z) - R
        return np.sqrt(qx * qx + Y * Y) - r

    can = sdf(X, Y, Z)
    # live: bend (x-dependent shear in y) and rigid offset
    Xl = X - offset[0]
    Yl = Y - offset[1] - bend * (Xl / size) ** 2 * size
    Zl = Z - offset[2]
    live = sdf(Xl, Yl, Zl)
    c = np.where(can > trunc, trunc + 1e-5, np.maximum(can, -trunc - 1e-3))
    lv = np.where(live > trunc, trunc + 1e-5, np.maximum(live, -trunc - 1e-3))
    return c.astype(np.float32), lv.astype(np.float32), voxel


def write_dataset(root: str, frames, K: np.ndarray, min_depth: float, max_depth: float) -> None:
    """Write float32 depth frames in the layout the C++ DatasetReader reads:
    intrinsics.txt (row-major K), meta.txt ("width height frames minDepth
    maxDepth") and depth_%06d.f32 (float32 metres, row-major)."""
    import os

    os.makedirs(root, exist_ok=True)
    frames = [np.ascontiguousarray(f, dtype=np.float32) for f in frames]
    h, w = frames[0].shape
    with open(os.path.join(root, "intrinsics.txt"), "w") as f:
        f.write(" ".join(repr(float(v)) for v in np.asarray(K, dtype=np.float64).reshape(-1)) + "\n")
    with open(os.path.join(root, "meta.txt"), "w") as f:
        f.write("%d %d %d %r %r\n" % (w, h, len(frames), float(min_depth), float(max_depth)))
    for i, d in enumerate(frames):
        d.tofile(os.path.join(root, "depth_%06d.f32" % i))


def frustum_bounds(K: np.ndarray, width: int, height: int, min_depth: float, max_depth: float):
    """KillingFusion::computeBounds (KillingFusion.cpp:478-519): min and max
    corner of the camera frustum between the two depths at pose = identity."""
    Ki = _inverse3(K)
    cu = [0, 0, width - 1, width - 1] * 2
    cv = [0, height - 1, height - 1, 0] * 2
    pts = []
    for j in range(8):
        d = min_depth if j < 4 else max_depth
        p = [(Ki[r][0] * cu[j] + Ki[r][1] * cv[j] + Ki[r][2] * 1.0) * d for r in range(2)] + [d]
        pts.append(p)
    pts = np.array(pts)
    return pts.min(axis=0), pts.max(axis=0)


def _inverse3(m):
    """3x3 inverse by cofactors, det expanded along column 0."""
    m = np.asarray(m, dtype=np.float64)

    def cof(i, j):
        i1, i2, j1, j2 = (i + 1) % 3, (i + 2) % 3, (j + 1) % 3, (j + 2) % 3
        return float(m[i1, j1] * m[i2, j2] - m[i1, j2] * m[i2, j1])

    det = cof(0, 0) * m[0, 0] + cof(1, 0) * m[1, 0] + cof(2, 0) * m[2, 0]
    inv_det = 1.0 / float(det)
    return [[cof(j, i) * inv_det for j in range(3)] for i in range(3)]


def grid_from_bounds(lo, hi, voxel: float):
    """SDF::computeVoxelGridSize (SDF.cpp:117-124): int(bound / voxel) + 1."""
    return tuple(int((float(hi[k]) - float(lo[k])) / voxel) + 1 for k in range(3))

