"""Shared inputs for the tests: small seeded SDF pairs and the 64^3 sphere
pair of the small benchmark configuration, in the oracle's layouts."""
import numpy as np

from killingfusion_gb300 import synth


def sphere_sdf(n, centre, radius, voxel, trunc, scale=(1.0, 1.0, 1.0)):
    """Truncated SDF (metres, float32) of an ellipsoid on an n^3 grid (voxel
    centres at i+0.5), unobserved (beyond +trunc) set to trunc + 1e-5."""
    ax = np.arange(n) + 0.5
    Z, Y, X = np.meshgrid(ax, ax, ax, indexing="ij")
    q = np.sqrt(((X - centre[0]) / scale[0]) ** 2 + ((Y - centre[1]) / scale[1]) ** 2 +
                ((Z - centre[2]) / scale[2]) ** 2)
    d = (q - radius) * voxel
    d = np.where(d > trunc, trunc + 1e-5, d)
    return d.astype(np.float32)


def small_pair(n=24, voxel=0.004, trunc_voxels=5.0, seed=0):
    """A canonical sphere and a moved, stretched live sphere, float32."""
    rng = np.random.default_rng(seed)
    c = np.array([n / 2, n / 2, n / 2]) + rng.uniform(-0.5, 0.5, 3)
    r = n * 0.25
    trunc = voxel * trunc_voxels
    can = sphere_sdf(n, c, r, voxel, trunc)
    live = sphere_sdf(n, c + rng.uniform(-0.8, 0.8, 3), r, voxel, trunc,
                      scale=(1.05, 1.0, 0.97))
    return can, live


def sphere_frames():
    """The 64^3 / 4 mm sphere pair: grid and two float32 depth frames."""
    return synth.sphere_pair()


def integrate_oracle(oracle, grid, frame, params):
    n = grid.dims[::-1]
    phi = np.full(n, params.max_surface + params.epsilon)
    w = np.zeros(n, np.int64)
    return oracle.integrate(phi, w, grid.voxel, grid.origin, params.unknown_clip,
                            frame.astype(np.float64), np.eye(4), synth.K, 0.05, 1.2)


def band_voxels(live, params, psi=None):
    """xyz of the voxels whose own value lies in the band."""
    m = (live <= params.max_surface - params.epsilon) & (live >= -params.unknown_clip)
    z, y, x = np.nonzero(m)
    return np.stack([x, y, z], axis=1)
