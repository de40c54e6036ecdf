"""FUSE_BY_MERGE's running mean against the reference's float64 expression.

SDF::fuse (SDF.cpp:212-236) stores (w1 * d1 + w2 * d2) / (w1 + w2), computed
in float64, as float32.  The GPU decides that float in float-float
arithmetic and falls back to float64 only where the float-float value cannot
tell which float the float64 one rounds to.  Checked bit for bit against
numpy's float64 evaluation of the same expression on 8 M voxels:
* random values and weights (1..1000, some empty on either side);
* crafted ties: d2 the float after d1 with equal weights, so the mean lies
  exactly halfway between two floats (round half to even decides);
* weights from 2^23 up, which the float-float path leaves to float64.
Both entry points that fuse are covered: kf_fuse and kf_warp_fuse (with
psi = 0 the warp is the identity).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_fuse(p1, w1, p2, w2):
    out_p, out_w = p1.copy(), w1.copy()
    m = w2 != 0
    copy = m & (w1 == 0)
    out_p[copy], out_w[copy] = p2[copy], w2[copy]
    mix = m & (w1 != 0)
    a, b = w1[mix].astype(np.float64), w2[mix].astype(np.float64)
    out_p[mix] = ((a * p1[mix].astype(np.float64) + b * p2[mix].astype(np.float64)) / (a + b)).astype(np.float32)
    out_w[mix] = w1[mix] + w2[mix]
    return out_p, out_w


def inputs(n, seed):
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    p1 = rng.uniform(-0.05, 0.05, shape).astype(np.float32)
    p2 = rng.uniform(-0.05, 0.05, shape).astype(np.float32)
    w1 = rng.integers(0, 1000, shape).astype(np.int32)
    w2 = rng.integers(0, 6, shape).astype(np.int32)
    f1, f2, g1, g2 = p1.ravel(), p2.ravel(), w1.ravel(), w2.ravel()
    # ties: the mean of a float and the next float, equal weights
    t = rng.choice(f1.size, f1.size // 16, replace=False)
    f2[t] = np.nextafter(f1[t], np.float32(np.inf))
    g1[t] = g2[t] = rng.integers(1, 50, t.size)
    # large weights (float64 path)
    big = rng.choice(f1.size, f1.size // 64, replace=False)
    g1[big] = rng.integers(1 << 23, 1 << 28, big.size)
    return p1, w1, p2, w2


@pytest.mark.parametrize("entry", ["fuse", "warp_fuse"])
def test_running_mean_bit_exact(gpu, entry):
    capi = gpu
    n = 200
    P = capi.Params.reference(0.005, 5.0)
    p1, w1, p2, w2 = inputs(n, seed=11 if entry == "fuse" else 12)
    dims = (n, n, n)
    can = capi.Grid(dims, 0.005, (0, 0, 0), P.unknown_clip, P)
    live = capi.Grid(dims, 0.005, (0, 0, 0), P.unknown_clip, P)
    can.upload(p1, w1)
    live.upload(p2, w2)
    if entry == "fuse":
        capi.check(capi.load().kf_fuse(can.h, live.h, None))
    else:
        psi = capi.Field(dims, capi.KF_F32)
        capi.warp_fuse(can, live, psi, P)
        psi.close()
    gp, gw = can.download()
    ep, ew = reference_fuse(p1, w1, p2, w2)
    np.testing.assert_array_equal(gw, ew)
    bad = np.flatnonzero(gp.view(np.int32) != ep.view(np.int32))
    assert bad.size == 0, (bad.size, bad[:5], gp.ravel()[bad[:5]], ep.ravel()[bad[:5]])
    can.close()
    live.close()
