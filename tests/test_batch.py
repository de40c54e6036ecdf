"""Batched solves (kf_batch_*): every problem's psi, statistics and
convergence equal what kf_psi_solve(KF_SOLVER_BAND) gives it alone, bit for
bit; the autotuner leaves psi alone; a diverging problem does not disturb
the others."""
import numpy as np
import pytest

from killingfusion_gb300 import synth

pytestmark = pytest.mark.gpu

SIZES = [32, 47, 64, 40, 81, 33]


def make_problem(gpu, seed, n, early_exit=False, threshold=1e-6):
    can, live, voxel = synth.shape_problem(seed, n)
    P = gpu.Params.paper(voxel).with_(early_exit=early_exit, threshold=threshold)
    gl = gpu.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
    gc = gpu.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
    gl.upload(live, (live <= P.max_surface).astype(np.int32))
    gc.upload(can, (can <= P.max_surface).astype(np.int32))
    f = gpu.Field((n, n, n), gpu.KF_F32)
    return gl, gc, f, P


def single(gpu, gl, gc, P, iters, psi0=None):
    f = gpu.Field(gl.dims, gpu.KF_F32)
    if psi0 is not None:
        f.upload(psi0)
    st = gpu.psi_solve(gl, gc, f, P, iters, "band")
    return f.download(), st


STAT_KEYS = ("iterations_run", "converged", "diverged", "active_first", "active_last", "max_delta_last")


@pytest.mark.parametrize("iters", [1, 2, 37])
def test_batch_equals_single_band_solves(gpu, iters):
    probs = [make_problem(gpu, 100 + k, n) for k, n in enumerate(SIZES)]
    b = gpu.Batch(probs, iters)
    st = b.run()
    for (gl, gc, f, P), s in zip(probs, st):
        want, ws = single(gpu, gl, gc, P, iters)
        np.testing.assert_array_equal(f.download(), want)
        for k in STAT_KEYS:
            assert s[k] == ws[k], k
        assert s["active_first"] > 0
    # a second run continues from the solved psi, as a second solve would
    st2 = b.run()
    for (gl, gc, f, P), s in zip(probs, st2):
        want, _ = single(gpu, gl, gc, P, iters)
        want2, ws2 = single(gpu, gl, gc, P, iters, psi0=want)
        np.testing.assert_array_equal(f.download(), want2)
        assert s["iterations_run"] == ws2["iterations_run"]
    b.close()


def test_batch_per_problem_convergence(gpu):
    """Problems stop at different iterations under early_exit; each matches
    its own early-exit solve."""
    probs = [make_problem(gpu, 200 + k, n, early_exit=True, threshold=t)
             for k, (n, t) in enumerate([(32, 2e-2), (48, 1e-3), (40, 5e-3), (36, 1e-9)])]
    iters = 60
    b = gpu.Batch(probs, iters)
    st = b.run()
    runs = []
    for (gl, gc, f, P), s in zip(probs, st):
        want, ws = single(gpu, gl, gc, P, iters)
        np.testing.assert_array_equal(f.download(), want)
        for k in STAT_KEYS:
            assert s[k] == ws[k], k
        runs.append(s["iterations_run"])
    assert len(set(runs)) > 1, runs
    assert any(s["converged"] for s in st)
    b.close()


def test_autotune_keeps_psi(gpu):
    probs = [make_problem(gpu, 300 + k, n) for k, n in enumerate([48, 56, 32])]
    rng = np.random.default_rng(1)
    psi0 = []
    for gl, gc, f, P in probs:
        p = (rng.normal(0, 0.1, gl.shape + (3,))).astype(np.float32)
        f.upload(p)
        psi0.append(p)
    b = gpu.Batch(probs, 20)
    sh = b.autotune()
    band = (sh["band_threads"], sh["band_chunk"], sh["band_blocks_per_sm"], sh["band_registers"])
    assert band in gpu.BATCH_BAND_SHAPES and sh["slab"] in gpu.BATCH_SLABS
    assert sh["band_ms"] > 0 and sh["stream_ms"] > 0
    for (gl, gc, f, P), p in zip(probs, psi0):
        np.testing.assert_array_equal(f.download(), p)
    b.run()
    for (gl, gc, f, P), p in zip(probs, psi0):
        want, _ = single(gpu, gl, gc, P, 20, psi0=p)
        np.testing.assert_array_equal(f.download(), want)
    b.close()


def test_diverging_problem_is_isolated(gpu):
    probs = [make_problem(gpu, 400 + k, n) for k, n in enumerate([40, 36, 44])]
    gl, gc, f, P = probs[1]
    live, _ = gl.download()
    z, y, x = np.argwhere(np.abs(live) < 0.5 * P.unknown_clip)[len(live) // 3]
    bad = np.zeros(gl.shape + (3,), np.float32)
    bad[z, y, x, 0] = np.nan
    f.upload(bad)
    b = gpu.Batch(probs, 10)
    st = b.run(raise_on_divergence=False)
    assert st[1]["diverged"] == 1
    assert st[0]["diverged"] == 0 and st[2]["diverged"] == 0
    for k in (0, 2):
        gl, gc, f, P = probs[k]
        want, _ = single(gpu, gl, gc, P, 10)
        np.testing.assert_array_equal(f.download(), want)
    with pytest.raises(gpu.DivergedError):
        b.run()
    b.close()


def test_batch_argument_checks(gpu):
    gl, gc, f, P = make_problem(gpu, 500, 32)
    with pytest.raises(gpu.KFError):
        gpu.Batch([(gl, gc, f, P), (gl, gc, f, P)], 5)  # the same field twice
    f64 = gpu.Field(gl.dims, gpu.KF_F64)
    with pytest.raises(gpu.KFError):
        gpu.Batch([(gl, gc, f64, P)], 5)
    with pytest.raises(gpu.KFError):
        gpu.Batch([(gl, gc, f, P)], 0)


def test_every_launch_shape_gives_the_same_psi(gpu):
    """Each band-pass shape (CTA size, chunk size, resident CTAs) and slab
    depth the autotuner may choose gives every problem the bits of its own
    band-only solve."""
    probs = [make_problem(gpu, 500 + k, n) for k, n in enumerate([37, 52, 30, 61])]
    iters = 9
    want = [single(gpu, gl, gc, P, iters) for gl, gc, _, P in probs]
    b = gpu.Batch(probs, iters)
    for k, band in enumerate(gpu.BATCH_BAND_SHAPES):
        for slab in gpu.BATCH_SLABS if k == 0 else (gpu.BATCH_SLABS[k % 3],):
            for _, _, f, _ in probs:
                f.zero()
            b.set_shape(band, slab)
            st = b.run()
            for (_, _, f, _), (w, ws), s in zip(probs, want, st):
                np.testing.assert_array_equal(f.download(), w)
                for key in STAT_KEYS:
                    assert s[key] == ws[key], (band, slab, key)
    with pytest.raises(gpu.KFError):
        b.set_shape((256, 768, 2, 128), 8)
    b.close()


def test_batch_timeout_status(gpu):
    """A zero wait limit makes the persistent batch launch give up at its first
    barrier: KF_ERR_TIMEOUT, and the next run with the default limit is right."""
    probs = [make_problem(gpu, 600 + k, n) for k, n in enumerate([40, 33])]
    want = [single(gpu, gl, gc, P, 12) for gl, gc, _, P in probs]
    b = gpu.Batch(probs, 12)
    prev = gpu.set_wait_limit(0.0)
    try:
        with pytest.raises(gpu.KFError) as e:
            b.run()
        assert e.value.status == gpu.KF_ERR_TIMEOUT
    finally:
        gpu.set_wait_limit(prev)
    for _, _, f, _ in probs:
        f.zero()
    b.run()
    for (_, _, f, _), (w, _) in zip(probs, want):
        np.testing.assert_array_equal(f.download(), w)
    b.close()
