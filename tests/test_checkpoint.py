"""Checkpoint and resume of a frame sequence (state files, kf_fusion_save /
kf_fusion_load, kf_state_*), and the reader of the reference's SDF dump.

* A pipeline (KillingFusion::processNextFrame, KillingFusion.cpp:109-175) runs
  6 frames of a 128^3 ellipsoid sequence.  A second pipeline runs the first 3,
  saves its state; a third, fresh pipeline loads it and runs frames 4-6.  Every
  mesh of the resumed frames and the final canonical SDF (values and weights)
  equal the uninterrupted run's bit for bit, with the dense fused solver and
  with the float64 exact solver (float64 psi in the file).
* The state file's header describes the grid; loading into a grid of another
  size, or from a file that is not a state file, is refused.
* kf_grid_load_ref_bin reads the layout of SDF::dumpToBinFile (SDF.cpp:432-446,
  written here with numpy): values as float32, weight 1 wherever the value is
  not the initial MaxSurfaceVoxelDistance + epsilon.
"""
import ctypes as C
import os

import numpy as np
import pytest

from killingfusion_gb300 import synth

pytestmark = pytest.mark.gpu

FRAMES = 6
CHECKPOINT = 3


def pipeline(capi, seq, P, solver):
    g = seq.grid
    return capi.Fusion(g.dims, g.voxel, g.origin, P, max_depth=1.6, iterations=40, solver=solver)


def canonical(capi, fusion, shape):
    c, _, _ = fusion.state()
    phi = np.empty(shape, np.float32)
    w = np.empty(shape, np.int32)
    capi.check(capi.load().kf_grid_download(c, phi.ctypes.data, w.ctypes.data, None))
    return phi, w


@pytest.mark.parametrize("solver", ["fused", "exact"])
def test_resume_equals_uninterrupted(gpu, tmp_path, solver):
    capi = gpu
    seq = synth.EllipsoidSequence(seed=2, frames=30, n=128)
    P = capi.Params.reference(seq.grid.voxel, 5.0)
    shape = seq.grid.dims[::-1]
    frames = [seq.frame(f) for f in range(FRAMES)]
    full = pipeline(capi, seq, P, solver)
    want = [full.process_frame(d) for d in frames]
    want_phi, want_w = canonical(capi, full, shape)
    full.close()

    first = pipeline(capi, seq, P, solver)
    for d in frames[:CHECKPOINT]:
        first.process_frame(d)
    path = str(tmp_path / "state.kfs")
    first.save(path)
    first.close()
    dims = (C.c_int * 3)()
    frame, prec = C.c_int32(-1), C.c_int(-2)
    capi.check(capi.load().kf_state_info(os.fsencode(path), dims, None, None, None, C.byref(frame),
                                         C.byref(prec)))
    assert tuple(dims) == seq.grid.dims and frame.value == CHECKPOINT
    assert prec.value == (capi.KF_F64 if solver == "exact" else capi.KF_F32)

    resumed = pipeline(capi, seq, P, solver)
    resumed.load(path)
    for f in range(CHECKPOINT, FRAMES):
        got = resumed.process_frame(frames[f])
        assert got["frame"] == want[f]["frame"] == f + 1
        for name in ("live", "registered", "canonical"):
            assert got[name].shape == want[f][name].shape and len(got[name]) > 100, (f, name)
            np.testing.assert_array_equal(got[name], want[f][name])
    phi, w = canonical(capi, resumed, shape)
    np.testing.assert_array_equal(w, want_w)
    np.testing.assert_array_equal(phi.view(np.int32), want_phi.view(np.int32))
    resumed.close()


def test_state_file_checks(gpu, tmp_path):
    capi = gpu
    L = capi.load()
    P = capi.Params.reference(0.004, 5.0)
    g = capi.Grid((20, 21, 22), 0.004, (0.0, 0.0, 0.0), P.unknown_clip, P)
    rng = np.random.default_rng(3)
    phi = rng.uniform(-0.02, 0.02, g.shape).astype(np.float32)
    w = rng.integers(0, 9, g.shape).astype(np.int32)
    g.upload(phi, w)
    f = capi.Field(g.dims, capi.KF_F32)
    psi = rng.normal(0, 0.3, g.shape + (3,)).astype(np.float32)
    f.upload(psi)
    path = os.fsencode(str(tmp_path / "s.kfs"))
    capi.check(L.kf_state_save(path, g.h, f.h, 17, None))
    # round trip into fresh handles
    g2 = capi.Grid((20, 21, 22), 0.004, (0.0, 0.0, 0.0), P.unknown_clip, P)
    f2 = capi.Field(g.dims, capi.KF_F32)
    fr = C.c_int32(0)
    capi.check(L.kf_state_load(path, g2.h, f2.h, C.byref(fr), None))
    p2, w2 = g2.download()
    assert fr.value == 17
    np.testing.assert_array_equal(p2, phi)
    np.testing.assert_array_equal(w2, w)
    np.testing.assert_array_equal(f2.download(), psi)
    # other size, other placement, other precision, not a state file
    g3 = capi.Grid((20, 21, 23), 0.004, (0.0, 0.0, 0.0), P.unknown_clip, P)
    assert L.kf_state_load(path, g3.h, None, None, None) == capi.KF_ERR_INVALID
    g4 = capi.Grid((20, 21, 22), 0.004, (0.1, 0.0, 0.0), P.unknown_clip, P)
    assert L.kf_state_load(path, g4.h, None, None, None) == capi.KF_ERR_INVALID
    f64 = capi.Field(g.dims, capi.KF_F64)
    assert L.kf_state_load(path, g2.h, f64.h, None, None) == capi.KF_ERR_INVALID
    bad = tmp_path / "bad.kfs"
    bad.write_bytes(b"not a state file at all" * 10)
    assert L.kf_state_load(os.fsencode(str(bad)), g2.h, None, None, None) == capi.KF_ERR_INVALID
    trunc = tmp_path / "trunc.kfs"
    trunc.write_bytes(open(str(tmp_path / "s.kfs"), "rb").read()[:5000])
    assert L.kf_state_load(os.fsencode(str(trunc)), g2.h, None, None, None) == capi.KF_ERR_INVALID
    assert b"truncated" in L.kf_last_error()
    for h in (g, g2, g3, g4, f, f2, f64):
        h.close()


def test_reference_sdf_dump_reader(gpu, tmp_path):
    capi = gpu
    L = capi.load()
    P = capi.Params.reference(0.004, 5.0)
    dims = (17, 13, 11)
    rng = np.random.default_rng(5)
    vals = rng.uniform(-0.03, 0.5, dims[::-1])
    init = P.max_surface + P.epsilon
    vals[rng.random(vals.shape) < 0.3] = init  # untouched voxels
    path = tmp_path / "sdf.bin"
    with open(path, "wb") as fh:  # SDF::dumpToBinFile's layout
        np.array(dims, "<i4").tofile(fh)
        np.array([0.1, -0.2, 0.3], "<f8").tofile(fh)
        np.array([0.004, 5.0], "<f8").tofile(fh)
        vals.astype("<f8").tofile(fh)
    h = capi._vp()
    trunc = C.c_double(0)
    capi.check(L.kf_grid_load_ref_bin(os.fsencode(str(path)), C.byref(P.c()), P.unknown_clip, C.byref(h),
                                      C.byref(trunc), None))
    g = capi.Grid.__new__(capi.Grid)
    g.h, g.dims, g.shape = h, dims, dims[::-1]
    phi, w = g.download()
    assert trunc.value == 5.0
    np.testing.assert_array_equal(phi, vals.astype(np.float32))
    np.testing.assert_array_equal(w, (vals.astype(np.float32) != np.float32(init)).astype(np.int32))
    n, vs, mn, clip = (C.c_int * 3)(), C.c_double(), (C.c_double * 3)(), C.c_double()
    capi.check(L.kf_grid_info(h, n, C.byref(vs), mn, C.byref(clip)))
    assert tuple(n) == dims and vs.value == 0.004 and tuple(mn) == (0.1, -0.2, 0.3)
    g.close()
    short = tmp_path / "short.bin"
    short.write_bytes(open(path, "rb").read()[:-8])
    h2 = capi._vp()
    assert L.kf_grid_load_ref_bin(os.fsencode(str(short)), C.byref(P.c()), P.unknown_clip, C.byref(h2),
                                  None, None) == capi.KF_ERR_INVALID
