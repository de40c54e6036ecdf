"""The two-frames-in-flight pipeline (killingfusion_gb300.pipeline, the one
bench.py times) against kf_fusion_process_frame, which runs
KillingFusion::processNextFrame (KillingFusion.cpp:109-175) one frame at a
time on one stream: every frame's three meshes and the final canonical SDF
must be equal bit for bit, from device and from host depth."""
import numpy as np
import pytest

from killingfusion_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("source", ["device", "host"])
def test_two_frames_in_flight_equal_one_at_a_time(gpu, source):
    import torch
    from killingfusion_gb300.pipeline import FramePipeline

    seq = synth.EllipsoidSequence(seed=2, frames=30, n=64)
    g = seq.grid
    P = gpu.Params.paper(g.voxel)
    frames = [seq.frame(f).astype(np.float32) for f in range(7)]
    iters = 30

    ref = gpu.Fusion(g.dims, g.voxel, g.origin, P, max_depth=1.6, iterations=iters, solver="fused")
    ref.process_frame(frames[0])
    want = []
    for f in range(1, len(frames)):
        r = ref.process_frame(frames[f])
        want.append((r["live"], r["registered"], r["canonical"]))
    hc, _, _ = ref.state()
    L = gpu.load()
    shape = g.dims[::-1]
    cphi, cw = np.empty(shape, np.float32), np.empty(shape, np.int32)
    gpu.check(L.kf_grid_download(hc, cphi.ctypes.data, cw.ctypes.data, None))
    ref.close()

    if source == "device":
        depth = [torch.from_numpy(d).cuda() for d in frames]
    else:
        depth = [torch.from_numpy(d).pin_memory() for d in frames]
    pipe = FramePipeline(g.dims, g.voxel, g.origin, P, iters, "fused", max_depth=1.6, mesh_capacity=200_000)
    got = {}
    pipe.start(depth[0])
    _, tris, _ = pipe.run([(f, depth[f]) for f in range(1, len(frames))], copy=True,
                          on_frame=lambda f, ms: got.__setitem__(f, ms))
    torch.cuda.synchronize()
    assert sorted(got) == list(range(1, len(frames)))
    for f in range(1, len(frames)):
        for j in range(3):
            np.testing.assert_array_equal(got[f][j], want[f - 1][j])
        assert tris[f - 1] == tuple(len(m) for m in want[f - 1])
    assert min(len(m) for m in want[-1]) > 100
    phi, w = pipe.can.download()
    np.testing.assert_array_equal(w, cw)
    np.testing.assert_array_equal(phi, cphi)
    pipe.close()
