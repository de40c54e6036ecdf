"""KillingFusion::processNextFrame (KillingFusion.cpp:123-170) over a depth
sequence with two frames in flight, through the C ABI's non-waiting calls.

Frame f uses slot f % 2: its own live SDF, psi field (each with its own
captured solve graph), device mesh buffers and triangle counts.  Four CUDA
streams:

* ``s_in``: the frame's reset, integration, psi zeroing and live mesh (the
  mesh of the SDF as integrated, which the solve only reads), beside the
  solve of the frame before;
* ``s_main``: the solve and warp + fuse, the canonical SDF's chain;
* ``s_out``: the registered and canonical meshes, beside the next solve;
* ``s_copy``: host copies of a finished frame's meshes.

Events order what the streams share: a slot's live SDF and psi are reused
only after that slot's meshes of two frames back, warp + fuse waits for the
canonical mesh of the frame before, and a slot's mesh buffers are rewritten
only after their host copies.  Each frame gives the meshes, SDFs and psi of
the one-frame-at-a-time pipeline (``kf_fusion_process_frame``) bit for bit.
"""
import ctypes as C

import numpy as np

from . import capi, synth


class FramePipeline:
    """Canonical SDF plus two slots; ``start`` makes the canonical SDF from a
    first frame, ``run`` registers and fuses frames in order."""

    def __init__(self, dims, voxel_size, origin, params: "capi.Params", iterations: int,
                 solver: str = "fused", K=None, min_depth: float = 0.05, max_depth: float = 1.2,
                 mesh_capacity: int = 4_000_000, device=None):
        import torch

        self.torch = torch
        self.dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.L = capi.load()
        self.P = params
        self.Pc = params.c()
        self.iterations = int(iterations)
        self.solver = capi.SOLVERS[solver]
        self.min_depth, self.max_depth = float(min_depth), float(max_depth)
        self.cap = int(mesh_capacity)
        self.eye = capi._d(np.eye(4).ravel())
        self.K = capi._d((synth.K if K is None else np.asarray(K, dtype=np.float64)).ravel())
        g = lambda: capi.Grid(dims, voxel_size, origin, params.unknown_clip, params)  # noqa: E731
        self.can = g()
        self.lives = [g(), g()]
        prec = capi.KF_F64 if solver == "exact" else capi.KF_F32
        self.psis = [capi.Field(dims, prec), capi.Field(dims, prec)]
        f32 = torch.float32
        self.meshes = [[torch.empty((self.cap, 9), dtype=f32, device=self.dev) for _ in range(3)]
                       for _ in range(2)]
        self.host_mesh = [torch.empty((self.cap, 9), dtype=f32).pin_memory() for _ in range(3)]
        self.counts = torch.zeros((2, 3), dtype=torch.int64).pin_memory()  # written by the device
        self.s_in, self.s_main, self.s_out, self.s_copy = (torch.cuda.Stream(self.dev) for _ in range(4))
        ev = lambda: [torch.cuda.Event(), torch.cuda.Event()]  # noqa: E731
        self.ev_integ, self.ev_fused, self.ev_meshed, self.ev_copied = ev(), ev(), ev(), ev()
        self.stats = capi.SolveStats()
        # a list to record, per queued frame, timing events between its steps
        # on each stream ((frame, {step: event}) pairs; see queue)
        self.marks = None

    def _compute_sdf(self, grid, depth, stream):
        """KillingFusion::computeSDF: the grid reset and the frame integrated
        in one pass."""
        capi.check(self.L.kf_compute_sdf(grid.h, C.byref(self.Pc), depth.data_ptr(), depth.shape[1],
                                         depth.shape[0], self.eye, self.K, self.min_depth, self.max_depth,
                                         stream.cuda_stream))

    def start(self, depth):
        """The first frame becomes the canonical SDF (KillingFusion.cpp:115-121).
        depth: a float32 [h, w] CUDA tensor or pinned host tensor."""
        self.torch.cuda.synchronize(self.dev)
        self._compute_sdf(self.can, depth, self.s_main)
        self.s_main.synchronize()

    def queue(self, f: int, depth):
        """Queue frame f on the four streams without waiting; returns the
        solve's (start, end) timing events."""
        torch, L, Pc = self.torch, self.L, self.Pc
        k = f % 2
        lv, ps, ms = self.lives[k], self.psis[k], self.meshes[k]
        cptr = self.counts.data_ptr() + 24 * k
        s_in, s_main, s_out = self.s_in, self.s_main, self.s_out
        marks = {}

        def mark(name, stream):
            if self.marks is not None:
                marks[name] = torch.cuda.Event(enable_timing=True)
                marks[name].record(stream)

        s_in.wait_event(self.ev_meshed[k])
        mark("in_start", s_in)
        self._compute_sdf(lv, depth, s_in)
        mark("integrated", s_in)
        ps.zero(stream=s_in)
        mark("zeroed", s_in)
        s_in.wait_event(self.ev_copied[k])
        capi.check(L.kf_marching_cubes_async(lv.h, C.byref(Pc), ms[0].data_ptr(), self.cap, cptr,
                                             s_in.cuda_stream))
        self.ev_integ[k].record(s_in)
        mark("live_meshed", s_in)
        s_main.wait_event(self.ev_integ[k])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s_main)
        capi.check(L.kf_psi_solve_async(lv.h, self.can.h, ps.h, C.byref(Pc), self.iterations, self.solver,
                                        s_main.cuda_stream))
        e1.record(s_main)
        s_main.wait_event(self.ev_meshed[1 - k])  # the canonical mesh of frame f - 1
        mark("fuse_start", s_main)
        capi.check(L.kf_warp_fuse(self.can.h, lv.h, ps.h, C.byref(Pc), s_main.cuda_stream))
        self.ev_fused[k].record(s_main)
        mark("fused", s_main)
        s_out.wait_event(self.ev_fused[k])
        s_out.wait_event(self.ev_copied[k])
        mark("out_start", s_out)
        capi.check(L.kf_marching_cubes_async(lv.h, C.byref(Pc), ms[1].data_ptr(), self.cap, cptr + 8,
                                             s_out.cuda_stream))
        mark("registered_meshed", s_out)
        capi.check(L.kf_marching_cubes_async(self.can.h, C.byref(Pc), ms[2].data_ptr(), self.cap, cptr + 16,
                                             s_out.cuda_stream))
        self.ev_meshed[k].record(s_out)
        mark("canonical_meshed", s_out)
        if self.marks is not None:
            marks["solve_start"], marks["solved"] = e0, e1
            self.marks.append((f, marks))
        return e0, e1

    def finish(self, f: int, copy: bool = False, wait_copy: bool = False):
        """Wait for frame f: raises on a diverged solve or a mesh above the
        capacity; returns (triangle counts, bytes copied, meshes).  copy
        queues the host copies of its meshes on s_copy; wait_copy also waits
        for them and returns them as float32 [T, 3, 3] arrays."""
        k = f % 2
        capi.check(self.L.kf_psi_solve_wait(self.psis[k].h, C.byref(self.stats)))
        self.ev_meshed[k].synchronize()
        n = [int(v) for v in self.counts[k].tolist()]
        if max(n) > self.cap:
            raise capi.KFError(capi.KF_ERR_CAPACITY, "mesh of %d triangles above the buffers' %d"
                               % (max(n), self.cap))
        d2h, out = 0, None
        if copy or wait_copy:
            with self.torch.cuda.stream(self.s_copy):
                for j in range(3):
                    self.host_mesh[j][:n[j]].copy_(self.meshes[k][j][:n[j]], non_blocking=True)
                    d2h += n[j] * 36
            self.ev_copied[k].record(self.s_copy)
            if wait_copy:
                self.ev_copied[k].synchronize()
                out = [self.host_mesh[j][:n[j]].numpy().reshape(-1, 3, 3).copy() for j in range(3)]
        return tuple(n), d2h, out

    def run(self, frames, copy: bool = False, ev_start=None, ev_end=None, on_frame=None):
        """frames: (index, depth) pairs in order, two in flight.  Returns the
        solve event pairs, the triangle counts and the bytes copied to the
        host; on_frame(index, meshes) receives each frame's host meshes (and
        makes the copies wait).  ev_start / ev_end bracket all the work."""
        torch = self.torch
        if ev_start is not None:
            ev_start.record(self.s_main)
            for s in (self.s_in, self.s_out, self.s_copy):
                s.wait_event(ev_start)
        solve_ev, tris, d2h = [], [], 0

        def done(f):
            nonlocal d2h
            n, b, ms = self.finish(f, copy, wait_copy=on_frame is not None)
            tris.append(n)
            d2h += b
            if on_frame is not None:
                on_frame(f, ms)

        for j, (f, depth) in enumerate(frames):
            solve_ev.append(self.queue(f, depth))
            if j > 0:
                done(frames[j - 1][0])
        done(frames[-1][0])
        if ev_end is not None:
            for s in (self.s_in, self.s_out, self.s_copy):
                e = torch.cuda.Event()
                e.record(s)
                self.s_main.wait_event(e)
            ev_end.record(self.s_main)
        return solve_ev, tris, d2h

    def close(self):
        for h in [self.can] + self.lives + self.psis:
            h.close()
