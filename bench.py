#!/usr/bin/env python
"""Benchmark of the KillingFusion registration loop on GB300.

Workload: the 256^3 / 5 mm sequence -- a union of 5 ellipsoids bending about
a seeded hinge, 640x480 float32 depth with 1.5 mm noise -- with 200 psi
iterations per frame, at the reference's compiled-in weights (alpha 0.025,
omega_k 0.04, gamma 0, omega_s 0.1, config.cpp:45-54; `--weights paper` for
alpha 0.1, omega_k 0.5, gamma 0.1, omega_s 0.2).  At the paper weights the
reference's own FP64 iteration amplifies rounding beyond a few tens of
iterations, so psi can be compared with the oracle at 200 iterations only at
the reference's weights.  One step is one frame of the per-frame pipeline of
KillingFusion::processNextFrame (KillingFusion.cpp:123-170): integrate the
live frame, zero psi, 200 fused Jacobi iterations, mesh the live SDF, warp it
by psi and fuse it into the canonical SDF, mesh the registered and the
canonical SDF.

Frames run two deep on four CUDA streams: a frame's reset, integration and
live mesh beside the solve of the frame before, its registered and canonical
meshes beside the solve of the frame after, with events ordering what they share
(the canonical SDF, each slot's live SDF, psi and mesh buffers).

value: voxel-updates/s = 256^3 * 200 * steps / time, every frame's inputs
resident in HBM.  e2e: the same through the C ABI with the depth frame copied
from pinned host memory and the three meshes copied back each step.
psi_err_vs_oracle: one frame's float32 psi against the FP64 oracle's on the
same SDFs, measured in the CPU-baseline leg, which runs that frame in full.

`--impl reference` times the FP64 CPU restatement of the reference (the
oracle) on the host cores: every timed step is one full frame (integrate,
200 Jacobi iterations, update + fuse, three meshes); the untimed warm-up
steps run the frame with 2 iterations.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel-updates/s at 256³ fused vs plain GPU (ψ err≤1e-4 vox); ms/frame; HBM %"
# Compulsory DRAM bytes of one dense Jacobi iteration: every voxel reads psi
# (12) and phi_live (4) for the band test; a voxel outside the band keeps its
# psi, so only the band voxels also read phi_can and write psi (through the
# side buffer and the scatter: 4 + 12 + 12 + 4 + 12 + 4 with the list).
ALGO_BYTES_PER_VOXEL = 16
ALGO_BYTES_PER_BAND_VOXEL = 48
MESH_CAP = 4_000_000       # triangles per mesh buffer


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--iters", type=int, default=None,
                    help="psi iterations per frame (default: 200 ellipsoid, 100 sphere, 300 large)")
    ap.add_argument("--solver", default="fused", choices=["fused", "plain"])
    ap.add_argument("--weights", default="reference", choices=["reference", "paper"],
                    help="reference: the compiled-in alpha/omega_k/gamma/omega_s (config.cpp:45-54); "
                         "paper: the values in the comment at config.cpp:32-41")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-band-frame", action="store_true", help="skip the band-only frame measurement")
    ap.add_argument("--timeline", default=None, choices=["band", "fused"],
                    help="instead of the bench line: per-frame, per-stream step times (CUDA events) of "
                         "--steps frames of the per-frame workload in the two-frame pipeline with this solver")
    ap.add_argument("--log", default=None,
                    help="JSONL log: the configuration, each timed frame's solve time, the per-iteration "
                         "energy, max |dpsi| and band count of the parity frame's solve, the result line")
    ap.add_argument("--workload", default="ellipsoid", choices=["ellipsoid", "sphere", "batch", "large"],
                    help="ellipsoid: 256^3 sequence (the bench line); sphere: the 64^3 two-frame sphere "
                         "pair, 100 iterations; batch: 64 registration problems of 32-160^3, 150 "
                         "iterations; large: 512^3 capsule sequence, 300 iterations")
    args = ap.parse_args()
    if args.iters is None:
        args.iters = {"sphere": 100, "large": 300}.get(args.workload, 200)
    return args


def workload_sequence(args):
    """(sequence, frames in it, max depth, workload name) of the per-frame
    workloads."""
    from killingfusion_gb300 import synth
    if args.workload == "sphere":
        return synth.SpherePairSequence(), 2, 1.2, "sphere-pair-64"
    return (synth.EllipsoidSequence(seed=2, frames=30, n=args.size), 30, 1.6,
            "ellipsoid-sequence-%d" % args.size)


def dist_info():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", rank))
    return rank, world, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per voxel of one fused iteration from the committed ncu
    summary (profiles/fused_iteration_traffic.json), if present."""
    p = os.path.join(ROOT, "profiles", "fused_iteration_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
            time.sleep(0.5)  # the first samples come after the tool has started
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.out.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def mesh_once(capi, L, g, P, buf, cap):
    n = C.c_int64(0)
    capi.check(L.kf_marching_cubes(g.h, C.byref(P.c()), buf, cap, C.byref(n), None))
    return n.value


def fused_solve_launches(n3, iters):
    """Kernel launches of one dense fused solve: a stream pass and a band pass
    per iteration and one final write-back; on grids of at least 512 runs of
    2048 voxels the split schedule adds the run split once and a cold pass
    per iteration after the first."""
    runs = max((n3 // 4 + 511) // 512, 1)
    return 3 * iters + 1 if runs >= 512 else 2 * iters + 1


WEIGHTS_TEXT = {
    "reference": "reference (config.cpp:45-54): alpha 0.025, omega_k 0.04, gamma 0, omega_s 0.1",
    "paper": "paper (config.cpp:32-41): alpha 0.1, omega_k 0.5, gamma 0.1, omega_s 0.2",
}


def bench_params(args, voxel):
    """Solver parameters of the workloads: 5-voxel truncation band, the
    weights chosen by --weights."""
    from killingfusion_gb300 import capi
    if args.weights == "paper":
        return capi.Params.paper(voxel, 5.0)
    return capi.Params.reference(voxel, 5.0)


def bench_config(args):
    """The workload's description, the same on both arms."""
    seq, _, _, name = workload_sequence(args)
    n = seq.grid.dims
    sphere = args.workload == "sphere"
    return {
        "workload": name, "grid": "%dx%dx%d" % tuple(n), "voxel_mm": seq.grid.voxel * 1e3,
        "iterations_per_frame": args.iters, "weights": WEIGHTS_TEXT[args.weights],
        "frames": "frame 0 canonical, then live frames 1..%d in turn" % (seq.frames - 1),
        "step": "one processNextFrame: integrate, zero psi, %d psi iterations, 3 meshes, warp+fuse" % args.iters,
        "l2": ("inputs fit in L2 (16 B x 64^3 = 4.2 MB per iteration)" if sphere else
               "inputs larger than L2 (psi 201 MB + phi_live 67 MB read per iteration)"),
    }


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    from killingfusion_gb300 import capi
    from killingfusion_gb300.pipeline import FramePipeline

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    seq, nseq, max_depth, _ = workload_sequence(args)
    grid = seq.grid
    P = bench_params(args, grid.voxel)
    nframes = 1 + args.warmup + args.steps
    # frame 0 is the canonical frame; the live frames cycle through the rest
    host_frames = [seq.frame(0 if f == 0 else 1 + (f - 1) % (nseq - 1)) for f in range(nframes)]
    dev_frames = [torch.from_numpy(f).to(dev) for f in host_frames]
    pinned = [torch.from_numpy(f).pin_memory() for f in host_frames]

    N3 = int(np.prod(grid.dims))
    # reset, integrate (3 kernels), the solve (fused: stream + band per
    # iteration and one write-back; plain: 7 kernels), warp+fuse (3), 3
    # meshes of 3 kernels each
    launches_per_frame = 1 + 3 + fused_solve_launches(N3, args.iters) + 3 + 3 * 3 if args.solver == "fused" else \
        1 + 3 + 7 * args.iters + 3 + 3 * 3

    # two frames in flight on four streams (killingfusion_gb300.pipeline)
    pipe = FramePipeline(grid.dims, grid.voxel, grid.origin, P, args.iters, args.solver,
                         max_depth=max_depth, mesh_capacity=MESH_CAP, device=local)
    stats = pipe.stats

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()

    # warm-up (also captures the solve graph of each slot)
    pipe.start(dev_frames[0])
    pipe.run([(f, dev_frames[f]) for f in range(1, 1 + args.warmup)])
    barrier()

    clocks = Clocks(local)
    clocks.start()
    t0 = time.perf_counter()
    ev_start, ev_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    solve_events, tri_counts, _ = pipe.run([(f, dev_frames[f]) for f in range(1 + args.warmup, nframes)],
                                           False, ev_start, ev_end)
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    elapsed_ms = ev_start.elapsed_time(ev_end)
    solve_ms = [a.elapsed_time(b) for a, b in solve_events]
    active = stats.active_first

    # end to end through the C ABI with host buffers: the canonical SDF
    # starts again from frame 0 and the warm-up frames are replayed, so the
    # timed frames meet the same canonical SDF (and must give the same meshes)
    pipe.start(pinned[0])
    pipe.run([(f, pinned[f]) for f in range(1, 1 + args.warmup)], True)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    _, tri_e2e, d2h_total = pipe.run([(f, pinned[f]) for f in range(1 + args.warmup, nframes)], True, e0, e1)
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    if tri_e2e != tri_counts:
        raise RuntimeError("end-to-end frames gave other meshes: %s vs %s" % (tri_e2e, tri_counts))
    live, psi, can_e2e = pipe.lives[0], pipe.psis[0], pipe.can

    # plain per-term solver on the same frame (fewer iterations), for the ratio
    plain_it = 10
    live.reset(P)
    live.integrate(dev_frames[-1], min_depth=0.05, max_depth=max_depth)
    psi.zero()
    st_plain = capi.psi_solve(live, can_e2e, psi, P, plain_it, "plain" if args.solver == "fused" else "fused")
    other_vups = N3 * plain_it / (st_plain["device_ms"] / 1e3)

    # band-only solver on the same frame: same psi, visits only the band
    band_ms = []
    for _ in range(3):
        psi.zero()
        stb = capi.psi_solve(live, can_e2e, psi, P, args.iters, "band")
        band_ms.append(stb["device_ms"])
    pipe.close()

    # whole frames with the band-only solver in the same pipeline: the same
    # psi, so the same meshes
    band_frame = None
    if not args.no_band_frame and args.solver == "fused":
        pb = FramePipeline(grid.dims, grid.voxel, grid.origin, P, args.iters, "band",
                           max_depth=max_depth, mesh_capacity=MESH_CAP, device=local)
        pb.start(dev_frames[0])
        pb.run([(f, dev_frames[f]) for f in range(1, 1 + args.warmup)])
        barrier()
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        bsolve, tri_band, _ = pb.run([(f, dev_frames[f]) for f in range(1 + args.warmup, nframes)], False, b0, b1)
        barrier()
        if tri_band != tri_counts:
            raise RuntimeError("band-only frames gave other meshes: %s vs %s" % (tri_band, tri_counts))
        band_frame = {"ms_per_frame": b0.elapsed_time(b1) / args.steps,
                      "solve_ms": statistics.mean(a.elapsed_time(b) for a, b in bsolve)}
        pb.close()

    # one frame for the psi comparison with the oracle (CPU-baseline leg):
    # frame 1 registered onto frame 0 by the dense fused solver
    parity = None
    if world == 1 and not args.no_cpu_baseline:
        gc = capi.Grid(grid.dims, grid.voxel, grid.origin, P.unknown_clip, P)
        gl = capi.Grid(grid.dims, grid.voxel, grid.origin, P.unknown_clip, P)
        gc.integrate(dev_frames[0], min_depth=0.05, max_depth=max_depth)
        gl.integrate(torch.from_numpy(seq.frame(1)).to(dev), min_depth=0.05, max_depth=max_depth)
        fp = capi.Field(grid.dims, capi.KF_F32)
        stp = capi.psi_solve(gl, gc, fp, P, args.iters, args.solver)
        parity = {"live": gl.download()[0], "can": gc.download()[0], "psi": fp.download(), "stats": stp,
                  "history": capi.solve_history(fp) if args.solver != "plain" else None}
        for h in (gc, gl, fp):
            h.close()

    res = {
        "elapsed_ms": elapsed_ms, "wall_s": wall, "solve_ms": solve_ms, "e2e_ms": e2e_ms,
        "d2h_bytes_per_step": d2h_total / args.steps, "tris": tri_counts, "active": active,
        "clocks": clk, "N3": N3, "other_vups": other_vups, "launches": launches_per_frame * args.steps,
        "band_ms": statistics.median(band_ms[1:]), "band_active_last": stb["active_last"],
        "band_frame": band_frame, "parity": parity,
    }
    return res, seq, P


def batch_sizes(count=64, seed=4):
    """Edges of the batched workload: log-uniform in [32, 160]."""
    import numpy as np
    rng = np.random.default_rng(seed)
    return [int(round(float(np.exp(rng.uniform(np.log(32), np.log(160)))))) for _ in range(count)]


def run_batch(args, local):
    """64 independent two-frame registrations (sphere, ellipsoid or torus,
    rigid offset + bend, edges 32-160), 150 band-only iterations each, all in
    one batch; beside it the same problems solved one after another."""
    import numpy as np
    import torch

    from killingfusion_gb300 import capi, synth

    torch.cuda.set_device(local)
    iters = 150
    sizes = batch_sizes()
    probs = []
    for k, n in enumerate(sizes):
        can, live, voxel = synth.shape_problem(1000 + k, n)
        P = bench_params(args, voxel)
        gl = capi.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
        gc = capi.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
        gl.upload(live, (live <= P.max_surface).astype(np.int32))
        gc.upload(can, (can <= P.max_surface).astype(np.int32))
        probs.append((gl, gc, capi.Field((n, n, n), capi.KF_F32), P))
    voxels = sum(n ** 3 for n in sizes)
    batch = capi.Batch(probs, iters)
    shape = batch.autotune()

    def zero_all():
        for _, _, f, _ in probs:
            f.zero()

    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        zero_all()
        batch.run()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    band_total = 0
    for _ in range(args.steps):
        zero_all()
        st = batch.run()
        band_total = sum(x["active_first"] for x in st)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    # the same problems one after another (band-only and dense fused solves)
    seq_ms = {}
    for solver in ("band", "fused"):
        for rep in range(2):
            zero_all()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for gl, gc, f, P in probs:
                capi.psi_solve(gl, gc, f, P, iters, solver)
            b.record(stream)
            torch.cuda.synchronize()
            seq_ms[solver] = a.elapsed_time(b)
    batch.close()
    small = small_batch(capi, synth, torch, iters, lambda v: bench_params(args, v))
    value = voxels * iters / (ms / 1e3)
    return {
        "metric": METRIC, "value": value, "unit": "voxel-updates/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batch-64", "problems": len(sizes), "edges": [min(sizes), max(sizes)],
                   "voxels": voxels, "iterations": iters, "weights": WEIGHTS_TEXT[args.weights],
                   "solver": "batched band-only",
                   "autotuned_shape": "band CTA %d threads, chunks of %d voxels, %d CTAs/SM, %d registers; "
                                      "dense slab %d planes" % (shape["band_threads"], shape["band_chunk"],
                                                                 shape["band_blocks_per_sm"],
                                                                 shape["band_registers"], shape["slab"]),
                   "step": "zero psi of all 64 problems, one kf_batch_run (150 iterations each: a dense "
                           "first pass, then every band pass in one persistent launch)"},
        "band_voxels_first_iteration": band_total,
        "sequential_band_ms": seq_ms["band"], "sequential_fused_ms": seq_ms["fused"],
        "batched_over_sequential_band": seq_ms["band"] / ms,
        "small_problems": small,
        "shape": shape,
        "clocks": clk, "gpu_launches": 2 * args.steps,
    }


def small_batch(capi, synth, torch, iters, params, count=192):
    """Many small problems (edges 16-40), where one launch per problem and
    iteration is latency-bound: batched vs one after another."""
    import numpy as np
    rng = np.random.default_rng(9)
    sizes = [int(v) for v in rng.integers(16, 41, count)]
    probs = []
    for k, n in enumerate(sizes):
        can, live, voxel = synth.shape_problem(5000 + k, n)
        P = params(voxel)
        gl = capi.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
        gc = capi.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
        gl.upload(live, (live <= P.max_surface).astype(np.int32))
        gc.upload(can, (can <= P.max_surface).astype(np.int32))
        probs.append((gl, gc, capi.Field((n, n, n), capi.KF_F32), P))
    batch = capi.Batch(probs, iters)
    shape = batch.autotune()
    stream = torch.cuda.current_stream()

    def timed(fn):
        for _, _, f, _ in probs:
            f.zero()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    def sequential():
        for gl, gc, f, P in probs:
            capi.psi_solve(gl, gc, f, P, iters, "band")

    timed(batch.run)
    tb = min(timed(batch.run) for _ in range(3))
    timed(sequential)
    ts = min(timed(sequential) for _ in range(2))
    batch.close()
    vox = sum(n ** 3 for n in sizes)
    return {"problems": count, "edges": [min(sizes), max(sizes)], "voxels": vox, "iterations": iters,
            "batched_ms": tb, "sequential_band_ms": ts, "batched_over_sequential_band": ts / tb,
            "batched_voxel_updates_per_s": vox * iters / (tb / 1e3), "shape": shape}


def run_large(args, local):
    """512^3 / 2 mm capsule sequence: per frame integrate, zero psi, 300
    dense fused iterations; warp + fuse and the three meshes every 10th
    frame."""
    import numpy as np
    import torch

    from killingfusion_gb300 import capi, synth

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = capi.load()
    iters = 300
    seq = synth.CapsuleSequence(seed=5, frames=100, n=512)
    grid = seq.grid
    P = bench_params(args, grid.voxel)
    steps = max(args.steps, 10)
    nframes = 1 + args.warmup + steps
    dev_frames = [torch.from_numpy(seq.frame(f)).to(dev) for f in range(nframes)]
    can = capi.Grid(grid.dims, grid.voxel, grid.origin, P.unknown_clip, P)
    live = capi.Grid(grid.dims, grid.voxel, grid.origin, P.unknown_clip, P)
    psi = capi.Field(grid.dims, capi.KF_F32)
    can.integrate(dev_frames[0], min_depth=0.05, max_depth=1.6)
    mesh = torch.empty((MESH_CAP, 9), dtype=torch.float32, device=dev)
    N3 = int(np.prod(grid.dims))
    stream = torch.cuda.current_stream(dev)
    stats = capi.SolveStats()

    def frame(f, fuse):
        live.compute_sdf(P, dev_frames[f], min_depth=0.05, max_depth=1.6)
        psi.zero()
        capi.check(L.kf_psi_solve(live.h, can.h, psi.h, C.byref(P.c()), iters, capi.KF_SOLVER_FUSED,
                                  C.byref(stats), None))
        if fuse:
            mesh_once(capi, L, live, P, mesh.data_ptr(), MESH_CAP)
            capi.check(L.kf_warp_fuse(can.h, live.h, psi.h, C.byref(P.c()), None))
            mesh_once(capi, L, live, P, mesh.data_ptr(), MESH_CAP)
            mesh_once(capi, L, can, P, mesh.data_ptr(), MESH_CAP)

    for f in range(1, 1 + args.warmup):
        frame(f, f == args.warmup)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k, f in enumerate(range(1 + args.warmup, nframes)):
        frame(f, (k + 1) % 10 == 0)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / steps
    solve_ms = stats.device_ms
    peak, peak_kind = peaks()
    algo = ALGO_BYTES_PER_VOXEL * N3 + ALGO_BYTES_PER_BAND_VOXEL * stats.active_first
    achieved = algo / (solve_ms / iters / 1e3) / 1e9
    return {
        "metric": METRIC, "value": N3 * iters / (ms / 1e3), "unit": "voxel-updates/s", "n_gpus": 1,
        "steps": steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "capsule-sequence-512", "grid": [512] * 3, "voxel_mm": 2.0,
                   "iterations_per_frame": iters, "weights": WEIGHTS_TEXT[args.weights], "solver": "fused",
                   "step": "one frame: integrate, zero psi, 300 iterations; warp+fuse and 3 meshes "
                           "every 10th frame"},
        "solve_ms_last_frame": solve_ms, "band_voxels": stats.active_first,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "kernel": "fused psi iteration", "peak_source": peak_kind},
        "clocks": clk,
    }


class CpuFrame:
    """One frame of the reference's pipeline on the host cores through the
    FP64 oracle (the reference's arithmetic restated in C, OpenMP over all
    host threads): integrate the live frame, `iters` Jacobi iterations
    (a fresh delta field each iteration, as KillingFusion.cpp:256 allocates),
    mesh the live SDF, warp it by psi, fuse it into the canonical SDF, mesh
    the registered and the canonical SDF.  The canonical SDF is frame 0,
    integrated once when the object is made (untimed)."""

    def __init__(self, seq, P, max_depth):
        import numpy as np

        from oracle.oracle import Oracle, Params as OParams
        from killingfusion_gb300 import synth

        self.np, self.synth = np, synth
        self.O = Oracle()
        self.OP = OParams(**{k: getattr(P, k) for k in OParams.__dataclass_fields__})
        self.seq, self.max_depth = seq, max_depth
        shape = seq.grid.dims[::-1]
        self.base = np.full(shape, self.OP.max_surface + self.OP.epsilon)
        self.w0 = np.zeros(shape, np.int64)
        self.can, self.wc = self._integrate(0)

    def _integrate(self, f):
        g = self.seq.grid
        return self.O.integrate(self.base, self.w0, g.voxel, g.origin, self.OP.unknown_clip,
                                self.seq.frame(f).astype(self.np.float64), self.np.eye(4), self.synth.K,
                                0.05, self.max_depth)

    def run(self, f, iters, solve_inputs=None):
        """Frame f; returns (seconds per stage, psi).  solve_inputs: (live,
        canonical) SDFs to solve on instead of the oracle's own (the GPU's
        float32 SDFs, for the psi comparison); the work is the same."""
        np = self.np
        t = {}
        a = time.perf_counter()
        live, wl = self._integrate(f)
        t["integrate"] = time.perf_counter() - a
        sl, sc = solve_inputs if solve_inputs is not None else (live, self.can)
        a = time.perf_counter()
        st, psi = self.O.solve(sl, sc, np.zeros(sl.shape + (3,)), iters, self.OP)
        t["solve"] = time.perf_counter() - a
        a = time.perf_counter()
        self.O.mesh(live, self.OP)
        uphi, uw = self.O.update(live, wl, psi, self.OP)
        fphi, _ = self.O.fuse(self.can, self.wc, uphi, uw)
        self.O.mesh(uphi, self.OP)
        self.O.mesh(fphi, self.OP)
        t["fuse_mesh"] = time.perf_counter() - a
        return t, psi


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def main():
    args = parse()
    rank, world, local = dist_info()
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")

    if args.impl == "reference" and rank != 0:
        return
    if args.timeline:
        if rank == 0:
            print(json.dumps(run_timeline(args, local)))
        return
    if args.workload not in ("ellipsoid", "sphere"):
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the CPU port is timed on the "
                                  "per-frame workloads (ellipsoid, sphere) only"}))
            return
        line = run_batch(args, local) if args.workload == "batch" else run_large(args, local)
        if rank == 0:
            print(json.dumps(line))
        return
    run_main(args, rank, world, local)


def run_timeline(args, local):
    """Each frame's steps on the pipeline's streams (killingfusion_gb300.pipeline),
    in microseconds from CUDA events: when the frame's solve started, how long
    each step took, and the time between two frames' ends of warp + fuse."""
    import torch

    from killingfusion_gb300.pipeline import FramePipeline

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    seq, nseq, max_depth, name = workload_sequence(args)
    grid = seq.grid
    P = bench_params(args, grid.voxel)
    nframes = 1 + args.warmup + args.steps
    frames = [torch.from_numpy(seq.frame(0 if f == 0 else 1 + (f - 1) % (nseq - 1))).to(dev) for f in range(nframes)]
    pipe = FramePipeline(grid.dims, grid.voxel, grid.origin, P, args.iters, args.timeline, max_depth=max_depth,
                         mesh_capacity=MESH_CAP, device=local)
    pipe.start(frames[0])
    pipe.run([(f, frames[f]) for f in range(1, 1 + args.warmup)])
    torch.cuda.synchronize(dev)
    t0 = torch.cuda.Event(enable_timing=True)
    t0.record(pipe.s_main)
    for s in (pipe.s_in, pipe.s_out):
        s.wait_event(t0)
    pipe.marks = []
    pipe.run([(f, frames[f]) for f in range(1 + args.warmup, nframes)])
    torch.cuda.synchronize(dev)
    steps = [("integrate", "in_start", "integrated"), ("zero_psi", "integrated", "zeroed"),
             ("live_mesh", "zeroed", "live_meshed"), ("solve", "solve_start", "solved"),
             ("wait_before_fuse", "solved", "fuse_start"), ("warp_fuse", "fuse_start", "fused"),
             ("registered_mesh", "out_start", "registered_meshed"),
             ("canonical_mesh", "registered_meshed", "canonical_meshed")]
    out, prev = [], None
    for f, m in pipe.marks:
        t = {k: t0.elapsed_time(e) * 1e3 for k, e in m.items()}
        row = {"frame": f, "solve_start_us": round(t["solve_start"], 1)}
        row.update({k + "_us": round(t[b] - t[a], 1) for k, a, b in steps})
        if prev is not None:
            row["frame_us"] = round(t["fused"] - prev, 1)
        prev = t["fused"]
        out.append(row)
    pipe.close()
    per = [r["frame_us"] for r in out if "frame_us" in r]
    return {"timeline": args.timeline, "workload": name, "iterations_per_frame": args.iters,
            "mean_frame_us": round(sum(per) / len(per), 1) if per else None, "frames": out}


def max_over_ranks(values, device="cuda"):
    """Element-wise maximum of per-rank times over all ranks (the slowest
    replica sets the whole job's time)."""
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def run_reference(args):
    """The reference arm: the FP64 CPU restatement of the reference on all
    host threads, every timed step one full frame of the workload."""
    import numpy as np

    seq, nseq, max_depth, name = workload_sequence(args)
    P = bench_params(args, seq.grid.voxel)
    N3 = int(np.prod(seq.grid.dims))
    cores = cpu_threads()
    cf = CpuFrame(seq, P, max_depth)
    live_frame = lambda k: 1 + k % (nseq - 1)  # noqa: E731
    warm_iters = min(2, args.iters)
    for k in range(args.warmup):
        cf.run(live_frame(k), warm_iters)
    per = []
    for k in range(args.warmup, args.warmup + args.steps):
        t, _ = cf.run(live_frame(k), args.iters)
        per.append(sum(t.values()))
    total_s = sum(per)
    value = N3 * args.iters * args.steps / total_s
    sample = ("%d full frames of the %s workload (integrate, %d Jacobi iterations, update+fuse, 3 meshes), "
              "each timed in full; FP64 oracle port on %d threads; the %d untimed warm-up frames ran %d "
              "iterations" % (args.steps, name, args.iters, cores, args.warmup, warm_iters))
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "voxel-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_s / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": bench_config(args),
        "cpu_baseline": {"value": value, "unit": "voxel-updates/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "voxel-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "frame_seconds": [round(v, 3) for v in per],
    }


def run_main(args, rank, world, local):
    import numpy as np

    if args.impl == "reference":
        print(json.dumps(run_reference(args)))
        return

    res, seq, P = run_ours(args, rank, world, local)
    el = res["elapsed_ms"]
    e2e_ms = res["e2e_ms"]
    if world > 1:
        el, e2e_ms = max_over_ranks([el, e2e_ms], "cuda")
    if rank != 0:
        return
    N3 = res["N3"]
    updates = N3 * args.iters * args.steps * world
    value = updates / (el / 1e3)
    e2e_value = updates / (e2e_ms / 1e3)
    solve_ms = statistics.mean(res["solve_ms"])
    iter_ms = solve_ms / args.iters
    peak, peak_kind = peaks()
    algo_bytes = ALGO_BYTES_PER_VOXEL * N3 + ALGO_BYTES_PER_BAND_VOXEL * res["active"]
    achieved = algo_bytes / (iter_ms / 1e3) / 1e9
    prof = profile_traffic()
    traffic = None
    if prof and prof.get("dram_bytes_per_voxel"):
        traffic = prof["dram_bytes_per_voxel"] * N3
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "voxel-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": el / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": bench_config(args),
        "solver": args.solver,
        "parallelism": "replicas" if world > 1 else "1 GPU",
        "e2e": {"value": e2e_value, "unit": "voxel-updates/s",
                "h2d_bytes_per_step": 640 * 480 * 4, "d2h_bytes_per_step": res["d2h_bytes_per_step"]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": ("fused psi iteration: k_fused_stream_runs over the hot and the cold runs "
                                "+ k_fused_band, the cold runs streamed beside the band pass"
                                if max((N3 // 4 + 511) // 512, 1) >= 512 else
                                "fused psi iteration (k_fused_stream + k_fused_band)"),
                     "algorithmic_bytes_per_iteration": algo_bytes,
                     "algorithmic_bytes_per_voxel": ALGO_BYTES_PER_VOXEL,
                     "algorithmic_bytes_per_band_voxel": ALGO_BYTES_PER_BAND_VOXEL, "peak_source": peak_kind},
        "clocks": res["clocks"],
        "gpu_launches": res["launches"],
        "solve_ms_per_frame": solve_ms,
        "solve_voxel_updates_per_s": N3 * args.iters / (solve_ms / 1e3),
        "plain_voxel_updates_per_s" if args.solver == "fused" else "fused_voxel_updates_per_s": res["other_vups"],
        "band_voxels": res["active"],
        "triangles_last_frame": res["tris"][-1],
    }
    if args.workload == "sphere":
        # 64^3: 4.2 MB of psi and phi per iteration stay in the 129 MB L2
        line["roofline"] = None
        line["roofline_note"] = "L2-resident workload: the HBM roofline applies to the 256^3 bench line"
    if args.solver == "fused":
        line["fused_over_plain"] = line["solve_voxel_updates_per_s"] / res["other_vups"]
    band = {
        "solve_ms": res["band_ms"],
        "dense_equivalent_voxel_updates_per_s": N3 * args.iters / (res["band_ms"] / 1e3),
        "band_voxels_last_iteration": res["band_active_last"],
        "note": "KF_SOLVER_BAND: identical psi; after the first dense pass it visits only the band, "
                "which can only shrink (a voxel outside the band keeps psi)",
    }
    if res["band_frame"]:
        band["ms_per_frame"] = res["band_frame"]["ms_per_frame"]
        band["solve_ms_in_frame"] = res["band_frame"]["solve_ms"]
        band["frame_note"] = ("whole frames measured in the same two-frame pipeline with the band-only "
                              "solver (same meshes as the dense frames)")
    line["band_solver"] = band
    if world == 1 and not args.no_cpu_baseline:
        import numpy as np
        par = res["parity"]
        cf = CpuFrame(seq, P, workload_sequence(args)[2])
        t, opsi = cf.run(1, args.iters, (par["live"].astype(np.float64), par["can"].astype(np.float64)))
        frame_s = sum(t.values())
        err = np.abs(par["psi"].astype(np.float64) - opsi)
        line["cpu_baseline"] = {
            "value": N3 * args.iters / frame_s, "unit": "voxel-updates/s", "cores": cpu_threads(),
            "kind": "port", "ms_per_frame": frame_s * 1e3,
            "stage_s": {k: round(v, 3) for k, v in t.items()},
            "sample": ("one full frame of the %s workload (frame 1 onto frame 0: integrate, %d Jacobi "
                       "iterations, update+fuse, 3 meshes); FP64 oracle port on %d threads"
                       % (workload_sequence(args)[3], args.iters, cpu_threads())),
        }
        line["psi_err_vs_oracle"] = {
            "max_voxel": float(err.max()), "rms_voxel": float(np.sqrt((err ** 2).mean())),
            "voxels_above_1e-4": int((err > 1e-4).sum()), "max_abs_psi_voxel": float(np.abs(opsi).max()),
            "iterations": args.iters, "weights": args.weights, "solver": args.solver,
            "frame": "frame 1 registered onto frame 0, float32 psi of the GPU against the FP64 oracle "
                     "on the same float32 SDFs, every voxel",
        }
    if args.log:
        write_log(args.log, line, res)
    print(json.dumps(line))


def write_log(path, line, res):
    """JSONL: one record per line (kind = config, frame, iteration, result)."""
    with open(path, "w") as f:
        f.write(json.dumps({"kind": "config", "config": line["config"], "solver": line.get("solver"),
                            "metric": line["metric"]}) + "\n")
        for k, ms in enumerate(res["solve_ms"]):
            f.write(json.dumps({"kind": "frame", "frame": k, "solve_ms": ms}) + "\n")
        par = res.get("parity")
        if par and par.get("history"):
            h = par["history"]
            for k in range(len(h["energy"])):
                f.write(json.dumps({"kind": "iteration", "frame": "parity", "iteration": k,
                                    "energy": float(h["energy"][k]), "max_delta": float(h["max_delta"][k]),
                                    "band_voxels": int(h["active"][k])}) + "\n")
        f.write(json.dumps({"kind": "result", **line}) + "\n")


if __name__ == "__main__":
    main()
