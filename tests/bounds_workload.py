"""Small-grid workloads for the bounds-check build (not collected by pytest:
tests/test_bounds_check.py runs this module in a process of its own with
KF_LIBRARY=bounds_check, so that capi loads libkillingfusion_bc.so).

Every hot-path kernel runs on 8^3-32^3 grids (and ragged ones): integration,
the dense fused, band-only (persistent), per-voxel, float64 exact and
trust-region solves, a batch, warp + fuse, and marching cubes (listed and
allocation-free).  The results are checked against each other and against
the oracle where the bits must agree, and the bounds record is printed as
JSON.  With --limit N every bound is lowered to N first, so the checks fire
while every access stays inside its buffer.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

from helpers import small_pair  # noqa: E402
from killingfusion_gb300 import capi, synth  # noqa: E402


def grids(P, dims, seed):
    n = max(dims)
    can, live = small_pair(n, P.voxel_size, 5.0, seed=seed)
    can, live = can[:dims[2], :dims[1], :dims[0]], live[:dims[2], :dims[1], :dims[0]]
    gl = capi.Grid(dims, P.voxel_size, (0, 0, 0), P.unknown_clip, P)
    gc = capi.Grid(dims, P.voxel_size, (0, 0, 0), P.unknown_clip, P)
    gl.upload(np.ascontiguousarray(live), (live <= P.max_surface).astype(np.int32))
    gc.upload(np.ascontiguousarray(can), (can <= P.max_surface).astype(np.int32))
    return gl, gc


def solve(gl, gc, P, iters, solver, prec=capi.KF_F32):
    f = capi.Field(gl.dims, prec)
    st = capi.psi_solve(gl, gc, f, P, iters, solver)
    out = f.download()
    f.close()
    return out, st


def run(check):
    P = capi.Params.paper(0.004)
    checked = 0
    for k, dims in enumerate([(8, 8, 8), (16, 16, 16), (32, 32, 32), (19, 23, 17), (32, 9, 24)]):
        gl, gc = grids(P, dims, 70 + k)
        a, _ = solve(gl, gc, P, 6, "fused")
        b, _ = solve(gl, gc, P, 6, "band")
        check(np.array_equal(a, b), "band == fused %s" % (dims,))
        solve(gl, gc, P, 4, "pervoxel")
        solve(gl, gc, P, 3, "exact", capi.KF_F64)
        PT = P.with_(use_levelset=False, use_killing=False, use_trust=True)
        t1, _ = solve(gl, gc, PT, 4, "fused")
        t2, _ = solve(gl, gc, PT, 4, "band")
        check(np.array_equal(t1, t2), "trust band == fused %s" % (dims,))
        f = capi.Field(gl.dims, capi.KF_F32)
        f.upload(a)
        capi.warp_fuse(gc, gl, f, P)
        f.close()
        tris = capi.marching_cubes(gc, P)
        checked += 1 + len(tris) * 0
        gl.close()
        gc.close()
    # a batch of ragged problems
    probs = []
    for k, dims in enumerate([(17, 12, 9), (24, 24, 24), (8, 30, 11)]):
        gl, gc = grids(P, dims, 90 + k)
        probs.append((gl, gc, capi.Field(dims, capi.KF_F32), P))
    bt = capi.Batch(probs, 5)
    bt.run()
    for gl, gc, f, _ in probs:
        want, _ = solve(gl, gc, P, 5, "band")
        check(np.array_equal(f.download(), want), "batch == band %s" % (gl.dims,))
    bt.close()
    # integration and meshing of a frame on a 32^3 grid
    grid, frames = synth.sphere_pair()
    g = capi.Grid((32, 32, 32), 0.008, (-0.128, -0.128, 0.272), P.unknown_clip, P)
    g.integrate(frames[0], min_depth=0.05, max_depth=1.2)
    phi, w = g.download()
    check(int((w > 0).sum()) > 100, "integration observed voxels")
    n_mc = len(capi.marching_cubes(g, P))
    check(n_mc > 10, "mesh of the integrated frame")
    g.close()
    return checked


def main():
    limit = 0
    if "--limit" in sys.argv:
        limit = int(sys.argv[sys.argv.index("--limit") + 1])
    capi.load()
    capi.bounds_reset(limit)
    failures = []

    def check(ok, what):
        if not ok:
            failures.append(what)

    run(check)
    st = capi.bounds_status()
    st["failures"] = failures
    print(json.dumps(st))


if __name__ == "__main__":
    main()
