"""Batched problems against the FP64 oracle.

The first three problems of the 64-problem batched workload -- a sphere, a
torus and an ellipsoid pair (synth.shape_problem seeds 1000-1002, at the
workload's edge lengths) -- are solved in one batch (with two more problems
beside them) at the reference's compiled-in weights (config.cpp:45-54) for
the workload's 150 iterations, and each problem's psi is compared with the
FP64 oracle's Jacobi solve (KillingFusion.cpp:248-352) on the same float32
SDFs: within 1e-4 voxel everywhere, the band counts equal.
"""
import numpy as np
import pytest

from killingfusion_gb300 import synth
from oracle.oracle import Params as OParams

pytestmark = pytest.mark.gpu

PSI_TOL = 1e-4
ITERATIONS = 150
# (seed, edge) of the batched workload's first problems, and two more
PROBLEMS = [(1000, 146), (1001, 73), (1002, 154), (1003, 36), (1004, 85)]
KINDS = {1000: "sphere", 1001: "torus", 1002: "ellipsoid"}


def test_batch_problems_match_oracle(gpu, oracle):
    probs, inputs = [], []
    for seed, n in PROBLEMS:
        can, live, voxel = synth.shape_problem(seed, n)
        P = gpu.Params.reference(voxel, 5.0)
        gl = gpu.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
        gc = gpu.Grid((n, n, n), voxel, (0, 0, 0), P.unknown_clip, P)
        gl.upload(live, (live <= P.max_surface).astype(np.int32))
        gc.upload(can, (can <= P.max_surface).astype(np.int32))
        probs.append((gl, gc, gpu.Field((n, n, n), gpu.KF_F32), P))
        inputs.append((live, can, P))
    b = gpu.Batch(probs, ITERATIONS)
    b.autotune()
    stats = b.run()
    for (seed, n), (gl, gc, f, P), (live, can, _), st in zip(PROBLEMS, probs, inputs, stats):
        if seed not in KINDS:
            continue
        OP = OParams(**{k: getattr(P, k) for k in OParams.__dataclass_fields__})
        ost, opsi, counts = oracle.solve(live.astype(np.float64), can.astype(np.float64),
                                         np.zeros((n, n, n, 3)), ITERATIONS, OP, active_counts=True)
        assert ost == 0
        assert st["iterations_run"] == ITERATIONS
        assert st["active_first"] == counts[0] > 100, KINDS[seed]
        assert st["active_last"] == counts[-1], KINDS[seed]
        err = np.abs(f.download().astype(np.float64) - opsi)
        assert err.max() <= PSI_TOL, (KINDS[seed], err.max(), int((err > PSI_TOL).sum()))
        assert np.abs(opsi).max() > 50 * PSI_TOL, KINDS[seed]  # psi moved well beyond the tolerance
    b.close()
