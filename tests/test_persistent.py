"""The band-only solver's persistent launch (KF_SOLVER_BAND).

Every band pass of a solve runs in one cooperative launch, the iterations
separated by a grid-wide barrier whose wait is bounded (kf_set_wait_limit).
* psi and the statistics equal the dense fused solver's, over solves long
  enough to cross many barriers, including one that converges early;
* a wait limit of zero makes every block but the last to arrive give up at
  the first barrier: the solve returns KF_ERR_TIMEOUT, the GPU context stays
  usable, and the next solve with the default limit is correct again.  No
  kernel is made to fault or hang: the barrier's own bound ends the wait.
"""
import numpy as np
import pytest

from helpers import small_pair

pytestmark = pytest.mark.gpu


def grids(capi, P, n=40, seed=60):
    can, live = small_pair(n, P.voxel_size, 5.0, seed=seed)
    dims = (n, n, n)
    gl = capi.Grid(dims, P.voxel_size, (0, 0, 0), P.unknown_clip, P)
    gc = capi.Grid(dims, P.voxel_size, (0, 0, 0), P.unknown_clip, P)
    gl.upload(live, (live <= P.max_surface).astype(np.int32))
    gc.upload(can, (can <= P.max_surface).astype(np.int32))
    return gl, gc, dims


def solve(capi, gl, gc, dims, P, iters, solver):
    f = capi.Field(dims, capi.KF_F32)
    st = capi.psi_solve(gl, gc, f, P, iters, solver)
    out = f.download()
    f.close()
    return out, st


@pytest.mark.parametrize("iters", [1, 2, 7, 150])
def test_persistent_band_equals_dense(gpu, iters):
    capi = gpu
    P = capi.Params.paper(0.004)
    gl, gc, dims = grids(capi, P)
    a, sa = solve(capi, gl, gc, dims, P, iters, "band")
    b, sb = solve(capi, gl, gc, dims, P, iters, "fused")
    np.testing.assert_array_equal(a, b)
    for k in ("iterations_run", "active_first", "active_last", "max_delta_last", "converged", "diverged"):
        assert sa[k] == sb[k], k
    assert abs(sa["energy_last"] - sb["energy_last"]) <= 1e-9 * max(abs(sb["energy_last"]), 1.0)


def test_persistent_band_early_exit(gpu):
    capi = gpu
    # the steps of this pair start at 1.3e-4 voxel and fall below 1.05e-4 after
    # about 100 iterations (FP64 oracle)
    P = capi.Params.reference(0.004, 5.0).with_(early_exit=True, threshold=1.05e-4)
    gl, gc, dims = grids(capi, P, seed=61)
    a, sa = solve(capi, gl, gc, dims, P, 300, "band")
    b, sb = solve(capi, gl, gc, dims, P, 300, "fused")
    assert sa["converged"] == 1 and 1 < sa["iterations_run"] < 300
    assert sa["iterations_run"] == sb["iterations_run"]
    np.testing.assert_array_equal(a, b)


def test_wait_limit_gives_timeout_status(gpu):
    capi = gpu
    L = capi.load()
    P = capi.Params.paper(0.004)
    gl, gc, dims = grids(capi, P, seed=62)
    expect, _ = solve(capi, gl, gc, dims, P, 20, "fused")
    prev = capi.set_wait_limit(0.0)
    try:
        f = capi.Field(dims, capi.KF_F32)
        st = L.kf_psi_solve(gl.h, gc.h, f.h, capi.C.byref(P.c()), 20, capi.KF_SOLVER_BAND, None, None)
        assert st == capi.KF_ERR_TIMEOUT, (st, L.kf_last_error())
        assert b"gave up" in L.kf_last_error()
        f.close()
    finally:
        assert capi.set_wait_limit(prev) == 0.0
    # the context is usable and the next solve is right
    got, st = solve(capi, gl, gc, dims, P, 20, "band")
    np.testing.assert_array_equal(got, expect)
    assert st["iterations_run"] == 20
    with pytest.raises(ValueError):
        capi.set_wait_limit(-1.0)


@pytest.mark.parametrize("probe", [40, 41])
def test_persistent_band_early_exit_either_parity(gpu, probe):
    """The gate of the next iteration comes with the barrier, in one of two
    words by the barrier's parity: a threshold at the last step of a solve
    of `probe` iterations stops the loop after an even and an odd
    iteration, where the dense solver stops."""
    capi = gpu
    P0 = capi.Params.reference(0.004, 5.0)
    gl, gc, dims = grids(capi, P0, seed=61)
    _, sp = solve(capi, gl, gc, dims, P0, probe, "band")
    P = P0.with_(early_exit=True, threshold=float(sp["max_delta_last"]) * 1.0001)
    a, sa = solve(capi, gl, gc, dims, P, 300, "band")
    b, sb = solve(capi, gl, gc, dims, P, 300, "fused")
    assert sa["converged"] == 1 and 1 < sa["iterations_run"] <= probe
    for k in ("iterations_run", "active_first", "active_last", "max_delta_last", "converged", "diverged"):
        assert sa[k] == sb[k], k
    np.testing.assert_array_equal(a, b)


def test_persistent_band_divergence_equals_dense(gpu):
    """A non-finite psi inside the band: the band solver reports
    KF_ERR_DIVERGED after the same iterations as the dense solver, with the
    same psi and statistics."""
    capi = gpu
    L = capi.load()
    P = capi.Params.paper(0.004)
    gl, gc, dims = grids(capi, P, seed=63)
    live, _ = gl.download()
    z, y, x = np.argwhere((live > -0.004) & (live < 0.004))[0]
    psi = np.zeros(live.shape + (3,), np.float32)
    psi[z, y, x, 0] = np.nan
    got = {}
    for solver in ("band", "fused"):
        f = capi.Field(dims, capi.KF_F32)
        f.upload(psi)
        st = capi.SolveStats()
        rc = L.kf_psi_solve(gl.h, gc.h, f.h, capi.C.byref(P.c()), 20, capi.SOLVERS[solver], capi.C.byref(st), None)
        assert rc == capi.KF_ERR_DIVERGED, (solver, rc)
        got[solver] = (f.download(), st.as_dict())
        f.close()
    (a, sa), (b, sb) = got["band"], got["fused"]
    assert sa["diverged"] == 1
    for k in ("iterations_run", "active_first", "active_last", "converged", "diverged"):
        assert sa[k] == sb[k], k
    np.testing.assert_array_equal(a, b)


def test_band_first_pass_on_a_zero_field(gpu):
    """Once the band-only solver has used a field, kf_field_zero clears both
    of its buffers (all of them, or only the places the field has recorded),
    and the next band-only solve's first pass reads phi_live alone.
    Whatever wrote psi before the zero (a warp, which borrows the second
    buffer; an upload; a fill; a dense solve; a per-voxel update), a
    band-only solve from zero gives the dense solver's psi and statistics;
    and a write after the zero sends the solve back to the first pass that
    reads psi, with the dense solver's result from the same psi."""
    capi = gpu
    P = capi.Params.reference(0.004, 5.0)
    gl, gc, dims = grids(capi, P, seed=64)
    expect, se = solve(capi, gl, gc, dims, P, 40, "fused")
    scratch = capi.Grid(dims, P.voxel_size, (0, 0, 0), P.unknown_clip, P)
    scratch.upload(*gl.download())
    rng = np.random.default_rng(5)
    nonzero = (rng.standard_normal(gl.shape + (3,)) * 0.2).astype(np.float32)
    keys = ("iterations_run", "active_first", "active_last", "max_delta_last", "converged", "diverged")
    f = capi.Field(dims, capi.KF_F32)
    writes = [
        lambda g: None,
        lambda g: capi.warp(scratch, g, P),
        lambda g: g.upload(nonzero),
        lambda g: capi.field_fill(g, (0.05, -0.025, 0.0125)),
        lambda g: capi.psi_solve(gl, gc, g, P, 3, "fused"),
        lambda g: capi.field_add_voxels(g, [[20, 21, 19]], [[0.3, 0.0, -0.2]]),
    ]
    for k, write in enumerate(writes):
        write(f)
        f.zero()
        st = capi.psi_solve(gl, gc, f, P, 40, "band")
        np.testing.assert_array_equal(f.download(), expect, err_msg=str(k))
        for key in keys:
            assert st[key] == se[key], (k, key)
    # the frame pipeline's cycle: a band-only solve from zero records the
    # voxels it can change; warp + fuse finds the moved ones among them
    # (against warp + fuse reading psi at every voxel, from a field holding
    # the same psi) and records the entries of the second buffer it borrows;
    # the next zero clears those alone
    def copy(g):
        c = capi.Grid(dims, P.voxel_size, (0, 0, 0), P.unknown_clip, P)
        c.upload(*g.download())
        return c

    for _ in range(3):
        f.zero()
        assert not f.download().any()
        st = capi.psi_solve(gl, gc, f, P, 40, "band")
        np.testing.assert_array_equal(f.download(), expect)
        can1, live1, can2, live2 = copy(gc), copy(gl), copy(gc), copy(gl)
        capi.warp_fuse(can1, live1, f, P)
        g = capi.Field(dims, capi.KF_F32)
        g.upload(f.download())
        capi.warp_fuse(can2, live2, g, P)
        for a, b in ((can1, can2), (live1, live2)):
            for x, y in zip(a.download(), b.download()):
                np.testing.assert_array_equal(x, y)
        for h in (can1, live1, can2, live2, g):
            h.close()
    for k, write in enumerate(writes[2:]):
        f.zero()
        write(f)
        st = capi.psi_solve(gl, gc, f, P, 40, "band")
        g = capi.Field(dims, capi.KF_F32)
        write(g)
        sg = capi.psi_solve(gl, gc, g, P, 40, "fused")
        np.testing.assert_array_equal(f.download(), g.download(), err_msg=str(k))
        for key in keys:
            assert st[key] == sg[key], (k, key)
        g.close()
    f.close()
