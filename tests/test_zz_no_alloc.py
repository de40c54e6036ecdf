"""The allocation-free marching-cubes entry point, through the C ABI.

kf_marching_cubes_noalloc serves callers that cannot allocate device memory
themselves (a frame loop that must not stall on cudaMalloc/cudaFree, or a
host whose device memory belongs to another allocator).  Its output must be
the same as kf_marching_cubes' on the same SDF, call after call, although
every call reuses one scratch array inside the library.  The inputs and
output buffers here are allocated by the test, as such a caller would bring
its own.

This file is collected last on purpose, and it also runs alone in a fresh
process.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import small_pair, sphere_sdf

pytestmark = pytest.mark.gpu

VERTEX_TOL = 1e-4  # voxel, as for the other mesh tests


def mesh_noalloc(capi, phi_dev, dims, P, cap):
    import torch
    L = capi.load()
    verts = torch.full((max(cap, 1), 9), float("nan"), dtype=torch.float32, device="cuda")
    n = C.c_int64(-1)
    st = L.kf_marching_cubes_noalloc(phi_dev.data_ptr(), capi._i3(dims), C.byref(P.c()),
                                     verts.data_ptr(), cap, C.byref(n), None)
    return st, n.value, verts


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(gpu):
    import torch
    capi = gpu
    P = capi.Params.paper(0.004)
    # two different SDFs, one after the other: the second call must not see the first's state
    c0, _ = small_pair(24, 0.004, 5.0, seed=40)
    c1 = sphere_sdf(40, (19.3, 21.1, 20.4), 9.0, 0.004, P.max_surface)
    c1[:, :, :3] = P.max_surface + 1e-5   # a slab with no surface (zero-triangle blocks)
    for phi in (c0, c1):
        nz, ny, nx = phi.shape
        dims = (nx, ny, nz)
        g = capi.Grid(dims, 0.004, (0.0, 0.0, 0.0), P.unknown_clip, P)
        g.upload(phi, (phi <= P.max_surface).astype(np.int32))
        expect = capi.marching_cubes(g, P)  # the allocating entry point
        phi_dev = torch.from_numpy(np.ascontiguousarray(phi, dtype=np.float32)).cuda()
        st, n, verts = mesh_noalloc(capi, phi_dev, dims, P, len(expect) + 7)
        assert st == capi.KF_OK, capi.load().kf_last_error()
        assert n == len(expect) > 100
        got = verts[:n].cpu().numpy().reshape(-1, 3, 3)
        err_vox = np.abs(got - expect).max() / (2.0 / max(dims))
        assert err_vox <= VERTEX_TOL, err_vox
        assert torch.isnan(verts[n:]).all()  # nothing written past the mesh


def test_noalloc_capacity_and_size_limits(gpu):
    import torch
    capi = gpu
    L = capi.load()
    P = capi.Params.paper(0.004)
    c, _ = small_pair(24, 0.004, 5.0, seed=41)
    phi_dev = torch.from_numpy(c).cuda()
    st, n, _ = mesh_noalloc(capi, phi_dev, (24, 24, 24), P, 3)
    assert st == capi.KF_ERR_CAPACITY and n > 3
    n2 = C.c_int64(-1)  # count only: no vertex buffer
    st = L.kf_marching_cubes_noalloc(phi_dev.data_ptr(), capi._i3((24, 24, 24)), C.byref(P.c()),
                                     None, 0, C.byref(n2), None)
    assert st == capi.KF_OK and n2.value == n
    # above the limit: rejected before any device work (the small buffer is never read)
    big = (1024, 1024, 1024)
    assert np.prod(big) > 512 ** 3
    m = C.c_int64(0)
    st = L.kf_marching_cubes_noalloc(phi_dev.data_ptr(), capi._i3(big), C.byref(P.c()), None, 0,
                                     C.byref(m), None)
    assert st == capi.KF_ERR_INVALID
    assert "at most" in L.kf_last_error().decode()


def test_noalloc_calls_allocate_no_device_memory(gpu):
    """The point of the entry point: once the library is loaded and the
    first call has looked up the scratch array's address, further calls
    leave the device's free memory as it was.  Inputs and outputs are the
    caller's, allocated here before the measurement."""
    import torch
    capi = gpu
    L = capi.load()
    P = capi.Params.paper(0.004)
    grids = []
    for k, n in enumerate((24, 40, 33)):
        c, _ = small_pair(n, 0.004, 5.0, seed=50 + k)
        grids.append((torch.from_numpy(c).cuda(), (n, n, n)))
    verts = torch.empty((200_000, 9), dtype=torch.float32, device="cuda")
    counts = []

    def call(phi_dev, dims):
        n = C.c_int64(-1)
        st = L.kf_marching_cubes_noalloc(phi_dev.data_ptr(), capi._i3(dims), C.byref(P.c()),
                                         verts.data_ptr(), verts.shape[0], C.byref(n), None)
        assert st == capi.KF_OK, L.kf_last_error()
        return n.value

    for phi_dev, dims in grids:  # first calls: module load, symbol lookup
        counts.append(call(phi_dev, dims))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(4):
        for k, (phi_dev, dims) in enumerate(grids):
            assert call(phi_dev, dims) == counts[k]
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
