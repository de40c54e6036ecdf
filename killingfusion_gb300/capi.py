"""ctypes binding of the C ABI (include/killingfusion.h).

The library is ``killingfusion_gb300/_lib/libkillingfusion.so``, built in-tree
by ``killingfusion_gb300._build`` (``__graft_entry__.build()``).  There is no
fallback: if the library is missing, importing this module raises.

Device buffers that the ABI writes into (mesh vertices, gradient queries) are
torch CUDA tensors; torch is used only as device-memory plumbing.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, asdict, replace

import numpy as np

from . import _build

# KF_LIBRARY=bounds_check selects the build with checked indices
# (_build.LIB_BC); tests run it in a process of its own
LIB_PATH = _build.LIB_BC if os.environ.get("KF_LIBRARY") == "bounds_check" else _build.LIB

(KF_OK, KF_ERR_INVALID, KF_ERR_OOM, KF_ERR_CUDA, KF_ERR_DIVERGED, KF_ERR_TIMEOUT, KF_ERR_CAPACITY,
 KF_ERR_INTERNAL) = range(8)
KF_F32, KF_F64 = 0, 1
KF_SOLVER_FUSED, KF_SOLVER_PLAIN, KF_SOLVER_EXACT, KF_SOLVER_BAND, KF_SOLVER_PERVOXEL = 0, 1, 2, 3, 4
SOLVERS = {"fused": KF_SOLVER_FUSED, "plain": KF_SOLVER_PLAIN, "exact": KF_SOLVER_EXACT,
           "band": KF_SOLVER_BAND, "pervoxel": KF_SOLVER_PERVOXEL}


class KFError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("kf status %d: %s" % (status, msg))
        self.status = status


class DivergedError(KFError):
    """psi turned non-finite inside the band (the reference throws -1)."""


class _Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "voxel_size", "unknown_clip", "max_surface", "epsilon", "delta_size", "alpha",
        "omega_k", "gamma_k", "omega_s", "threshold", "killing_clamp")] + [
        ("use_data", C.c_int), ("use_levelset", C.c_int), ("use_killing", C.c_int),
        ("early_exit", C.c_int), ("use_trust", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iterations_run", C.c_int32), ("converged", C.c_int32), ("diverged", C.c_int32),
                ("capped", C.c_int32), ("active_first", C.c_int64), ("active_last", C.c_int64),
                ("energy_first", C.c_double), ("energy_last", C.c_double),
                ("max_delta_last", C.c_double), ("device_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


@dataclass(frozen=True)
class Params:
    """kf_params: the reference's config.h globals (config.cpp:4-57)."""

    voxel_size: float = 0.012
    unknown_clip: float = 0.048
    max_surface: float = 0.048
    epsilon: float = 1e-5
    delta_size: float = 0.05
    alpha: float = 0.025
    omega_k: float = 0.04
    gamma_k: float = 0.0
    omega_s: float = 0.1
    threshold: float = 1e-6
    killing_clamp: float = 0.1
    use_data: bool = True
    use_levelset: bool = True
    use_killing: bool = True
    early_exit: bool = False
    use_trust: bool = False

    @staticmethod
    def reference(voxel_size: float = 0.012, trunc_voxels: float = 4.0) -> "Params":
        """The reference's compiled-in weights, with a chosen voxel/band."""
        t = voxel_size * trunc_voxels
        return Params(voxel_size=voxel_size, unknown_clip=t, max_surface=t)

    @staticmethod
    def paper(voxel_size: float, trunc_voxels: float = 5.0) -> "Params":
        t = voxel_size * trunc_voxels
        return Params(voxel_size=voxel_size, unknown_clip=t, max_surface=t, alpha=0.1,
                      omega_k=0.5, gamma_k=0.1, omega_s=0.2)

    def with_(self, **kw) -> "Params":
        return replace(self, **kw)

    def c(self) -> _Params:
        d = asdict(self)
        return _Params(**{k: (int(v) if isinstance(v, bool) else v) for k, v in d.items()})


_vp = C.c_void_p
_ip3 = C.POINTER(C.c_int)
_ip6 = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_PP = C.POINTER(_Params)

# name -> (restype, argtypes); the full ABI of include/killingfusion.h
SIGNATURES = {
    "kf_version": (C.c_int, []),
    "kf_last_error": (C.c_char_p, []),
    "kf_params_reference": (None, [_PP]),
    "kf_params_paper": (None, [_PP, C.c_double, C.c_double]),
    "kf_mc_case": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "kf_grid_create": (C.c_int, [_ip3, C.c_double, _dp, C.c_double, _PP, C.POINTER(_vp)]),
    "kf_grid_destroy": (C.c_int, [_vp]),
    "kf_grid_info": (C.c_int, [_vp, _ip3, _dp, _dp, _dp]),
    "kf_grid_reset": (C.c_int, [_vp, _PP, _vp]),
    "kf_grid_upload": (C.c_int, [_vp, _vp, _vp, _vp]),
    "kf_grid_download": (C.c_int, [_vp, _vp, _vp, _vp]),
    "kf_grid_device": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp)]),
    "kf_field_create": (C.c_int, [_ip3, C.c_int, C.POINTER(_vp)]),
    "kf_field_destroy": (C.c_int, [_vp]),
    "kf_field_zero": (C.c_int, [_vp, _vp]),
    "kf_field_upload": (C.c_int, [_vp, _vp, _vp]),
    "kf_field_download": (C.c_int, [_vp, _vp, _vp]),
    "kf_field_device": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp)]),
    "kf_integrate_depth": (C.c_int, [_vp, _vp, C.c_int, C.c_int, _dp, _dp, C.c_double,
                                     C.c_double, _vp]),
    "kf_integrate_depth_u16": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_double,
                                         C.c_double, _vp]),
    "kf_compute_sdf": (C.c_int, [_vp, _PP, _vp, C.c_int, C.c_int, _dp, _dp, C.c_double, C.c_double, _vp]),
    "kf_compute_sdf_u16": (C.c_int, [_vp, _PP, _vp, C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_double,
                                     C.c_double, _vp]),
    "kf_psi_solve": (C.c_int, [_vp, _vp, _vp, _PP, C.c_int, C.c_int, C.POINTER(SolveStats), _vp]),
    "kf_psi_solve_async": (C.c_int, [_vp, _vp, _vp, _PP, C.c_int, C.c_int, _vp]),
    "kf_psi_solve_wait": (C.c_int, [_vp, C.POINTER(SolveStats)]),
    "kf_psi_gradient_ref": (C.c_int, [_vp, _vp, _vp, _PP, _vp, C.c_int, _vp, _vp, _vp]),
    "kf_energy": (C.c_int, [_vp, _vp, _vp, _PP, _vp, _ip6, C.c_int, _dp, _vp]),
    "kf_energy_adjoint": (C.c_int, [_vp, _vp, _vp, _PP, _vp, _vp, _vp]),
    "kf_energy_fd": (C.c_int, [_vp, _vp, _vp, _PP, _vp, _vp, C.c_int, C.c_double, _vp, _vp]),
    "kf_batch_create": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(_vp)]),
    "kf_batch_destroy": (C.c_int, [_vp]),
    "kf_batch_autotune": (C.c_int, [_vp, C.c_void_p, _vp]),
    "kf_batch_set_shape": (C.c_int, [_vp, C.c_void_p]),
    "kf_batch_run": (C.c_int, [_vp, _vp, _vp]),
    "kf_warp": (C.c_int, [_vp, _vp, _PP, _vp]),
    "kf_fuse": (C.c_int, [_vp, _vp, _vp]),
    "kf_warp_fuse": (C.c_int, [_vp, _vp, _vp, _PP, _vp]),
    "kf_fuse_warped": (C.c_int, [_vp, _vp, _vp, _PP, _vp]),
    "kf_marching_cubes": (C.c_int, [_vp, _PP, _vp, C.c_int64, C.POINTER(C.c_int64), _vp]),
    "kf_marching_cubes_async": (C.c_int, [_vp, _PP, _vp, C.c_int64, _vp, _vp]),
    "kf_marching_cubes_noalloc": (C.c_int, [_vp, _ip3, _PP, _vp, C.c_int64, C.POINTER(C.c_int64),
                                            _vp]),
    "kf_mesh_host": (C.c_int, [_vp, _PP, _vp, C.c_int64, C.POINTER(C.c_int64), _vp]),
    "kf_field_add": (C.c_int, [_vp, _vp, _vp]),
    "kf_field_fill": (C.c_int, [_vp, _dp, _vp]),
    "kf_field_get_voxels": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp]),
    "kf_field_add_voxels": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp]),
    "kf_field_sample": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp]),
    "kf_grid_sample": (C.c_int, [_vp, _PP, _vp, C.c_int, _vp, _vp, _vp]),
    "kf_grid_get_voxels": (C.c_int, [_vp, _PP, _vp, C.c_int, _vp, _vp, _vp]),
    "kf_fusion_create": (C.c_int, [C.c_void_p, C.POINTER(_vp)]),
    "kf_fusion_destroy": (C.c_int, [_vp]),
    "kf_fusion_process_frame": (C.c_int, [_vp, _vp, _dp, C.c_int, C.c_void_p, _vp]),
    "kf_fusion_state": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp)]),
    "kf_set_wait_limit": (C.c_double, [C.c_double]),
    "kf_psi_solve_history": (C.c_int, [_vp, C.c_int32, _vp, _vp, _vp, C.POINTER(C.c_int32)]),
    "kf_bounds_status": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int64), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "kf_bounds_reset": (C.c_int, [C.c_int64]),
    "kf_fusion_save": (C.c_int, [_vp, C.c_char_p, _vp]),
    "kf_fusion_load": (C.c_int, [_vp, C.c_char_p, _vp]),
    "kf_state_save": (C.c_int, [C.c_char_p, _vp, _vp, C.c_int32, _vp]),
    "kf_state_info": (C.c_int, [C.c_char_p, _ip3, _vp, _vp, _vp, _vp, _vp]),
    "kf_state_load": (C.c_int, [C.c_char_p, _vp, _vp, _vp, _vp]),
    "kf_grid_load_ref_bin": (C.c_int, [C.c_char_p, _PP, C.c_double, C.POINTER(_vp), _vp, _vp]),
}

_lib = None


def load() -> C.CDLL:
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("%s is missing: run __graft_entry__.build() (or python -m "
                              "killingfusion_gb300._build) first" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def solve_history(field, max_iterations: int = 100000) -> dict:
    """Per-iteration energy, max |dpsi| and band count of the last solve on
    field (kf_psi_solve_history)."""
    e = np.zeros(max_iterations)
    d = np.zeros(max_iterations)
    a = np.zeros(max_iterations, np.int64)
    n = C.c_int32(0)
    check(load().kf_psi_solve_history(field.h, max_iterations, e.ctypes.data, d.ctypes.data, a.ctypes.data,
                                      C.byref(n)))
    k = n.value
    return {"energy": e[:k], "max_delta": d[:k], "active": a[:k]}


def bounds_status() -> dict:
    """The bounds-check build's record (enabled = 0 in the normal build)."""
    en, n, site, idx, bound = C.c_int(), C.c_int64(), C.c_int(), C.c_int64(), C.c_int64()
    check(load().kf_bounds_status(C.byref(en), C.byref(n), C.byref(site), C.byref(idx), C.byref(bound)))
    return {"enabled": en.value, "violations": n.value, "site": site.value, "index": idx.value,
            "bound": bound.value}


def bounds_reset(limit: int = 0):
    check(load().kf_bounds_reset(int(limit)))


def set_wait_limit(seconds: float) -> float:
    """Limit of one device-side wait of the persistent kernels (default 1 s);
    returns the previous limit."""
    prev = load().kf_set_wait_limit(float(seconds))
    if prev < 0:
        raise ValueError("wait limit outside [0, 60] s")
    return prev


def check(status: int):
    if status != KF_OK:
        msg = load().kf_last_error().decode()
        if status == KF_ERR_DIVERGED:
            raise DivergedError(status, msg)
        raise KFError(status, msg)


def _stream(stream) -> int | None:
    if stream is None:
        return None
    return int(getattr(stream, "cuda_stream", stream))


def _i3(v):
    return (C.c_int * 3)(*[int(x) for x in v])


def _d(v):
    v = list(v)
    return (C.c_double * len(v))(*[float(x) for x in v])


class Grid:
    """An SDF grid (class SDF): float32 phi + int32 weights on the device."""

    def __init__(self, dims, voxel_size: float, origin, unknown_clip: float, params: Params):
        L = load()
        self.dims = tuple(int(d) for d in dims)  # (nx, ny, nz)
        self.shape = self.dims[::-1]
        self.voxel_size = float(voxel_size)
        self.origin = np.asarray(origin, dtype=np.float64)
        h = _vp()
        check(L.kf_grid_create(_i3(self.dims), voxel_size, _d(self.origin), unknown_clip,
                               C.byref(params.c()), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().kf_grid_destroy(self.h)
            self.h = None

    __del__ = close

    def upload(self, phi=None, weight=None, stream=None):
        p = np.ascontiguousarray(phi, dtype=np.float32) if phi is not None else None
        w = np.ascontiguousarray(weight, dtype=np.int32) if weight is not None else None
        if p is not None:
            assert p.size == np.prod(self.dims)
        check(load().kf_grid_upload(self.h, p.ctypes.data if p is not None else None,
                                    w.ctypes.data if w is not None else None, _stream(stream)))

    def download(self, stream=None):
        phi = np.empty(self.shape, dtype=np.float32)
        w = np.empty(self.shape, dtype=np.int32)
        check(load().kf_grid_download(self.h, phi.ctypes.data, w.ctypes.data, _stream(stream)))
        return phi, w

    def reset(self, params: Params, stream=None):
        check(load().kf_grid_reset(self.h, C.byref(params.c()), _stream(stream)))

    def device_ptrs(self):
        p, w = _vp(), _vp()
        check(load().kf_grid_device(self.h, C.byref(p), C.byref(w)))
        return p.value, w.value

    def integrate(self, depth, c2w=None, K=None, min_depth=0.05, max_depth=1.2, stream=None):
        """SDF::integrateDepthFrame; depth: numpy float32 [h, w] or a CUDA tensor."""
        from . import synth
        c2w = np.eye(4) if c2w is None else np.asarray(c2w, dtype=np.float64)
        K = synth.K if K is None else np.asarray(K, dtype=np.float64)
        if isinstance(depth, np.ndarray):
            d = np.ascontiguousarray(depth, dtype=np.float32)
            ptr, (hh, ww) = d.ctypes.data, d.shape
        else:
            ptr, (hh, ww) = depth.data_ptr(), tuple(depth.shape)
        check(load().kf_integrate_depth(self.h, ptr, ww, hh, _d(c2w.ravel()), _d(K.ravel()),
                                        min_depth, max_depth, _stream(stream)))

    def compute_sdf(self, params, depth, c2w=None, K=None, min_depth=0.05, max_depth=1.2, u16_scale=None,
                    stream=None):
        """KillingFusion::computeSDF: reset + integrate in one pass (the same
        result as reset() then integrate() / integrate_u16()).  depth: numpy
        float32 (or uint16 with u16_scale) [h, w], or a CUDA tensor."""
        from . import synth
        c2w = np.eye(4) if c2w is None else np.asarray(c2w, dtype=np.float64)
        K = synth.K if K is None else np.asarray(K, dtype=np.float64)
        dt = np.float32 if u16_scale is None else np.uint16
        if isinstance(depth, np.ndarray):
            d = np.ascontiguousarray(depth, dtype=dt)
            ptr, (hh, ww) = d.ctypes.data, d.shape
        else:
            ptr, (hh, ww) = depth.data_ptr(), tuple(depth.shape)
        if u16_scale is None:
            check(load().kf_compute_sdf(self.h, C.byref(params.c()), ptr, ww, hh, _d(c2w.ravel()),
                                        _d(K.ravel()), min_depth, max_depth, _stream(stream)))
        else:
            check(load().kf_compute_sdf_u16(self.h, C.byref(params.c()), ptr, ww, hh, float(u16_scale),
                                            _d(c2w.ravel()), _d(K.ravel()), min_depth, max_depth,
                                            _stream(stream)))

    def integrate_u16(self, depth, scale=0.001, c2w=None, K=None, min_depth=0.05, max_depth=1.2, stream=None):
        """SDF::integrateDepthFrame on 16-bit depth (numpy uint16 [h, w] or a
        CUDA tensor); each value is (double)v * scale."""
        from . import synth
        c2w = np.eye(4) if c2w is None else np.asarray(c2w, dtype=np.float64)
        K = synth.K if K is None else np.asarray(K, dtype=np.float64)
        if isinstance(depth, np.ndarray):
            d = np.ascontiguousarray(depth, dtype=np.uint16)
            ptr, (hh, ww) = d.ctypes.data, d.shape
        else:
            ptr, (hh, ww) = depth.data_ptr(), tuple(depth.shape)
        check(load().kf_integrate_depth_u16(self.h, ptr, ww, hh, float(scale), _d(c2w.ravel()),
                                            _d(K.ravel()), min_depth, max_depth, _stream(stream)))


class Field:
    """A displacement field psi (class DisplacementField)."""

    def __init__(self, dims, precision: int = KF_F32):
        L = load()
        self.dims = tuple(int(d) for d in dims)
        self.shape = self.dims[::-1]
        self.precision = precision
        self.dtype = np.float32 if precision == KF_F32 else np.float64
        h = _vp()
        check(L.kf_field_create(_i3(self.dims), precision, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().kf_field_destroy(self.h)
            self.h = None

    __del__ = close

    def zero(self, stream=None):
        check(load().kf_field_zero(self.h, _stream(stream)))

    def upload(self, psi, stream=None):
        a = np.ascontiguousarray(psi, dtype=self.dtype)
        assert a.shape == self.shape + (3,)
        check(load().kf_field_upload(self.h, a.ctypes.data, _stream(stream)))

    def download(self, stream=None):
        a = np.empty(self.shape + (3,), dtype=self.dtype)
        check(load().kf_field_download(self.h, a.ctypes.data, _stream(stream)))
        return a


def psi_solve(live: Grid, can: Grid, psi: Field, params: Params, iterations: int,
              solver: str = "fused", stream=None) -> dict:
    st = SolveStats()
    check(load().kf_psi_solve(live.h, can.h, psi.h, C.byref(params.c()), int(iterations),
                              SOLVERS[solver], C.byref(st), _stream(stream)))
    return st.as_dict()


def psi_solve_async(live: Grid, can: Grid, psi: Field, params: Params, iterations: int,
                    solver: str = "fused", stream=None) -> None:
    """Queue a solve (kf_psi_solve_async); psi_solve_wait reads its stats."""
    check(load().kf_psi_solve_async(live.h, can.h, psi.h, C.byref(params.c()), int(iterations),
                                    SOLVERS[solver], _stream(stream)))


def psi_solve_wait(psi: Field) -> dict:
    st = SolveStats()
    check(load().kf_psi_solve_wait(psi.h, C.byref(st)))
    return st.as_dict()


def psi_gradient_ref(live: Grid, can: Grid, psi: Field, params: Params, voxels_xyz):
    """Reference gradient (KillingFusion::computeEnergyGradient) and band flag
    at voxels (int [n, 3] of x, y, z)."""
    import torch
    v = torch.as_tensor(np.ascontiguousarray(voxels_xyz, dtype=np.int32)).cuda()
    n = v.shape[0]
    out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    act = torch.empty((n,), dtype=torch.uint8, device="cuda")
    check(load().kf_psi_gradient_ref(live.h, can.h, psi.h, C.byref(params.c()), v.data_ptr(),
                                     n, out.data_ptr(), act.data_ptr(), None))
    torch.cuda.synchronize()
    return out.cpu().numpy(), act.cpu().numpy()


def _active_tensor(active, count):
    import torch
    if active is None:
        return None
    a = torch.as_tensor(np.ascontiguousarray(active, dtype=np.uint8).reshape(-1)).cuda()
    assert a.numel() == count
    return a


def energy(live: Grid, can: Grid, psi: Field, params: Params, active=None, box=None,
           arith: str = "f64") -> np.ndarray:
    """Project energy terms (data, level set, Killing) over the active voxels
    (uint8 mask of the grid, None = all) inside box (x0, y0, z0, x1, y1, z1,
    half-open; None = the grid)."""
    a = _active_tensor(active, int(np.prod(live.dims)))
    terms = np.zeros(3)
    b = (C.c_int * 6)(*[int(v) for v in box]) if box is not None else None
    check(load().kf_energy(live.h, can.h, psi.h, C.byref(params.c()), a.data_ptr() if a is not None else None,
                           b, KF_F64 if arith == "f64" else KF_F32,
                           terms.ctypes.data_as(C.POINTER(C.c_double)), None))
    return terms


def energy_adjoint(live: Grid, can: Grid, psi: Field, params: Params, active=None) -> np.ndarray:
    """Exact gradient of the project energy with respect to psi, float64
    [nz, ny, nx, 3]."""
    import torch
    a = _active_tensor(active, int(np.prod(live.dims)))
    out = torch.empty(live.shape + (3,), dtype=torch.float64, device="cuda")
    check(load().kf_energy_adjoint(live.h, can.h, psi.h, C.byref(params.c()),
                                   a.data_ptr() if a is not None else None, out.data_ptr(), None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def energy_fd(live: Grid, can: Grid, psi: Field, params: Params, voxels_xyz, h: float, active=None):
    """Central differences (float64) of the project energy at voxels (int
    [n, 3] of x, y, z), one column per psi component."""
    import torch
    a = _active_tensor(active, int(np.prod(live.dims)))
    v = torch.as_tensor(np.ascontiguousarray(voxels_xyz, dtype=np.int32)).cuda()
    n = v.shape[0]
    out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    check(load().kf_energy_fd(live.h, can.h, psi.h, C.byref(params.c()),
                              a.data_ptr() if a is not None else None, v.data_ptr(), n, float(h),
                              out.data_ptr(), None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def warp(g: Grid, psi: Field, params: Params, stream=None):
    check(load().kf_warp(g.h, psi.h, C.byref(params.c()), _stream(stream)))


def fuse(can: Grid, other: Grid, stream=None):
    check(load().kf_fuse(can.h, other.h, _stream(stream)))


def warp_fuse(can: Grid, live: Grid, psi: Field, params: Params, stream=None):
    check(load().kf_warp_fuse(can.h, live.h, psi.h, C.byref(params.c()), _stream(stream)))


def fuse_warped(dst: Grid, other: Grid, psi: Field, params: Params, stream=None):
    check(load().kf_fuse_warped(dst.h, other.h, psi.h, C.byref(params.c()), _stream(stream)))


def marching_cubes(g: Grid, params: Params):
    """SDF::getMesh as float32 [T, 3, 3] (numpy)."""
    import torch
    L = load()
    n = C.c_int64(0)
    check(L.kf_marching_cubes(g.h, C.byref(params.c()), None, 0, C.byref(n), None))
    t = torch.empty((max(n.value, 1), 9), dtype=torch.float32, device="cuda")
    check(L.kf_marching_cubes(g.h, C.byref(params.c()), t.data_ptr(), n.value, C.byref(n), None))
    torch.cuda.synchronize()
    return t[: n.value].cpu().numpy().reshape(-1, 3, 3)


def mc_case(cube: int):
    em = C.c_int(0)
    row = (C.c_int * 16)()
    check(load().kf_mc_case(cube, C.byref(em), row))
    return em.value, list(row)


# ---------------------------------------------------------------------------
# point queries (SDF / DisplacementField accessors)
# ---------------------------------------------------------------------------

def grid_sample(g: Grid, params: Params, pts):
    """SDF::getDistance / SDF::getWeight at grid points [n, 3] -> (phi, w)."""
    p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    phi = np.empty(len(p))
    w = np.empty(len(p))
    check(load().kf_grid_sample(g.h, C.byref(params.c()), p.ctypes.data, len(p), phi.ctypes.data,
                                w.ctypes.data, None))
    return phi, w


def grid_get_voxels(g: Grid, params: Params, xyz):
    v = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
    phi = np.empty(len(v))
    w = np.empty(len(v), dtype=np.int64)
    check(load().kf_grid_get_voxels(g.h, C.byref(params.c()), v.ctypes.data, len(v), phi.ctypes.data,
                                    w.ctypes.data, None))
    return phi, w


def field_get_voxels(f: Field, xyz):
    v = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
    out = np.empty((len(v), 3))
    check(load().kf_field_get_voxels(f.h, v.ctypes.data, len(v), out.ctypes.data, None))
    return out


def field_sample(f: Field, pts):
    p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    out = np.empty((len(p), 3))
    check(load().kf_field_sample(f.h, p.ctypes.data, len(p), out.ctypes.data, None))
    return out


def field_add_voxels(f: Field, xyz, delta):
    v = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
    d = np.ascontiguousarray(delta, dtype=np.float64).reshape(-1, 3)
    check(load().kf_field_add_voxels(f.h, v.ctypes.data, len(v), d.ctypes.data, None))


def field_add(f: Field, other: Field):
    check(load().kf_field_add(f.h, other.h, None))


def field_fill(f: Field, v):
    check(load().kf_field_fill(f.h, _d(v), None))


# ---------------------------------------------------------------------------
# per-frame pipeline (KillingFusion::processNextFrame)
# ---------------------------------------------------------------------------

class BatchItem(C.Structure):
    _fields_ = [("live", _vp), ("canonical", _vp), ("psi", _vp), ("params", _Params)]


class BatchShape(C.Structure):
    """kf_batch_shape: launch shape of a batch (band pass and dense pass)."""
    _fields_ = [("band_threads", C.c_int), ("band_chunk", C.c_int), ("band_blocks_per_sm", C.c_int),
                ("band_registers", C.c_int), ("slab", C.c_int), ("reserved", C.c_int),
                ("band_ms", C.c_double), ("stream_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


# (band threads, chunk voxels, CTAs per SM, registers) of every band-pass
# shape the autotuner tries, and its slab depths
BATCH_BAND_SHAPES = [(256, 256, 2, 128), (256, 256, 3, 80), (256, 512, 2, 128), (256, 512, 3, 80),
                     (512, 512, 1, 128), (512, 1024, 1, 128)]
BATCH_SLABS = [4, 8, 16]


class Batch:
    """Independent registration problems solved together (kf_batch_*):
    problems is a list of (live Grid, canonical Grid, psi Field, Params)."""

    def __init__(self, problems, iterations: int):
        items = (BatchItem * len(problems))()
        for k, (live, can, psi, params) in enumerate(problems):
            items[k].live, items[k].canonical, items[k].psi = live.h, can.h, psi.h
            items[k].params = params.c()
        self.problems = list(problems)  # keep the handles alive
        self.n = len(problems)
        h = _vp()
        check(load().kf_batch_create(items, len(problems), int(iterations), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().kf_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def autotune(self, stream=None) -> dict:
        """The fastest launch shape on this batch's data (kf_batch_shape)."""
        sh = BatchShape()
        check(load().kf_batch_autotune(self.h, C.byref(sh), _stream(stream)))
        return sh.as_dict()

    def set_shape(self, band, slab=8):
        """band: (threads, chunk, CTAs per SM, registers), one of
        BATCH_BAND_SHAPES; slab: one of BATCH_SLABS."""
        sh = BatchShape(*band, slab, 0, 0.0, 0.0)
        check(load().kf_batch_set_shape(self.h, C.byref(sh)))

    def run(self, stream=None, raise_on_divergence=True) -> list:
        st = (SolveStats * self.n)()
        rc = load().kf_batch_run(self.h, st, _stream(stream))
        if rc != KF_ERR_DIVERGED or raise_on_divergence:
            check(rc)
        return [x.as_dict() for x in st]


KF_MESH_LIVE, KF_MESH_REGISTERED, KF_MESH_CANONICAL = 1, 2, 4


class FusionConfig(C.Structure):
    _fields_ = [("dims", C.c_int * 3), ("voxel_size", C.c_double), ("min3d", C.c_double * 3),
                ("K", C.c_double * 9), ("width", C.c_int), ("height", C.c_int),
                ("min_depth", C.c_double), ("max_depth", C.c_double), ("params", _Params),
                ("iterations", C.c_int), ("solver", C.c_int)]


class FrameResult(C.Structure):
    _fields_ = [("frame", C.c_int32), ("reserved", C.c_int32), ("solve", SolveStats),
                ("ntri", C.c_int64 * 3), ("mesh", C.POINTER(C.c_float) * 3), ("device_ms", C.c_double)]


class Fusion:
    """KillingFusion's state on the device; process_frame is one
    processNextFrame call through the C ABI."""

    def __init__(self, dims, voxel_size, origin, params: Params, K=None, width=640, height=480,
                 min_depth=0.05, max_depth=1.2, iterations=100, solver="fused"):
        from . import synth
        cfg = FusionConfig()
        cfg.dims = (C.c_int * 3)(*[int(d) for d in dims])
        cfg.voxel_size = float(voxel_size)
        cfg.min3d = (C.c_double * 3)(*[float(v) for v in origin])
        K = synth.K if K is None else np.asarray(K, dtype=np.float64)
        cfg.K = (C.c_double * 9)(*[float(v) for v in K.ravel()])
        cfg.width, cfg.height = int(width), int(height)
        cfg.min_depth, cfg.max_depth = float(min_depth), float(max_depth)
        cfg.params = params.c()
        cfg.iterations = int(iterations)
        cfg.solver = SOLVERS[solver]
        self.cfg = cfg
        self.params = params
        h = _vp()
        check(load().kf_fusion_create(C.byref(cfg), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().kf_fusion_destroy(self.h)
            self.h = None

    __del__ = close

    def process_frame(self, depth, meshes=KF_MESH_LIVE | KF_MESH_REGISTERED | KF_MESH_CANONICAL,
                      c2w=None, copy=True):
        """depth: numpy float32 [h, w] (host) or a CUDA tensor.  Returns a
        dict with the solve statistics and the requested meshes as float32
        [T, 3, 3] arrays (copies unless copy=False)."""
        if isinstance(depth, np.ndarray):
            d = np.ascontiguousarray(depth, dtype=np.float32)
            ptr = d.ctypes.data
        else:
            ptr = depth.data_ptr()
        res = FrameResult()
        pose = _d(np.asarray(c2w, dtype=np.float64).ravel()) if c2w is not None else None
        check(load().kf_fusion_process_frame(self.h, ptr, pose, int(meshes), C.byref(res), None))
        out = {"frame": res.frame, "solve": res.solve.as_dict(), "device_ms": res.device_ms,
               "ntri": list(res.ntri)}
        names = ("live", "registered", "canonical")
        for k in range(3):
            if meshes & (1 << k) and res.mesh[k]:
                n = res.ntri[k]
                a = np.ctypeslib.as_array(res.mesh[k], shape=(max(n, 1) * 9,))[: n * 9].reshape(n, 3, 3)
                out[names[k]] = a.copy() if copy else a
        return out

    def state(self):
        c, l, f = _vp(), _vp(), _vp()
        check(load().kf_fusion_state(self.h, C.byref(c), C.byref(l), C.byref(f)))
        return c.value, l.value, f.value

    def save(self, path):
        """Checkpoint: canonical SDF, psi and frame count to a state file."""
        check(load().kf_fusion_save(self.h, os.fsencode(path), None))

    def load(self, path):
        """Resume from a state file written by a pipeline of this configuration."""
        check(load().kf_fusion_load(self.h, os.fsencode(path), None))
