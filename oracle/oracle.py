"""ctypes bindings for the FP64 oracle (TEST INFRASTRUCTURE ONLY).

``Oracle`` wraps ``oracle/_build/libkf_oracle.so`` (the C restatement);
``RefLib`` wraps ``oracle/_ref/libkf_ref.so`` (the reference's own sources
built against the project shims).  Both take numpy arrays in the oracle's
layouts: phi float64[nz,ny,nx], weights int64[nz,ny,nx], psi
float64[nz,ny,nx,3].

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs use
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import tempfile
from dataclasses import dataclass, asdict, replace

import numpy as np

from . import build as _build

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


@dataclass(frozen=True)
class Params:
    """The reference's config.h globals on the hot path (config.cpp:4-57)."""

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
    use_trust: bool = False

    @staticmethod
    def paper(voxel_size: float, trunc_voxels: float = 5.0) -> "Params":
        """Paper weights (alpha 0.1, omega_k 0.5, gamma 0.1, omega_s 0.2)."""
        t = voxel_size * trunc_voxels
        return Params(voxel_size=voxel_size, unknown_clip=t, max_surface=t, alpha=0.1,
                      omega_k=0.5, gamma_k=0.1, omega_s=0.2)

    def with_(self, **kw) -> "Params":
        return replace(self, **kw)


class _OrcParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "voxel_size", "unknown_clip", "max_surface", "epsilon", "delta_size", "alpha",
        "omega_k", "gamma_k", "omega_s", "threshold", "killing_clamp")] + [
        ("use_data", C.c_int), ("use_levelset", C.c_int), ("use_killing", C.c_int),
        ("use_trust", C.c_int)]

    @classmethod
    def of(cls, p: Params) -> "_OrcParams":
        d = asdict(p)
        return cls(**{k: (int(v) if isinstance(v, bool) else v) for k, v in d.items()})


def _dims(phi: np.ndarray) -> np.ndarray:
    nz, ny, nx = phi.shape[:3]
    return np.array([nx, ny, nz], dtype=np.int32)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Oracle:
    """FP64 C restatement of the reference hot path."""

    def __init__(self, path: str | None = None):
        path = path or _build.build_oracle()
        L = C.CDLL(path)
        self.L = L
        P = C.POINTER(_OrcParams)
        sig = {
            "orc_phi_sample": (C.c_double, [_dp, _i32p, P, _dp]),
            "orc_weight_sample": (C.c_double, [_ip, _i32p, _dp]),
            "orc_psi_sample": (None, [_dp, _i32p, _dp, _dp]),
            "orc_distance_gradient_at": (None, [_dp, _i32p, P, _dp, _dp]),
            "orc_distance_hessian_at": (None, [_dp, _i32p, P, _dp, _dp]),
            "orc_jacobian": (None, [_dp, _i32p, P, C.c_double, C.c_double, C.c_double, _dp]),
            "orc_killing_energy": (C.c_double, [_dp, _i32p, P, C.c_double, C.c_double, C.c_double]),
            "orc_killing_energy_gradient_fd": (None, [_dp, _i32p, P, C.c_int, C.c_int, C.c_int, _dp]),
            "orc_distance_gradient": (None, [_dp, _dp, _i32p, P, C.c_int, C.c_int, C.c_int, _dp]),
            "orc_distance_hessian": (None, [_dp, _dp, _i32p, P, C.c_int, C.c_int, C.c_int, _dp]),
            "orc_killing_gradient": (None, [_dp, _i32p, P, C.c_int, C.c_int, C.c_int, _dp]),
            "orc_energy_gradient": (None, [_dp, _dp, _dp, _i32p, P, C.c_int, C.c_int, C.c_int, _dp]),
            "orc_warped_distance": (C.c_double, [_dp, _dp, _i32p, P, C.c_int, C.c_int, C.c_int]),
            "orc_is_active": (C.c_int, [_dp, _dp, _i32p, P, C.c_int, C.c_int, C.c_int]),
            "orc_solve_jacobi": (C.c_int, [_dp, _dp, _dp, _i32p, P, C.c_int, C.c_int, C.c_void_p]),
            "orc_solve_pervoxel": (C.c_int, [_dp, _dp, _dp, _i32p, P, C.c_int, C.c_int, C.c_void_p]),
            "orc_integrate": (None, [_dp, _ip, _i32p, C.c_double, _dp, C.c_double, _dp, C.c_int,
                                     C.c_int, _dp, _dp, C.c_double, C.c_double]),
            "orc_update": (None, [_dp, _ip, _dp, _i32p, P]),
            "orc_invert4": (C.c_int, [_dp, _dp]),
            "orc_fuse": (None, [_dp, _ip, _dp, _ip, C.c_int64]),
            "orc_fuse_psi": (None, [_dp, _ip, _dp, _ip, _dp, _i32p, P]),
            "orc_mc_extract": (C.c_int64, [_dp, _i32p, P, C.c_void_p, C.c_int64]),
            "orc_mc_edge_mask": (C.c_int, [C.c_int]),
            "orc_mc_tri_row": (C.c_int, [C.c_int, _i32p]),
            "orc_project_energy": (C.c_double, [_dp, _dp, _dp, _u8p, _i32p, P]),
            "orc_project_energy_local": (C.c_double, [_dp, _dp, _dp, _u8p, _i32p, P, C.c_int,
                                                      C.c_int, C.c_int, C.c_int]),
            "orc_project_energy_grad": (None, [_dp, _dp, _dp, _u8p, _i32p, P, _dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args

    # -- samplers ---------------------------------------------------------
    def phi_sample(self, phi, p, P: Params):
        phi = _c(phi, np.float64)
        return self.L.orc_phi_sample(phi, _dims(phi), C.byref(_OrcParams.of(P)), _c(p, np.float64))

    def weight_sample(self, w, p):
        w = _c(w, np.int64)
        return self.L.orc_weight_sample(w, _dims(w), _c(p, np.float64))

    def psi_sample(self, psi, p):
        psi = _c(psi, np.float64)
        out = np.zeros(3)
        self.L.orc_psi_sample(psi, _dims(psi), _c(p, np.float64), out)
        return out

    def distance_gradient_at(self, phi, p, P):
        phi = _c(phi, np.float64)
        out = np.zeros(3)
        self.L.orc_distance_gradient_at(phi, _dims(phi), C.byref(_OrcParams.of(P)), _c(p, np.float64), out)
        return out

    def distance_hessian_at(self, phi, p, P):
        phi = _c(phi, np.float64)
        out = np.zeros(9)
        self.L.orc_distance_hessian_at(phi, _dims(phi), C.byref(_OrcParams.of(P)), _c(p, np.float64), out)
        return out.reshape(3, 3)

    def jacobian(self, psi, x, y, z, P):
        psi = _c(psi, np.float64)
        out = np.zeros(9)
        self.L.orc_jacobian(psi, _dims(psi), C.byref(_OrcParams.of(P)), x, y, z, out)
        return out.reshape(3, 3)

    def killing_energy(self, psi, x, y, z, P):
        psi = _c(psi, np.float64)
        return self.L.orc_killing_energy(psi, _dims(psi), C.byref(_OrcParams.of(P)), x, y, z)

    def killing_energy_gradient_fd(self, psi, x, y, z, P):
        psi = _c(psi, np.float64)
        out = np.zeros(3)
        self.L.orc_killing_energy_gradient_fd(psi, _dims(psi), C.byref(_OrcParams.of(P)), x, y, z, out)
        return out

    # -- per-voxel queries ------------------------------------------------
    def voxel_query(self, what, live, can, psi, xyz, P: Params):
        """what: 'grad' energy gradient, 'dgrad', 'hess', 'killing', 'warped', 'active'."""
        live = _c(live, np.float64)
        can = _c(can if can is not None else live, np.float64)
        psi = _c(psi, np.float64)
        n = _dims(live)
        pp = C.byref(_OrcParams.of(P))
        xyz = np.asarray(xyz, dtype=np.int64).reshape(-1, 3)
        width = {"grad": 3, "dgrad": 3, "hess": 9, "killing": 3, "warped": 1, "active": 1}[what]
        out = np.zeros((len(xyz), width))
        buf = np.zeros(9)
        for i, (x, y, z) in enumerate(xyz):
            x, y, z = int(x), int(y), int(z)
            if what == "grad":
                self.L.orc_energy_gradient(live, can, psi, n, pp, x, y, z, buf)
            elif what == "dgrad":
                self.L.orc_distance_gradient(live, psi, n, pp, x, y, z, buf)
            elif what == "hess":
                self.L.orc_distance_hessian(live, psi, n, pp, x, y, z, buf)
            elif what == "killing":
                self.L.orc_killing_gradient(psi, n, pp, x, y, z, buf)
            elif what == "warped":
                buf[0] = self.L.orc_warped_distance(live, psi, n, pp, x, y, z)
            else:
                buf[0] = self.L.orc_is_active(live, psi, n, pp, x, y, z)
            out[i] = buf[:width]
        return out

    def solve(self, live, can, psi, iters, P: Params, nthreads=0, active_counts=False):
        """Jacobi psi solve; returns (status, psi, [active counts])."""
        live = _c(live, np.float64)
        psi = np.array(psi, dtype=np.float64, order="C", copy=True)
        counts = np.zeros(max(iters, 1), dtype=np.int64)
        st = self.L.orc_solve_jacobi(live, _c(can, np.float64), psi, _dims(live),
                                     C.byref(_OrcParams.of(P)), iters, nthreads,
                                     counts.ctypes.data)
        return (st, psi, counts[:iters]) if active_counts else (st, psi)

    def solve_pervoxel(self, live, can, psi, max_iters, P: Params, colored=False):
        """The reference's default per-voxel schedule on one thread, in z, y, x
        order or colour by colour; returns (status, psi, (visited, steps,
        capped))."""
        live = _c(live, np.float64)
        psi = np.array(psi, dtype=np.float64, order="C", copy=True)
        counts = np.zeros(3, dtype=np.int64)
        st = self.L.orc_solve_pervoxel(live, _c(can, np.float64), psi, _dims(live),
                                       C.byref(_OrcParams.of(P)), max_iters, int(bool(colored)),
                                       counts.ctypes.data)
        return st, psi, tuple(int(c) for c in counts)

    def integrate(self, phi, w, voxel, min3, unknown_clip, depth, w2c, K, min_depth, max_depth):
        phi = np.array(phi, dtype=np.float64, order="C", copy=True)
        w = np.array(w, dtype=np.int64, order="C", copy=True)
        depth = _c(depth, np.float64)
        h, wd = depth.shape
        self.L.orc_integrate(phi, w, _dims(phi), voxel, _c(min3, np.float64), unknown_clip, depth,
                             wd, h, _c(w2c, np.float64).ravel(), _c(K, np.float64).ravel(),
                             min_depth, max_depth)
        return phi, w

    def invert4(self, m):
        out = np.zeros(16)
        if self.L.orc_invert4(_c(m, np.float64).ravel(), out) != 0:
            raise ValueError("singular pose")
        return out.reshape(4, 4)

    def update(self, phi, w, psi, P):
        phi = np.array(phi, dtype=np.float64, order="C", copy=True)
        w = np.array(w, dtype=np.int64, order="C", copy=True)
        self.L.orc_update(phi, w, _c(psi, np.float64), _dims(phi), C.byref(_OrcParams.of(P)))
        return phi, w

    def fuse(self, phi1, w1, phi2, w2):
        phi1 = np.array(phi1, dtype=np.float64, order="C", copy=True)
        w1 = np.array(w1, dtype=np.int64, order="C", copy=True)
        self.L.orc_fuse(phi1, w1, _c(phi2, np.float64), _c(w2, np.int64), phi1.size)
        return phi1, w1

    def fuse_psi(self, phi1, w1, phi2, w2, psi, P):
        phi1 = np.array(phi1, dtype=np.float64, order="C", copy=True)
        w1 = np.array(w1, dtype=np.int64, order="C", copy=True)
        self.L.orc_fuse_psi(phi1, w1, _c(phi2, np.float64), _c(w2, np.int64), _c(psi, np.float64),
                            _dims(phi1), C.byref(_OrcParams.of(P)))
        return phi1, w1

    def mesh(self, phi, P):
        """Triangle soup as float64[T,3,3] (SimpleMesh vertex convention)."""
        phi = _c(phi, np.float64)
        n = _dims(phi)
        pp = C.byref(_OrcParams.of(P))
        nt = self.L.orc_mc_extract(phi, n, pp, None, 0)
        out = np.zeros((max(nt, 1), 3, 3))
        self.L.orc_mc_extract(phi, n, pp, out.ctypes.data, nt)
        return out[:nt]

    def mc_tables(self):
        edges = np.array([self.L.orc_mc_edge_mask(c) for c in range(256)], dtype=np.int32)
        tris = np.zeros((256, 16), dtype=np.int32)
        row = np.zeros(16, dtype=np.int32)
        for c in range(256):
            self.L.orc_mc_tri_row(c, row)
            tris[c] = row
        return edges, tris

    # -- project energy ---------------------------------------------------
    def project_energy(self, live, can, psi, active, P):
        live = _c(live, np.float64)
        return self.L.orc_project_energy(live, _c(can, np.float64), _c(psi, np.float64),
                                         _c(active, np.uint8), _dims(live), C.byref(_OrcParams.of(P)))

    def project_energy_local(self, live, can, psi, active, xyz, radius, P):
        live = _c(live, np.float64)
        x, y, z = (int(v) for v in xyz)
        return self.L.orc_project_energy_local(live, _c(can, np.float64), _c(psi, np.float64),
                                               _c(active, np.uint8), _dims(live),
                                               C.byref(_OrcParams.of(P)), x, y, z, radius)

    def project_energy_grad(self, live, can, psi, active, P):
        live = _c(live, np.float64)
        g = np.zeros(live.shape + (3,))
        self.L.orc_project_energy_grad(live, _c(can, np.float64), _c(psi, np.float64),
                                       _c(active, np.uint8), _dims(live),
                                       C.byref(_OrcParams.of(P)), g)
        return g


def ref_env(P: Params, iterations: int) -> dict:
    """Environment that configures oracle/_ref's config globals."""
    return {
        "KF_REF_VOXEL_SIZE": repr(P.voxel_size), "KF_REF_UNKNOWN_CLIP": repr(P.unknown_clip),
        "KF_REF_MAX_SURFACE": repr(P.max_surface), "KF_REF_EPSILON": repr(P.epsilon),
        "KF_REF_DELTA_SIZE": repr(P.delta_size), "KF_REF_ALPHA": repr(P.alpha),
        "KF_REF_OMEGA_K": repr(P.omega_k), "KF_REF_GAMMA_K": repr(P.gamma_k),
        "KF_REF_OMEGA_S": repr(P.omega_s), "KF_REF_THRESHOLD": repr(P.threshold),
        "KF_REF_USE_DATA": str(int(P.use_data)), "KF_REF_USE_LEVELSET": str(int(P.use_levelset)),
        "KF_REF_USE_KILLING": str(int(P.use_killing)), "KF_REF_ITERATIONS": str(int(iterations)),
        "KF_REF_JACOBI": "1", "KF_REF_TRUST": str(int(P.use_trust)),
    }


class RefLib:
    """The reference's own code (oracle/_ref).  Its config globals are fixed
    when the library loads, so each (params, iterations) pair gets a private
    copy of the shared object."""

    _cache: dict = {}
    _tmp = None

    def __init__(self, P: Params, iterations: int = 1):
        if P.killing_clamp != 0.1:
            raise ValueError("the reference hard-codes the Killing clamp at 0.1")
        path = _build.build_ref()
        if path is None:
            raise FileNotFoundError("reference checkout absent")
        key = (P, iterations)
        if key not in RefLib._cache:
            if RefLib._tmp is None:
                RefLib._tmp = tempfile.mkdtemp(prefix="kf_ref_")
            copy = os.path.join(RefLib._tmp, "libkf_ref_%d.so" % len(RefLib._cache))
            shutil.copyfile(path, copy)
            old = {}
            for k, v in ref_env(P, iterations).items():
                old[k] = os.environ.get(k)
                os.environ[k] = v
            try:
                L = C.CDLL(copy, mode=C.RTLD_LOCAL)
            finally:
                for k, v in old.items():
                    if v is None:
                        os.environ.pop(k, None)
                    else:
                        os.environ[k] = v
            self._sig(L)
            RefLib._cache[key] = L
        self.L = RefLib._cache[key]
        self.P = P

    @staticmethod
    def _sig(L):
        sig = {
            "ref_grid_size": (C.c_int, [_dp, C.c_double, _i32p]),
            "ref_phi_sample": (None, [_dp, _i32p, _dp, C.c_int, _dp]),
            "ref_weight_sample": (None, [_ip, _i32p, _dp, C.c_int, _dp]),
            "ref_psi_sample": (None, [_dp, _i32p, _dp, C.c_int, _dp]),
            "ref_distance_gradient_at": (None, [_dp, _i32p, _dp, C.c_int, _dp]),
            "ref_distance_hessian_at": (None, [_dp, _i32p, _dp, C.c_int, _dp]),
            "ref_voxel_query": (None, [C.c_int, _dp, C.c_void_p, _dp, _i32p, _i32p, C.c_int, _dp]),
            "ref_solve": (C.c_int, [_dp, _dp, _dp, _i32p]),
            "ref_jacobian": (None, [_dp, _i32p, C.c_double, C.c_double, C.c_double, _dp]),
            "ref_killing_energy": (C.c_double, [_dp, _i32p, C.c_double, C.c_double, C.c_double]),
            "ref_killing_energy_gradient_fd": (None, [_dp, _i32p, C.c_int, C.c_int, C.c_int, _dp]),
            "ref_integrate": (None, [_dp, _ip, _i32p, C.c_double, _dp, C.c_double, _dp, C.c_int,
                                     C.c_int, _dp, _dp, C.c_double, C.c_double]),
            "ref_update": (None, [_dp, _ip, _dp, _i32p]),
            "ref_fuse": (None, [_dp, _ip, _dp, _ip, _i32p]),
            "ref_fuse_psi": (None, [_dp, _ip, _dp, _ip, _dp, _i32p]),
            "ref_mesh": (C.c_int64, [_dp, _i32p, C.c_void_p, C.c_int64]),
            "ref_two_spheres": (None, [C.c_double, C.c_double, _i32p, _dp, _ip, _dp, _ip]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args

    def grid_size(self, bound, voxel):
        out = np.zeros(3, dtype=np.int32)
        self.L.ref_grid_size(_c(bound, np.float64), voxel, out)
        return out

    def phi_sample(self, phi, pts):
        phi = _c(phi, np.float64)
        pts = _c(pts, np.float64).reshape(-1, 3)
        out = np.zeros(len(pts))
        self.L.ref_phi_sample(phi, _dims(phi), pts, len(pts), out)
        return out

    def weight_sample(self, w, pts):
        w = _c(w, np.int64)
        pts = _c(pts, np.float64).reshape(-1, 3)
        out = np.zeros(len(pts))
        self.L.ref_weight_sample(w, _dims(w), pts, len(pts), out)
        return out

    def psi_sample(self, psi, pts):
        psi = _c(psi, np.float64)
        pts = _c(pts, np.float64).reshape(-1, 3)
        out = np.zeros((len(pts), 3))
        self.L.ref_psi_sample(psi, _dims(psi), pts, len(pts), out)
        return out

    def distance_gradient_at(self, phi, pts):
        phi = _c(phi, np.float64)
        pts = _c(pts, np.float64).reshape(-1, 3)
        out = np.zeros((len(pts), 3))
        self.L.ref_distance_gradient_at(phi, _dims(phi), pts, len(pts), out)
        return out

    def distance_hessian_at(self, phi, pts):
        phi = _c(phi, np.float64)
        pts = _c(pts, np.float64).reshape(-1, 3)
        out = np.zeros((len(pts), 3, 3))
        self.L.ref_distance_hessian_at(phi, _dims(phi), pts, len(pts), out)
        return out

    def voxel_query(self, what, live, can, psi, xyz):
        code = {"grad": 0, "dgrad": 1, "hess": 2, "killing": 3, "warped": 4, "active": 5}[what]
        width = {"grad": 3, "dgrad": 3, "hess": 9, "killing": 3, "warped": 1, "active": 1}[what]
        live = _c(live, np.float64)
        can_arr = _c(can, np.float64) if can is not None else None
        xyz = _c(xyz, np.int32).reshape(-1, 3)
        out = np.zeros((len(xyz), width))
        self.L.ref_voxel_query(code, live, can_arr.ctypes.data if can_arr is not None else None,
                               _c(psi, np.float64), _dims(live), xyz, len(xyz), out)
        return out

    def solve(self, live, can, psi):
        psi = np.array(psi, dtype=np.float64, order="C", copy=True)
        live = _c(live, np.float64)
        st = self.L.ref_solve(live, _c(can, np.float64), psi, _dims(live))
        return st, psi

    def jacobian(self, psi, x, y, z):
        psi = _c(psi, np.float64)
        out = np.zeros(9)
        self.L.ref_jacobian(psi, _dims(psi), x, y, z, out)
        return out.reshape(3, 3)

    def killing_energy(self, psi, x, y, z):
        psi = _c(psi, np.float64)
        return self.L.ref_killing_energy(psi, _dims(psi), x, y, z)

    def killing_energy_gradient_fd(self, psi, x, y, z):
        psi = _c(psi, np.float64)
        out = np.zeros(3)
        self.L.ref_killing_energy_gradient_fd(psi, _dims(psi), x, y, z, out)
        return out

    def integrate(self, phi, w, voxel, min3, unknown_clip, depth, c2w, K, min_depth, max_depth):
        phi = np.array(phi, dtype=np.float64, order="C", copy=True)
        w = np.array(w, dtype=np.int64, order="C", copy=True)
        depth = _c(depth, np.float64)
        h, wd = depth.shape
        self.L.ref_integrate(phi, w, _dims(phi), voxel, _c(min3, np.float64), unknown_clip, depth,
                             wd, h, _c(c2w, np.float64).ravel(), _c(K, np.float64).ravel(),
                             min_depth, max_depth)
        return phi, w

    def update(self, phi, w, psi):
        phi = np.array(phi, dtype=np.float64, order="C", copy=True)
        w = np.array(w, dtype=np.int64, order="C", copy=True)
        self.L.ref_update(phi, w, _c(psi, np.float64), _dims(phi))
        return phi, w

    def fuse(self, phi1, w1, phi2, w2):
        phi1 = np.array(phi1, dtype=np.float64, order="C", copy=True)
        w1 = np.array(w1, dtype=np.int64, order="C", copy=True)
        self.L.ref_fuse(phi1, w1, _c(phi2, np.float64), _c(w2, np.int64), _dims(phi1))
        return phi1, w1

    def fuse_psi(self, phi1, w1, phi2, w2, psi):
        phi1 = np.array(phi1, dtype=np.float64, order="C", copy=True)
        w1 = np.array(w1, dtype=np.int64, order="C", copy=True)
        self.L.ref_fuse_psi(phi1, w1, _c(phi2, np.float64), _c(w2, np.int64), _c(psi, np.float64),
                            _dims(phi1))
        return phi1, w1

    def mesh(self, phi):
        phi = _c(phi, np.float64)
        n = _dims(phi)
        nt = self.L.ref_mesh(phi, n, None, 0)
        out = np.zeros((max(nt, 1), 3, 3))
        self.L.ref_mesh(phi, n, out.ctypes.data, nt)
        return out[:nt]

    def two_spheres(self, voxel, unknown_clip):
        n = np.zeros(3, dtype=np.int32)
        bufs = [np.zeros(4096), np.zeros(4096, dtype=np.int64), np.zeros(4096),
                np.zeros(4096, dtype=np.int64)]
        self.L.ref_two_spheres(voxel, unknown_clip, n, *bufs)
        N = int(np.prod(n))
        shp = (int(n[2]), int(n[1]), int(n[0]))
        return [b[:N].reshape(shp).copy() for b in bufs]
