"""Build of the CUDA library (sm_103a) and the C++ host layer.

Produces, in-tree:

* ``killingfusion_gb300/_lib/libkillingfusion.so`` -- the C ABI of
  ``include/killingfusion.h`` (CUDA kernels + host entry points);
* ``killingfusion_gb300/_lib/libkf_host.so`` -- the C++ classes with the
  reference's names and call shapes (``csrc/host``), linked against the former;
* ``killingfusion_gb300/_lib/libkillingfusion_bc.so`` -- the same C ABI built
  with ``-DKF_BOUNDS_CHECK`` (every data-derived index of the hot-path
  kernels checked, see ``csrc/kf_bounds.cuh``), for tests.

One ``-gencode arch=compute_103a,code=sm_103a``; translation units are
compiled in parallel.  ``kf_exact.cu`` is compiled with ``-fmad=false``: its
float64 expressions must round like the reference's.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(CSRC, "host")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIB_DIR, "libkillingfusion.so")
HOST_LIB = os.path.join(LIB_DIR, "libkf_host.so")
LIB_BC = os.path.join(LIB_DIR, "libkillingfusion_bc.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# (source, extra flags)
CUDA_UNITS = [
    ("kf_core.cu", []),
    ("kf_exact.cu", ["-fmad=false"]),
    ("kf_fused.cu", []),
    ("kf_plain.cu", []),
    ("kf_mc.cu", []),
    ("kf_energy.cu", ["-fmad=false"]),
    ("kf_batch.cu", []),
    ("kf_fusion.cu", []),
    ("kf_state.cu", []),
]
HOST_UNITS = ["SDF.cpp", "DisplacementField.cpp", "DatasetReader.cpp", "KillingFusion.cpp", "png.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every translation unit that changed and link the libraries."""
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    nv = nvcc()
    # host code: no contracted multiply-add, so host-side float64 (the pose
    # inverse) rounds the same on x86-64 and aarch64
    common = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC] + ARCH
    hdrs = _headers()
    jobs = []
    objs = {LIB: [], LIB_BC: []}
    for lib, obj_dir, defs in ((LIB, OBJ_DIR, []), (LIB_BC, os.path.join(OBJ_DIR, "bc"), ["-DKF_BOUNDS_CHECK"])):
        os.makedirs(obj_dir, exist_ok=True)
        for src, extra in CUDA_UNITS:
            s = os.path.join(CSRC, src)
            if not os.path.exists(s):
                continue
            o = os.path.join(obj_dir, src.replace(".cu", ".o"))
            objs[lib].append(o)
            if force or _stale(o, [s] + hdrs):
                jobs.append([nv] + common + defs + extra + ["-Xptxas", "-v"] * verbose + ["-c", s, "-o", o])
    # the longest units first, so that they do not start last
    jobs.sort(key=lambda j: 0 if any(u in j[-3] for u in ("kf_batch", "kf_fused", "kf_exact")) else 1)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    for lib, o in objs.items():
        if force or _stale(lib, o):
            _run([nv, "-shared"] + ARCH + ["-o", lib] + o + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"])
    _build_host(force)
    return LIB


def _build_host(force: bool) -> None:
    srcs = [os.path.join(HOST, f) for f in HOST_UNITS if os.path.exists(os.path.join(HOST, f))]
    if not srcs:
        return
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")] + [LIB]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    if not (force or _stale(HOST_LIB, deps)):
        return
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-Wall", "-I", INCLUDE, "-I", HOST, "-o", HOST_LIB]
         + srcs + ["-L", LIB_DIR, "-lkillingfusion", "-Wl,-rpath,$ORIGIN"])


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
