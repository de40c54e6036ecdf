"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

Two products:

* ``oracle/_build/libkf_oracle.so`` -- the FP64 C restatement
  (``oracle/kf_oracle.c``).  Built everywhere, including the GPU host, by
  ``__graft_entry__.build()``.
* ``oracle/_ref/libkf_ref.so`` -- the reference's own hot-path translation
  units (``KillingFusion/src/SDF.cpp``, ``DisplacementField.cpp``,
  ``KillingFusion.cpp``), compiled unmodified where they lie in the reference
  checkout, against the project's Eigen/OpenCV shims (``oracle/ref/shim``), a
  config that reads its values from the environment (``oracle/ref/ref_config.cpp``),
  a DatasetReader stub and a C harness (``oracle/ref/ref_harness.cpp``).  Built
  only where the reference checkout exists; it is the pin for the restatement.

Both use ``-ffp-contract=off`` so that no multiply-add is fused and the two
agree bit for bit on the same inputs, on x86-64 and on aarch64 alike.

The reference checkout is found at ``--ref REF_ROOT``, else at the path in the
environment variable ``KF_REFERENCE_ROOT``, else at ``/root/reference``.

Usage: ``python oracle/build.py [--ref REF_ROOT]``.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libkf_oracle.so")
REF_SO = os.path.join(REF_DIR, "libkf_ref.so")
FALLBACK_REF_ROOT = "/root/reference"


def default_ref_root() -> str:
    """The reference checkout: $KF_REFERENCE_ROOT, else the fallback path."""
    return os.environ.get("KF_REFERENCE_ROOT") or FALLBACK_REF_ROOT


COMMON = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    """Compile the FP64 restatement into oracle/_build/libkf_oracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, "kf_oracle.c"), os.path.join(HERE, "kf_oracle.h")]
    if force or _stale(ORACLE_SO, srcs):
        _run(["gcc", "-std=c11"] + COMMON + ["-shared", "-o", ORACLE_SO, srcs[0], "-lm"])
    return ORACLE_SO


def reference_available(ref_root: str | None = None) -> bool:
    ref_root = ref_root or default_ref_root()
    return os.path.isfile(os.path.join(ref_root, "KillingFusion", "src", "SDF.cpp"))


def build_ref(ref_root: str | None = None, force: bool = False) -> str | None:
    """Compile the reference's hot-path sources into oracle/_ref/libkf_ref.so.

    Returns the library path, or None when the reference checkout is absent.
    """
    ref_root = ref_root or default_ref_root()
    if not reference_available(ref_root):
        return None
    kf = os.path.join(ref_root, "KillingFusion")
    obj_dir = os.path.join(REF_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    flags = ["g++", "-std=c++14"] + COMMON + [
        "-DNDEBUG",
        '-DOUTPUT_DIR="/tmp/kf_ref_out/"', '-DDATA_DIR="/tmp/"', '-DPROJECT_DIR="/tmp/"',
        "-I", os.path.join(HERE, "ref", "shim"), "-I", os.path.join(kf, "include"),
        "-w",
    ]
    units = [os.path.join(kf, "src", f) for f in ("SDF.cpp", "DisplacementField.cpp", "KillingFusion.cpp")]
    units += [os.path.join(HERE, "ref", f) for f in ("ref_config.cpp", "ref_dataset.cpp", "ref_harness.cpp")]
    deps = [os.path.join(HERE, "ref", "shim", "Eigen", "Eigen"),
            os.path.join(HERE, "ref", "shim", "opencv2", "opencv.hpp")]
    objs = []
    jobs = []
    for u in units:
        o = os.path.join(obj_dir, os.path.splitext(os.path.basename(u))[0] + ".o")
        objs.append(o)
        if force or _stale(o, [u] + deps):
            jobs.append(flags + ["-c", u, "-o", o])
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        list(ex.map(_run, jobs))
    if force or _stale(REF_SO, objs):
        _run(["g++", "-shared", "-fopenmp", "-o", REF_SO] + objs)
    return REF_SO


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--ref", default=None, help="reference checkout root (default: $KF_REFERENCE_ROOT, "
                    "else %s)" % FALLBACK_REF_ROOT)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    print(build_oracle(a.force))
    r = build_ref(a.ref, a.force)
    print(r if r else "reference checkout absent: oracle/_ref not built")


if __name__ == "__main__":
    sys.exit(main())
