"""Host-side checks of the C ABI library that need no GPU: it loads, it
exports every function include/killingfusion.h declares, and its host-side
tables and parameter presets are the reference's."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(kf_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def capi():
    from killingfusion_gb300 import _build, capi
    if not os.path.exists(_build.LIB):
        _build.build()
    return capi


def test_library_exports_every_declared_symbol(capi):
    L = C.CDLL(capi.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the ctypes signature table covers the whole header
    assert set(names) <= set(capi.SIGNATURES), sorted(set(names) - set(capi.SIGNATURES))


def test_version_and_params_presets(capi):
    L = capi.load()
    assert L.kf_version() == 2  # KF_ABI_VERSION: kf_batch_autotune reports a kf_batch_shape
    p = capi._Params()
    L.kf_params_reference(C.byref(p))
    assert (p.voxel_size, p.alpha, p.omega_k, p.gamma_k, p.omega_s) == (0.012, 0.025, 0.04, 0.0, 0.1)
    assert (p.unknown_clip, p.max_surface, p.delta_size, p.epsilon) == (0.048, 0.048, 0.05, 1e-5)
    assert p.killing_clamp == 0.1 and p.early_exit == 0 and p.use_trust == 0
    L.kf_params_paper(C.byref(p), 0.004, 5.0)
    assert (p.alpha, p.omega_k, p.gamma_k, p.omega_s) == (0.1, 0.5, 0.1, 0.2)
    assert abs(p.unknown_clip - 0.02) < 1e-15


def test_params_struct_matches_header(capi):
    """The ctypes mirror of kf_params has the header's fields, in order and
    with the same C types."""
    src = open(os.path.join(ROOT, "include", "killingfusion.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct kf_params \{(.*?)\} kf_params;", src, flags=re.S).group(1)
    fields = []
    for ctype, names in re.findall(r"(double|int)\s+([^;]+);", body):
        fields += [(n.strip(), ctype) for n in names.split(",")]
    mirror = [(n, "double" if t is C.c_double else "int") for n, t in capi._Params._fields_]
    assert mirror == fields
    # the Python dataclass carries every field
    assert set(capi.Params.__dataclass_fields__) == {n for n, _ in fields}


def test_mc_table_matches_oracle(capi, oracle):
    edges, tris = oracle.mc_tables()
    for c in range(256):
        em, row = capi.mc_case(c)
        assert em == edges[c]
        assert row == list(tris[c])


def test_invalid_arguments_fail_cleanly(capi):
    """Argument checks run on the host before any device call."""
    L = capi.load()
    h = C.c_void_p()
    p = capi.Params().c()
    assert L.kf_grid_create((C.c_int * 3)(0, 4, 4), 0.01, None, 0.05, C.byref(p), C.byref(h)) == capi.KF_ERR_INVALID
    assert "dims" in L.kf_last_error().decode()
    assert L.kf_field_create((C.c_int * 3)(4, 4, 4), 7, C.byref(h)) == capi.KF_ERR_INVALID
    # voxel indices are 32-bit: grids of 2^31 voxels or more are refused
    for dims in ((1291, 1291, 1291), (65536, 65536, 1), (2 ** 31 - 1, 2, 1)):
        assert L.kf_grid_create((C.c_int * 3)(*dims), 0.01, None, 0.05, C.byref(p), C.byref(h)) == capi.KF_ERR_INVALID
        assert "2^31" in L.kf_last_error().decode()
        assert L.kf_field_create((C.c_int * 3)(*dims), capi.KF_F32, C.byref(h)) == capi.KF_ERR_INVALID
    assert L.kf_mc_case(256, None, None) == capi.KF_ERR_INVALID
    bad = capi.Params(delta_size=0.5).c()
    assert L.kf_grid_create((C.c_int * 3)(4, 4, 4), 0.01, None, 0.05, C.byref(bad), C.byref(h)) == capi.KF_ERR_INVALID
    assert L.kf_psi_solve(None, None, None, C.byref(p), 1, 0, None, None) == capi.KF_ERR_INVALID


def test_host_classes_compile_and_link(capi, tmp_path):
    """The C++ class layer (SDF, DisplacementField, KillingFusion,
    DatasetReader, SimpleMesh) builds and the test driver links against it;
    nothing is run (that needs a GPU)."""
    import subprocess
    from killingfusion_gb300 import _build
    _build.build()
    assert os.path.exists(_build.HOST_LIB)
    lib = os.path.dirname(_build.HOST_LIB)
    exe = str(tmp_path / "host_driver")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "killingfusion_gb300", "csrc", "host"),
                    os.path.join(ROOT, "tests", "cpp", "host_driver.cpp"), "-L", lib, "-lkf_host",
                    "-lkillingfusion", "-Wl,-rpath," + lib, "-o", exe], check=True)
    host = C.CDLL(_build.HOST_LIB)
    assert host is not None


def test_dataset_writer_and_bounds(tmp_path):
    """synth.write_dataset writes the layout the C++ DatasetReader reads, and
    the frustum bounds follow KillingFusion::computeBounds."""
    from killingfusion_gb300 import synth
    K = np.array([[52.5, 0.0, 31.5], [0.0, 52.5, 23.5], [0.0, 0.0, 1.0]])
    frames = [np.full((48, 64), 0.4, np.float32), np.zeros((48, 64), np.float32)]
    synth.write_dataset(str(tmp_path), frames, K, 0.3, 0.5)
    assert open(tmp_path / "meta.txt").read().split() == ["64", "48", "2", "0.3", "0.5"]
    np.testing.assert_array_equal(np.loadtxt(tmp_path / "intrinsics.txt").reshape(3, 3), K)
    np.testing.assert_array_equal(np.fromfile(tmp_path / "depth_000000.f32", np.float32).reshape(48, 64),
                                  frames[0])
    lo, hi = synth.frustum_bounds(K, 64, 48, 0.3, 0.5)
    np.testing.assert_allclose(lo, [-0.3, -23.5 / 52.5 * 0.5, 0.3], rtol=1e-15)
    np.testing.assert_allclose(hi, [0.3, 23.5 / 52.5 * 0.5, 0.5], rtol=1e-15)
    assert synth.grid_from_bounds(lo, hi, 0.008) == (76, 56, 26)


def test_batch_shape_struct_matches_header(capi):
    """The ctypes mirror of kf_batch_shape has the header's fields in order."""
    src = open(os.path.join(ROOT, "include", "killingfusion.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct kf_batch_shape \{(.*?)\} kf_batch_shape;", src, flags=re.S).group(1)
    fields = re.findall(r"(int|double)\s+(\w+);", body)
    ctypes_of = {"int": C.c_int, "double": C.c_double}
    assert [(n, ctypes_of[t]) for t, n in fields] == list(capi.BatchShape._fields_)


def test_wait_limit_setting(capi):
    """kf_set_wait_limit keeps values in [0, 60] s and returns the previous one
    (host-side only: no kernel runs)."""
    prev = capi.set_wait_limit(0.25)
    assert capi.set_wait_limit(prev) == 0.25
    assert capi.load().kf_set_wait_limit(-1.0) == -1.0
    assert capi.load().kf_set_wait_limit(61.0) == -1.0
    assert capi.set_wait_limit(prev) == prev
