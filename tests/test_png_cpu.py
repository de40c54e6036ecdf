"""The PNG reader of the C++ layer (csrc/host/png.cpp: DEFLATE and scanline
filters written from RFC 1951 and the PNG specification) on images the tests
write themselves: every filter type, stored/fixed/dynamic blocks, 8/16-bit,
grey and RGB; malformed files fail cleanly."""
import os
import subprocess

import numpy as np
import pytest

import pngio

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def decoder(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("png") / "png_driver")
    host = os.path.join(ROOT, "killingfusion_gb300", "csrc", "host")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", host,
                    os.path.join(HERE, "cpp", "png_driver.cpp"), os.path.join(host, "png.cpp"), "-o", exe],
                   check=True)

    def run(path, out):
        r = subprocess.run([exe, str(path), str(out)], capture_output=True, text=True, timeout=60)
        return r

    return run


@pytest.mark.parametrize("kind", ["depth16", "mask8", "rgb8", "rgb16"])
@pytest.mark.parametrize("level", [0, 1, 9])
def test_roundtrip(decoder, tmp_path, kind, level):
    rng = np.random.default_rng([ord(c) for c in kind] + [level])
    h, w = 37, 53
    if kind == "depth16":
        # smooth depth in millimetres with holes, like a Kinect frame
        yy, xx = np.mgrid[0:h, 0:w]
        img = (800 + 3 * xx + 2 * yy + rng.integers(0, 5, (h, w))).astype(np.uint16)
        img[rng.random((h, w)) < 0.2] = 0
    elif kind == "mask8":
        img = (rng.random((h, w)) < 0.5).astype(np.uint8) * 255
    elif kind == "rgb8":
        img = rng.integers(0, 256, (h, w, 3)).astype(np.uint8)
    else:
        img = rng.integers(0, 65536, (h, w, 3)).astype(np.uint16)
    p = tmp_path / "a.png"
    pngio.write(p, img, level=level)
    r = decoder(p, tmp_path / "a.raw")
    assert r.returncode == 0, r.stderr
    ww, hh, ch, bd = (int(v) for v in r.stdout.split())
    assert (ww, hh) == (w, h) and ch == (1 if img.ndim == 2 else 3)
    assert bd == (16 if img.dtype == np.uint16 else 8)
    got = np.fromfile(tmp_path / "a.raw", np.uint16).reshape(img.shape)
    np.testing.assert_array_equal(got, img.astype(np.uint16))


def test_long_runs_and_far_matches(decoder, tmp_path):
    """Large, repetitive image: long matches, distances far back."""
    img = np.tile(np.arange(640, dtype=np.uint16) * 7, (480, 1))
    img[::37] = 0
    p = tmp_path / "b.png"
    pngio.write(p, img, filters=[2], level=9)
    r = decoder(p, tmp_path / "b.raw")
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(np.fromfile(tmp_path / "b.raw", np.uint16).reshape(img.shape), img)


def test_malformed_inputs_fail_cleanly(decoder, tmp_path):
    good = pngio.encode(np.zeros((4, 4), np.uint8))
    for name, data in [("sig", b"not a png file"), ("trunc", good[:40]),
                       ("badzlib", good[:41] + b"\x00\x00" + good[43:])]:
        p = tmp_path / (name + ".png")
        p.write_bytes(data)
        r = decoder(p, tmp_path / "x.raw")
        assert r.returncode == 1 and "png:" in r.stderr, (name, r.stderr)
