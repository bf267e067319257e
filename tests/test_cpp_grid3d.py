"""The reference's 3D containers for C++ callers (include/MACGrid3D_gb300.hpp).

CPU: the header compiles with g++ (-Wall -Wextra, no warning) and links
against libfs2d.so; every host method, run on exact rational inputs, equals
the oracle restatement (oracle/restate/fs3d_oracle.c) bit for bit.
GPU: the fs3d_device:: wrappers (the C ABI of include/fs3d.h) on the same
inputs equal the host methods (tests/cpp/grid3d_api_test.cpp).
CPU: a plain C11 program over include/fs3d.h (tests/cpp/fs3d_args_test.c)
links and sees bad arguments refused before any device work.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle3d

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "grid3d_api_test.cpp")
LIBDIR = os.path.join(ROOT, "fluid-sim_gb300")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
SX, SY, SZ, NPTS = 9, 7, 5, 64
R = oracle3d.restated


def build(tmp_path, gpu=False):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    if not os.path.exists(os.path.join(LIBDIR, "libfs2d.so")):
        pytest.skip("libfs2d.so not built")
    exe = str(tmp_path / ("grid3d_api_test_gpu" if gpu else "grid3d_api_test"))
    # no contraction into FMA on any host, as the oracle is built
    cmd = [gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           SRC, "-o", exe, "-L", LIBDIR, "-lfs2d", "-Wl,-rpath," + LIBDIR]
    if gpu:
        cmd[1:1] = ["-DGRID3D_TEST_GPU", "-I", os.path.join(CUDA, "include")]
        cmd += ["-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "warning" not in r.stderr, r.stderr
    return exe


def value(e, salt):
    """The program's exact test values."""
    e = np.asarray(e, dtype=np.int64)
    return ((e * 37 + salt * 11) % 101 - 50).astype(np.float64) / 16.0


def points():
    e = np.arange(NPTS, dtype=np.int64)
    return np.stack([((e * 13) % 97) / 8.0 - 1.0, ((e * 29) % 89) / 8.0 - 1.0, ((e * 7) % 61) / 8.0 - 1.0],
                    axis=1).astype(np.float64)


def expected():
    dims, size = (SX, SY, SZ), (SX, SY, SZ)
    n = SX * SY * SZ
    u = value(np.arange((SX + 1) * SY * SZ), 1)
    v = value(np.arange(SX * (SY + 1) * SZ), 2)
    w = value(np.arange(SX * SY * (SZ + 1)), 3)
    a, b = value(np.arange(n), 4), value(np.arange(n), 5)
    pts = points()
    return {
        "add": R.add(a, b, dims),
        "sma": R.set_multiply_add(a, 0.375, b, dims),
        "dot": np.array([R.inner_product(a, b, dims)]),
        "norm": np.array([R.infinite_norm(a, dims)]),
        "tricubic": R.tricubic(a, dims, pts),
        "vel": R.mac_vel(u, v, w, size).ravel(),
        "velu": R.mac_face_vel(u, v, w, size, "u").ravel(),
        "velv": R.mac_face_vel(u, v, w, size, "v").ravel(),
        "velw": R.mac_face_vel(u, v, w, size, "w").ravel(),
        "div": R.mac_vel_div(u, v, w, size),
        "interp": R.mac_vel_interp(u, v, w, size, "uvw", pts).ravel(),
    }


def test_host_methods_match_oracle(tmp_path):
    exe = build(tmp_path)
    r = subprocess.run([exe, "host"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    got = {}
    for line in r.stdout.splitlines():
        name, *vals = line.split()
        got[name] = np.array([float.fromhex(x) for x in vals])
    want = expected()
    assert sorted(got) == sorted(want)
    for name, w in want.items():
        assert np.array_equal(got[name].view(np.uint64), np.asarray(w, dtype=np.float64).view(np.uint64)), name
    # the inputs reach both branches of the outside test and the clamp to 0
    assert (got["tricubic"] == 0).sum() > 3 and (got["tricubic"] > 0).sum() > 3


@pytest.mark.gpu
def test_device_wrappers_match_host_methods(tmp_path):
    if not os.path.exists(os.path.join(CUDA, "include", "cuda_runtime.h")):
        pytest.skip("CUDA runtime headers not found")
    exe = build(tmp_path, gpu=True)
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr


C_SRC = os.path.join(ROOT, "tests", "cpp", "fs3d_args_test.c")


def test_c_program_checks_arguments_without_a_device(tmp_path):
    """include/fs3d.h compiles as C11 (no warnings), links, and refuses bad
    arguments before any device work: the program runs here without a GPU."""
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    if not os.path.exists(os.path.join(LIBDIR, "libfs2d.so")):
        pytest.skip("libfs2d.so not built")
    exe = str(tmp_path / "fs3d_args_test")
    r = subprocess.run([gcc, "-std=c11", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), C_SRC, "-o",
                        exe, "-L", LIBDIR, "-lfs2d", "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0 and "warning" not in r.stderr, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
