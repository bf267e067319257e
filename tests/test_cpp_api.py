"""The reference's C++ API over the C ABI (include/FluidSim2D_gb300.hpp).

CPU: the header compiles with g++ against the reference's usage and links
against libfs2d.so.  GPU: the program runs a dam break through runFrame and
through the stage methods one by one (bit-identical host mirrors), in both
modes, then fills the reference's perfCounter (32 frames) and checks its
perf.csv against the library's.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "fluidsim2d_api_test.cpp")
LIBDIR = os.path.join(ROOT, "fluid-sim_gb300")


def build(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    if not os.path.exists(os.path.join(LIBDIR, "libfs2d.so")):
        pytest.skip("libfs2d.so not built")
    exe = str(tmp_path / "fluidsim2d_api_test")
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", LIBDIR, "-lfs2d", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "warning" not in r.stderr, r.stderr
    return exe


def test_cpp_api_builds(tmp_path):
    build(tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["sl", "pic"])
def test_cpp_api_runs(tmp_path, mode):
    exe = build(tmp_path)
    r = subprocess.run([exe, mode, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr


C_SRC = os.path.join(ROOT, "tests", "cpp", "capi_rollout_batch_test.c")


def build_c(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    if not os.path.exists(os.path.join(LIBDIR, "libfs2d.so")):
        pytest.skip("libfs2d.so not built")
    exe = str(tmp_path / "capi_rollout_batch_test")
    cmd = [gcc, "-std=c11", "-D_DEFAULT_SOURCE", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           C_SRC, "-o", exe, "-L", LIBDIR, "-lfs2d", "-Wl,-rpath," + LIBDIR, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "warning" not in r.stderr, r.stderr
    return exe


def test_c_abi_program_builds(tmp_path):
    """fs2d.h compiles as C11; the rollout, transfer and batch entry points link."""
    build_c(tmp_path)


@pytest.mark.gpu
def test_c_abi_rollout_and_batch_run(tmp_path):
    exe = build_c(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr


EXT_SNIPPET = r"""
#include "FluidSim2D_gb300.hpp"
// the extensions beyond the reference's API, as a caller writes them
void use(FluidSim2D& sim) {
    sim.setVolumeCorrection(0.05);
    fs2d_reseed_stats r = sim.reseed(4, 8, 1u);
    long long e = -1;
    double c = sim.cfl(&e);
    sim.saveCheckpoint("state.fs2d");
    sim.loadCheckpoint("state.fs2d");
    (void)r;
    (void)c;
}
"""


def test_cpp_api_extensions_compile(tmp_path):
    """Reseeding, volume correction, the CFL check and checkpoints through
    the C++ mirror compile without warnings (they run in the GPU tests of
    the C ABI they wrap)."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "ext.cpp"
    src.write_text(EXT_SNIPPET)
    r = subprocess.run([gxx, "-std=c++17", "-Wall", "-Wextra", "-c", "-I", os.path.join(ROOT, "include"), str(src),
                        "-o", str(tmp_path / "ext.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "warning" not in r.stderr, r.stderr
