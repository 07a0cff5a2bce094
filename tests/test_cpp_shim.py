"""The header-only C++ drop-in (include/watercube/Fluid.hpp) compiles against the C ABI and,
on a GPU, runs the reference's usage pattern (create, chained setters, setup, per-frame
update)."""
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent


def build_demo(tmp_path, wclib):
    exe = tmp_path / "fluid_shim_demo"
    lib_dir = REPO / "watercube_gb300"
    cmd = ["g++", "-std=c++17", "-O1", f"-I{REPO / 'include'}", str(REPO / "tests" / "cpp" / "fluid_shim_demo.cpp"),
           f"-L{lib_dir}", "-lwatercube", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles(tmp_path, wclib):
    assert build_demo(tmp_path, wclib).exists()


@pytest.mark.gpu
def test_shim_runs_reference_usage(tmp_path, wclib, gpu):
    exe = build_demo(tmp_path, wclib)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok 20000 30")
