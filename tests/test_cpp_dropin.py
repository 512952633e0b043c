"""The C++ drop-in types (include/orthotree_gpu.hpp) compile with g++ -std=c++20 against the C-ABI
library. Without a GPU the program checks that they fail loudly; with one it compares every query
with the CPU oracle."""
import os
import shutil
import subprocess

import pytest

import octree_gb300 as otg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_test.cpp")
ORACLE_DIR = os.path.join(ROOT, "oracle", "_build")


def _build(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ missing")
    if not os.path.exists(otg.LIB_PATH):
        pytest.skip("CUDA library not built")
    exe = str(tmp_path / "dropin_test")
    libdir = os.path.dirname(otg.LIB_PATH)
    cmd = ["g++", "-std=c++20", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", libdir, "-loctree_gb300", "-L", ORACLE_DIR, "-lotg_oracle",
           f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{ORACLE_DIR}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _run(exe):
    return subprocess.run([exe], capture_output=True, text=True, timeout=600)


def test_dropin_compiles_and_fails_loudly_without_device(tmp_path):
    if otg.device_count() > 0:
        pytest.skip("a GPU is present")
    r = _run(_build(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "no device" in r.stdout


@pytest.mark.gpu
def test_dropin_matches_oracle(tmp_path):
    r = _run(_build(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")
