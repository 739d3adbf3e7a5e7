"""The reference's own unit tests (unit-test/*.cpp) restated against the b2World facade.

The C++ program tests/cpp/reference_unit_tests.cpp is compiled against the facade headers and
linked with libb2g.so. Without a GPU only the host-side checks run (polygon mass data, sweep
transform); with a GPU the stepping checks run too (hello world pose, joint reaction forces,
BeginContact delivery).
"""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "box2d-optimized_gb300"
SRC = ROOT / "tests" / "cpp" / "reference_unit_tests.cpp"


def _build(tmp_path):
    exe = tmp_path / "reference_unit_tests"
    lib_dir = PKG / "_build"
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", f"-I{PKG / 'include'}", f"-I{ROOT / 'include'}",
           str(SRC), "-o", str(exe), f"-L{lib_dir}", "-lb2g", f"-Wl,-rpath,{lib_dir}"]
    subprocess.run(cmd, check=True)
    return exe


def test_reference_unit_tests_host(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe), "host-only"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK: 0 failures" in r.stdout


@pytest.mark.gpu
def test_reference_unit_tests_gpu(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK: 0 failures" in r.stdout
