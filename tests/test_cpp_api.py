"""The C++20 host API (include/bgt_gb300/bgt.hpp): it compiles with the host
compiler here, and on a device the reference's C++ pins
(tests/cpp/api_test.cpp) pass through it."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(REPO, "bayesiangrouptesting_gb300", "_build")


def _compile(tmp_path, link):
    exe = tmp_path / "api_test"
    cmd = ["g++", "-std=c++20", "-O1", "-Wall", "-Wextra", "-I", INCLUDE, os.path.join(HERE, "cpp", "api_test.cpp")]
    if link:
        cmd += ["-o", str(exe), "-L", BUILD, "-lbgt_gb300", f"-Wl,-rpath,{BUILD}"]
    else:
        cmd += ["-fsyntax-only"]
    try:
        out = subprocess.run(cmd, capture_output=True, text=True)
    except FileNotFoundError:
        pytest.skip("no host C++ compiler")
    assert out.returncode == 0, out.stderr
    return exe


def test_cpp_api_compiles(tmp_path):
    _compile(tmp_path, link=False)


@pytest.mark.gpu
def test_cpp_api_reference_pins(gpu, tmp_path):
    exe = _compile(tmp_path, link=True)
    out = subprocess.run([str(exe), str(tmp_path / "reports")], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().startswith("ok"), out.stdout
