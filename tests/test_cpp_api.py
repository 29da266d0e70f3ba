"""The C++ drop-in API (include/conicxx_gb300.hpp): a caller program written against ConicXX's
Solver/ConeSpec/Settings/Solution names (tests/cpp/api_example.cpp) compiled with g++ against the
header and linked to libconicxx_gb300.so. Host mode needs no GPU; gpu mode solves the README
example through it."""
import os
import shutil
import subprocess

import pytest

from conicxx_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "api_example.cpp")


def _build(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    libdir = os.path.dirname(_lib.LIB_PATH)
    _lib.lib()  # raises LibraryMissing with the build instruction if it is absent
    exe = str(tmp_path / "api_example")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", libdir, "-lconicxx_gb300", f"-Wl,-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_api_host_paths(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "host"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_cpp_api_readme_example_on_gpu(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
