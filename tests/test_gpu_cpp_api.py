"""The C++ mirror of KFR's DFT interface (include/kfr_dft.hpp) end to end on the GPU: a program written
against it (tests/cpp/test_cpp_api.cpp) is compiled, linked with libkfr_capi.so and run."""
import os
import subprocess

import pytest

import kfr_gb300 as k

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_api_program(tmp_path):
    exe = str(tmp_path / "test_cpp_api")
    libdir = os.path.dirname(k.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "test_cpp_api.cpp"), "-o", exe, "-L", libdir, "-lkfr_capi",
                        "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr
