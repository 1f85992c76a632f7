"""The C++ host layer (include/pd_gb300.hpp): compiled against the library on every machine, and its
chain tests (tests/cpp/test_host_api.cpp, written like the reference's spring_vertical.cpp) run on
the GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_host_api.cpp")


def build_test_binary(tmp_path):
    from pd_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path / "test_host_api")
    lib_dir = os.path.dirname(build.LIB)
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-o", out, "-L", lib_dir, "-lpd_gb300", f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_header_compiles_and_links(tmp_path):
    assert os.path.exists(build_test_binary(tmp_path))


@pytest.mark.gpu
def test_cpp_chain_tests_on_the_gpu(tmp_path):
    binary = build_test_binary(tmp_path)
    r = subprocess.run([binary], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
