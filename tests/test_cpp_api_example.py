"""The C++ classes of include/hashdag_gb300.hpp (the reference's HashDAG /
editor / DAGTracer / undo shapes over the C ABI): tests/cpp_api_example.cpp
compiles with g++ -std=c++17 -Wall -Wextra -Werror and links against the
library (CPU), and runs on a GPU."""
import os
import shutil
import subprocess

import pytest

from hashdag_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp_api_example.cpp")


def _cuda_dir():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.isdir(os.path.join(d, "include")):
            return d
    pytest.skip("no CUDA toolkit")


def _compile(out):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    build.build()
    cuda = _cuda_dir()
    lib_dir = os.path.join(ROOT, "hashdag_gb300")
    cmd = [cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), SRC, "-L", lib_dir, "-lhashdag_gb300",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + lib_dir,
           "-Wl,-rpath," + os.path.join(cuda, "lib64"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_program_compiles_and_links(tmp_path):
    _compile(str(tmp_path / "cpp_api_example"))


@pytest.mark.gpu
def test_cpp_program_runs(gpu, tmp_path):
    exe = str(tmp_path / "cpp_api_example")
    _compile(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "cpp api ok" in r.stdout
