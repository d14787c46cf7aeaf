"""The C ABI from plain C: tests/c_abi_example.c compiles against
include/hashdag_gb300.h with -std=c99 -Wall -Wextra -Werror and links
against the library (CPU), and runs on a GPU: scene, frame, carve, frame."""
import os
import shutil
import subprocess

import pytest

from hashdag_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_abi_example.c")


def _cuda_dir():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.isdir(os.path.join(d, "include")):
            return d
    pytest.skip("no CUDA toolkit")


def _compile(out):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    build.build()
    cuda = _cuda_dir()
    lib_dir = os.path.join(ROOT, "hashdag_gb300")
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), SRC, "-L", lib_dir, "-lhashdag_gb300",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + lib_dir,
           "-Wl,-rpath," + os.path.join(cuda, "lib64"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_c_program_compiles_and_links(tmp_path):
    _compile(str(tmp_path / "c_abi_example"))


@pytest.mark.gpu
def test_c_program_runs(gpu, tmp_path):
    exe = str(tmp_path / "c_abi_example")
    _compile(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "edited voxels" in r.stdout
