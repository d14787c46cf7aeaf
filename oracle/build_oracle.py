"""ORACLE build recipe (test infrastructure only).

Compiles the plain-C restatement (oracle/hd_oracle.c) into
oracle/_build/libhdoracle.so with every floating-point operation rounded on
its own (-ffp-contract=off, no fast-math) so results match IEEE evaluation in
source order on x86-64 and aarch64 alike.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libhdoracle.so")


def build(force=False, verbose=False):
    src = os.path.join(HERE, "hd_oracle.c")
    hdr = [os.path.join(HERE, "hd_oracle.h"),
           os.path.join(HERE, "..", "include", "hashdag_gb300.h")]
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in [src] + hdr)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp", src, "-lm", "-lpthread"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


LOADER = os.path.join(OUT_DIR, "libhdrefgpu.so")


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.isdir(os.path.join(cand, "include")):
            return cand
    raise FileNotFoundError("CUDA toolkit not found")


def build_loader(force=False):
    """oracle/refgpu_loader.cpp (own code, no reference header) into
    oracle/_build/libhdrefgpu.so: the loader of the reference GPU tracer's
    cubin.  Built on every machine; the cubin itself is made where the
    reference sources are (oracle/build_ref.py build_gpu_tracer)."""
    src = os.path.join(HERE, "refgpu_loader.cpp")
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LOADER) and os.path.getmtime(LOADER) >= os.path.getmtime(src):
        return LOADER
    cuda = _cuda_home()
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-Wall", "-I", os.path.join(cuda, "include"), src,
           "-o", LOADER + ".tmp", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    subprocess.check_call(cmd)
    os.replace(LOADER + ".tmp", LOADER)
    return LOADER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    print(build_loader(force="--force" in sys.argv))
