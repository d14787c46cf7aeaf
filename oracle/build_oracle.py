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


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
