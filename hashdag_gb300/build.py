"""Builds the sm_103a shared library libhashdag_gb300.so in-tree.

    python -m hashdag_gb300.build [--force]

Each .cu file of csrc/ compiles on its own (in parallel) with
`-gencode arch=compute_103a,code=sm_103a -lineinfo -O3 -fmad=false`, then one
shared library is linked.  -fmad=false keeps every float/double expression
rounded operation by operation so that results match the reference
bit-for-bit; the kernels place their fused multiply-adds explicitly.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhashdag_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
              "-Xptxas", "-v"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "hashdag_gb300.h"))
    return hs


def build(force=False, verbose=False):
    nvcc = _nvcc()
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sources()
    newest_hdr = max(os.path.getmtime(h) for h in headers())
    objs, jobs = [], []
    for s in srcs:
        o = os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_hdr):
            jobs.append((s, o))

    def compile_one(job):
        s, o = job
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-I", INCLUDE, "-c", s, "-o", o + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {s}:\n{r.stdout}\n{r.stderr}")
        os.replace(o + ".tmp", o)
        return s, r.stderr

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for s, log in ex.map(compile_one, jobs):
                if verbose:
                    print(f"== {os.path.basename(s)}\n{log}")
    if force or jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv or "--verbose" in sys.argv))
