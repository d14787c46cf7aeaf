"""ORACLE — builds the reference's own code from its sources (test
infrastructure only).

    python oracle/build_ref.py [depth] [color_tree_levels] [top_bucket_bits]

Compiles oracle/refharness/ref_host.cpp, which #includes the reference's
unmodified host sources (hash_table.cpp, stats.cpp, hash_dag_factory.cpp and
the headers of the edit path) from the reference checkout's src/ (see REF
below), into
oracle/_ref/libhdref_d<D>_t<T>_b<B>.so.  No reference file is copied; the
output directory is git-ignored.  Build flags follow the reference's
parity build: -O2 -ffp-contract=off, no fast-math.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: HD_REFERENCE_DIR, else a "reference" directory
# beside the repository.
REF = os.environ.get("HD_REFERENCE_DIR") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))
OUT = os.path.join(HERE, "_ref")


def lib_path(depth, ctl, top_bits, colors=False, tracer=False):
    return os.path.join(OUT, f"libhdref_d{depth}_t{ctl}_b{top_bits}{'_c' if colors else ''}"
                             f"{'_trace' if tracer else ''}.so")


def available():
    return os.path.isdir(os.path.join(REF, "src"))


def build(depth, ctl, top_bits, force=False, colors=False, tracer=False):
    """colors=True: EDITS_ENABLE_COLORS=1 and the colour entry points, linked
    with the oracle library for the scene's colour field.  tracer=True: the
    reference's traversal code (tracer.cu) compiled for the host on top of the
    harness (oracle/refharness/ref_tracer.cpp)."""
    out = lib_path(depth, ctl, top_bits, colors, tracer)
    if os.path.exists(out) and not force:
        return out
    if not available():
        raise FileNotFoundError("reference sources are not present on this machine")
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(REF, "src")
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w",
           "-DBENCHMARK=1", "-DUSE_BLOOM_FILTER=0", f"-DEDITS_ENABLE_COLORS={1 if colors else 0}",
           "-DEDITS_COUNTERS=1",
           "-DENABLE_CHECKS=0", "-DTRACK_GLOBAL_NEWDELETE=0",
           f"-DHARNESS_DEPTH={depth}", f"-DBUCKETS_BITS_FOR_TOP_LEVELS={top_bits}",
           f"-DC_colorTreeLevels=CTL_VALUE = {ctl}, CTL_IGNORED",
           "-I", os.path.join(HERE, "refharness", "shim"),
           "-I", src, "-I", os.path.join(src, "dags"), "-I", os.path.join(src, "dags", "hash_dag"),
           "-I", os.path.join(src, "gmath"), "-I", "/usr/local/cuda/include",
           os.path.join(HERE, "refharness", "ref_tracer.cpp" if tracer else "ref_host.cpp"), "-o", out + ".tmp"]
    if tracer:
        cmd += ["-I", os.path.join(HERE, "refharness"), "-pthread", "-DTOOL_OVERLAY=1"]
    if colors:
        from oracle import build_oracle
        lib = build_oracle.build()
        cmd += ["-include", os.path.join(HERE, "hd_oracle.h"), lib, "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


def cubin_path(depth, ctl, top_bits):
    return os.path.join(OUT, f"ref_tracer_d{depth}_t{ctl}_b{top_bits}.cubin")


def build_gpu_tracer(depth, ctl, top_bits, force=False):
    """The reference's tracer.cu, unmodified, compiled for sm_103a into a
    cubin with the harness kernels of oracle/refharness/ref_tracer_gpu.cu,
    with the reference's CUDA flags (CMakeLists.txt:21-28: nvcc defaults,
    --expt-relaxed-constexpr).  A device binary: it travels to the GPU
    machine with oracle/_ref and is loaded there by oracle/refgpu_loader.cpp."""
    out = cubin_path(depth, ctl, top_bits)
    if os.path.exists(out) and not force:
        return out
    if not available():
        raise FileNotFoundError("reference sources are not present on this machine")
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(REF, "src")
    nvcc = os.environ.get("NVCC") or "nvcc"
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "--expt-relaxed-constexpr",
           "-O3", "-w", "-DBENCHMARK=1", "-DUSE_BLOOM_FILTER=0", "-DEDITS_ENABLE_COLORS=0", "-DEDITS_COUNTERS=1",
           "-DENABLE_CHECKS=0", "-DTRACK_GLOBAL_NEWDELETE=0", f"-DHARNESS_DEPTH={depth}",
           f"-DBUCKETS_BITS_FOR_TOP_LEVELS={top_bits}", f"-DHARNESS_CTL={ctl}",
           "-I", os.path.join(HERE, "refharness", "shim"),
           "-I", src, "-I", os.path.join(src, "dags"), "-I", os.path.join(src, "dags", "hash_dag"),
           "-I", os.path.join(src, "gmath"),
           os.path.join(HERE, "refharness", "ref_tracer_gpu.cu"), "-o", out + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    d = int(sys.argv[1]) if len(sys.argv) > 1 else 10
    t = int(sys.argv[2]) if len(sys.argv) > 2 else min(10, d - 5)
    b = int(sys.argv[3]) if len(sys.argv) > 3 else (10 if d <= 10 else 12)
    print(build(d, t, b, force=True))
