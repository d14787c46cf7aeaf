"""ORACLE — test and measurement infrastructure only.

The reference's own GPU tracer on the local GPU: the cubin that
oracle/build_ref.py build_gpu_tracer compiles from the reference's
unmodified tracer.cu (Tracer::trace_paths, tracer.cu:145-252, and the hit
test of Tracer::trace_shadows, tracer.cu:589-697), loaded by
oracle/refgpu_loader.cpp and launched as the reference's headless
DAGTracer launches it (dag_tracer.cu:116-219).  The cubin is made where the
reference sources are and travels with oracle/_ref; the loader is built
anywhere (oracle/build_oracle.py build_loader).  Frames are the reference's
compile-time 1920 x 1080 (typedefs.h:683-684).
"""
import ctypes as C
import os

import numpy as np

from oracle import build_oracle, build_ref

_lib = None


def _loader():
    global _lib
    if _lib is None:
        path = build_oracle.build_loader()
        L = C.CDLL(path)
        L.refgpu_error.restype = C.c_char_p
        L.refgpu_open.argtypes = [C.c_char_p, C.c_void_p]
        L.refgpu_set_dag.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32]
        L.refgpu_trace_view.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_void_p]
        _lib = L
    return _lib


def available(depth, ctl, top_bits):
    return os.path.exists(build_ref.cubin_path(depth, ctl, top_bits))


class RefGpuTracer:
    """One tracer per process (the loader keeps one state)."""

    def __init__(self, depth, ctl, top_bits):
        cubin = build_ref.cubin_path(depth, ctl, top_bits)
        if not os.path.exists(cubin):
            raise FileNotFoundError(f"{cubin} is missing: it is built where the reference sources are")
        self.L = _loader()
        layout = (C.c_uint32 * 6)()
        if self.L.refgpu_open(cubin.encode(), layout):
            raise RuntimeError(self.L.refgpu_error().decode())
        self.dag_bytes, _, _, self.width, self.height, self.max_levels = list(layout)
        self.depth = depth

    def set_table(self, table, pool_top=None):
        """table: pool / page_table / root arrays (a library or oracle
        export)."""
        pool = np.ascontiguousarray(table["pool"], np.uint32)
        pt = np.ascontiguousarray(table["page_table"], np.uint32)
        top = int(pool_top if pool_top is not None else pool.size // 512)
        if self.L.refgpu_set_dag(pool.ctypes.data, pool.size, pt.ctypes.data, pt.size, top, int(table["root"])):
            raise RuntimeError(self.L.refgpu_error().decode())

    def trace_view(self, cam, light, bias, own_shadows=False, read=True):
        """cam: the camera dict of the workloads (position, ray_min,
        ray_ddx, ray_ddy).  Returns (paths (H, W, 4) uint32 in output rows,
        mask (H, W) uint8: 1 shadowed, 0 lit, 2 no hit; ms: trace_paths,
        shadow hits, trace_shadows)."""
        c = np.array([float(v) for f in ("position", "ray_min", "ray_ddx", "ray_ddy") for v in
                      (cam[f] if isinstance(cam, dict) else getattr(cam, f))], np.float64)
        l = np.array(light, np.float32)
        ms = (C.c_float * 3)()
        W, H = self.width, self.height
        paths = np.zeros((H, W, 4), np.uint32) if read else None
        mask = np.zeros((H, W), np.uint8) if read else None
        r = self.L.refgpu_trace_view(c.ctypes.data, l.ctypes.data, float(bias), int(own_shadows),
                                     paths.ctypes.data if read else None, mask.ctypes.data if read else None, ms)
        if r:
            raise RuntimeError(self.L.refgpu_error().decode())
        return paths, mask, tuple(ms)

    def close(self):
        self.L.refgpu_close()
