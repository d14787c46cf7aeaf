"""Generates tests/golden/ref_trace_colors.json from the reference's own
Tracer::trace_colors (tracer.cu:254-451, TOOL_OVERLAY=1), compiled for the
host with its traversal code by oracle/build_ref.py (tracer=True,
colors=True; oracle/refharness/ref_tracer.cpp).

    python tests/golden/make_golden_trace_colors.py

Scene: the seeded shell scene at depth 10 with the colour field of seed 2.
A first process loads it (load_from_DAG + load_colors_from_DAG) and writes
the BasicDAG and compressed-colour files with the reference's writers; a
second loads those files with the reference's loaders (one shared main colour
leaf), applies a paint, a sphere fill and a sphere carve, traces the orbit
pose at 1920 x 1080 (Tracer::trace_paths) and draws every colour view:
EDebugColors None to Weight, Index at several levels, and the ToolInfo
overlay of a sphere, a cube and a copy tool.  The fixture keeps the files'
SHA-256, the edits, the paths' SHA-256 and, per view, the SHA-256 of the
rgb888 image and a few pixels of one row.  Arithmetic as the host compile
does it (fp_mode 0).
"""
import ctypes as C
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from hashdag_gb300 import workloads  # noqa: E402
from oracle import build_ref, pyoracle as po  # noqa: E402
from tests.golden.make_golden import Silence  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
DEPTH, POOL = 10, 1 << 20
NAMES = ("scene.basic_dag.dag.bin", "scene.basic_dag.compressed_colors.variable.bin")
SAMPLE_ROW = 600


def load_lib():
    T, B = workloads.color_tree_levels(DEPTH), workloads.top_bucket_bits(DEPTH)
    R = C.CDLL(build_ref.build(DEPTH, T, B, colors=True, tracer=True))
    R.ref_get_value.argtypes = [C.c_uint32] * 3
    R.ref_save_files.argtypes = [C.c_char_p] * 3
    R.ref_load_files.argtypes = [C.c_char_p, C.c_char_p, C.c_uint32]
    R.ref_edit_colored.argtypes = [C.c_uint32, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    R.ref_trace_paths.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    R.ref_trace_colors.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_int, C.c_void_p, C.c_float, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_int]
    R.ref_root.restype = C.c_uint32
    return R, T


def phase_write(tmp):
    R, T = load_lib()
    words = po.generate_basic_dag(workloads.SEED_SCENE, DEPTH, T, flags=po.SCENE_SHELL)
    with Silence():
        assert R.ref_load_colored(words.ctypes.data_as(C.c_void_p), C.c_uint64(words.size), C.c_uint32(POOL),
                                  C.c_uint64(workloads.SEED_COLORS)) == 0
        R.ref_save_files(os.path.join(tmp, NAMES[0]).encode(), os.path.join(tmp, NAMES[1]).encode(), None)


def surface_points(R, n, rng):
    e = 1 << DEPTH
    pts = []
    while len(pts) < n:
        x, z = (int(v) for v in rng.integers(200, e - 200, 2))
        for y in range(e - 40, 40, -1):
            if R.ref_get_value(x, y, z):
                pts.append((x, y, z))
                break
    return pts


def views(T, centre):
    out = [dict(debug=d, level=0, tool=None) for d in range(8)]
    out += [dict(debug=1, level=lv, tool=None) for lv in (1, 3, T, DEPTH - 2)]
    c = [int(v) for v in centre]
    out += [dict(debug=0, level=0, tool=dict(kind=0, pos=c, radius=60.0, src=[0, 0, 0], dst=[0, 0, 0])),
            dict(debug=7, level=0, tool=dict(kind=3, pos=c, radius=45.0, src=[0, 0, 0], dst=[0, 0, 0])),
            dict(debug=0, level=0, tool=dict(kind=4, pos=c, radius=50.0, src=[v + 20 for v in c],
                                             dst=[v - 20 for v in c]))]
    return out


def phase_trace(tmp):
    R, T = load_lib()
    with Silence():
        assert R.ref_load_files(os.path.join(tmp, NAMES[0]).encode(), os.path.join(tmp, NAMES[1]).encode(), POOL) == 0
    rng = np.random.default_rng(29)
    pts = surface_points(R, 3, rng)
    edits = []
    for (tool, r), p in zip([(4, 40.0), (1, 18.0), (0, 25.0)], pts):
        c = [float(p[0]) + 0.5, float(p[1]) + 0.5, float(p[2]) + 0.5]
        st = np.zeros(2, np.uint64)
        with Silence():
            assert R.ref_edit_colored(tool, (C.c_float * 3)(*c), C.c_float(r), (C.c_float * 3)(0, 0, 0),
                                      (C.c_float * 3)(0, 0, 0), st.ctypes.data_as(C.c_void_p)) == 0
        edits.append(dict(tool=tool, center=c, radius=r))
    W, H = R.ref_image_width(), R.ref_image_height()
    cam = workloads.orbit_camera(DEPTH, W, H)
    camv = np.array(cam["position"] + cam["ray_min"] + cam["ray_ddx"] + cam["ray_ddy"], np.float64)
    threads = os.cpu_count() or 4
    paths = np.zeros(W * H * 4, np.uint32)
    R.ref_trace_paths(camv.ctypes.data, paths.ctypes.data, threads)
    p = paths.reshape(H, W, 4)
    hits = p[..., :3][(p[..., :3] != 0).any(-1)]
    centre = hits[len(hits) // 2]
    out = []
    for v in views(T, centre):
        colors = np.zeros(W * H, np.uint32)
        t = v["tool"]
        if t is None:
            R.ref_trace_colors(paths.ctypes.data, v["debug"], v["level"], -1, None, 0.0, None, None, colors.ctypes.data,
                               threads)
        else:
            pos, src, dst = (np.array(t[k], np.uint32) for k in ("pos", "src", "dst"))
            R.ref_trace_colors(paths.ctypes.data, v["debug"], v["level"], t["kind"], pos.ctypes.data, t["radius"],
                               src.ctypes.data, dst.ctypes.data, colors.ctypes.data, threads)
        img = colors.reshape(H, W)
        out.append(dict(v, sha256=hashlib.sha256(colors.tobytes()).hexdigest(),
                        row=img[SAMPLE_ROW, ::64].tolist()))
        print(v["debug"], v["level"], t and t["kind"], out[-1]["sha256"][:12])
    return dict(root=int(R.ref_root()), edits=edits, width=W, height=H, camera={k: [float(x) for x in cam[k]] for k in
                                                                             ("position", "ray_min", "ray_ddx",
                                                                              "ray_ddy")},
                paths_sha256=hashlib.sha256(paths.tobytes()).hexdigest(), hits=int(len(hits)),
                sample_row=SAMPLE_ROW, views=out)


def main():
    if len(sys.argv) > 3 and sys.argv[1] == "--phase":
        tmp, what = sys.argv[2], sys.argv[3]
        if what == "write":
            phase_write(tmp)
        else:
            with open(os.path.join(tmp, "trace.json"), "w") as f:
                json.dump(phase_trace(tmp), f)
        return
    with tempfile.TemporaryDirectory() as tmp:
        for what in ("write", "trace"):
            subprocess.check_call([sys.executable, os.path.abspath(__file__), "--phase", tmp, what])
        res = json.load(open(os.path.join(tmp, "trace.json")))
        files = {}
        for name in NAMES:
            raw = open(os.path.join(tmp, name), "rb").read()
            files[name] = dict(bytes=len(raw), sha256=hashlib.sha256(raw).hexdigest())
    T = workloads.color_tree_levels(DEPTH)
    out = dict(depth=DEPTH, color_tree_levels=T, top_bucket_bits=workloads.top_bucket_bits(DEPTH),
               seed=workloads.SEED_SCENE, color_seed=workloads.SEED_COLORS, shell=True, pool_pages=POOL,
               fp_mode=0, files=files, **res)
    with open(os.path.join(HERE, "ref_trace_colors_d10.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
