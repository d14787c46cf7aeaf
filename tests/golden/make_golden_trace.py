"""Generates tests/golden/ref_trace.json from the reference's own traversal
code: Tracer::trace_paths and the hit test of Tracer::trace_shadows
(intersect_ray_node_out_of_order on the exact hit point), compiled for the
host from tracer.cu by oracle/build_ref.py (tracer=True, see
oracle/refharness/ref_tracer.cpp).

    python tests/golden/make_golden_trace.py

Scenes: the seeded scene (seed 1) at depths 10 and 12, loaded with the
reference's HashDAGFactory::load_from_DAG.  Frames: the reference's
imageWidth x imageHeight (1920 x 1080), every pixel.  Cameras (the four
doubles[3] of TracePathsParams): the orbit pose, poses of the Catmull-Rom
path, a camera inside solid ground, one looking exactly down the y axis and
one exactly along x on a node plane (zero direction components).  Lights:
(0.3, 1, 0.2) with bias 1, and the reference's own sun (0.3, 1, 0.5) for
one pose.  Per frame the fixture keeps the SHA-256 of the paths image
(uint32 x, y, z, 0 per pixel in output rows) and of the shadow mask (1
shadowed, 0 lit, 2 no hit), the hit and shadowed counts, and every 16th
path of one row.  The host compile rounds every float and double operation
on its own (-ffp-contract=off): the fixtures pin fp_mode 0.
"""
import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from hashdag_gb300 import workloads  # noqa: E402
from oracle import build_ref, pyoracle as po  # noqa: E402
from tests.golden.make_golden import Silence  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
LIGHT = [0.3, 1.0, 0.2]
SUN = [0.3, 1.0, 0.5]
SAMPLE_ROW = 540


def axis_camera(position, forward, right, up, step):
    p = np.asarray(position, np.float64)
    return dict(position=p.tolist(), ray_min=(p + np.asarray(forward, np.float64)).tolist(),
                ray_ddx=(step * np.asarray(right, np.float64)).tolist(),
                ray_ddy=(step * np.asarray(up, np.float64)).tolist())


def cameras(depth, W, H):
    e = float(1 << depth)
    out = [("orbit", workloads.orbit_camera(depth, W, H), LIGHT)]
    for i, c in enumerate(workloads.catmull_rom_path(depth, 8, W, H)[:3]):
        out.append((f"path{i}", c, LIGHT))
    out.append(("path0_sun", workloads.catmull_rom_path(depth, 8, W, H)[0], SUN))
    if depth == 10:
        out.append(("inside_solid", workloads.trace_params((0.5 * e, 3.0, 0.5 * e), (e, 3.0, 0.6 * e), W, H), LIGHT))
        out.append(("down_the_y_axis", axis_camera((0.5 * e + 0.5, 2.0 * e, 0.5 * e + 0.5), (0, -1, 0), (1, 0, 0),
                                                   (0, 0, 1), 2.0 ** -11), LIGHT))
        out.append(("along_x_on_a_node_plane", axis_camera((-3.0, 0.5 * e, 0.25 * e), (1, 0, 0), (0, 0, 1),
                                                           (0, 1, 0), 2.0 ** -11), [1.0, 0.0, 0.0]))
    return out


def run(depth):
    T, B = workloads.color_tree_levels(depth), workloads.top_bucket_bits(depth)
    R = C.CDLL(build_ref.build(depth, T, B, tracer=True))
    R.ref_load.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32]
    R.ref_trace_paths.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    R.ref_trace_shadows.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_int]
    words = po.generate_basic_dag(workloads.SEED_SCENE, depth, T)
    with Silence():
        assert R.ref_load(words.ctypes.data, words.size, 1 << 20) == 0
    W, H = R.ref_image_width(), R.ref_image_height()
    threads = os.cpu_count() or 4
    frames = []
    for name, cam, light in cameras(depth, W, H):
        camv = np.array(cam["position"] + cam["ray_min"] + cam["ray_ddx"] + cam["ray_ddy"], np.float64)
        paths = np.zeros(W * H * 4, np.uint32)
        mask = np.zeros(W * H, np.uint8)
        lv = np.array(light, np.float32)
        R.ref_trace_paths(camv.ctypes.data, paths.ctypes.data, threads)
        R.ref_trace_shadows(camv.ctypes.data, paths.ctypes.data, lv.ctypes.data, 1.0, mask.ctypes.data, threads)
        p = paths.reshape(H, W, 4)
        frames.append(dict(name=name, camera={k: [float(v) for v in cam[k]] for k in
                                              ("position", "ray_min", "ray_ddx", "ray_ddy")},
                           light=light, bias=1.0,
                           paths_sha256=hashlib.sha256(paths.tobytes()).hexdigest(),
                           mask_sha256=hashlib.sha256(mask.tobytes()).hexdigest(),
                           hits=int((p[..., :3] != 0).any(-1).sum()), shadowed=int((mask == 1).sum()),
                           sample_row=SAMPLE_ROW, row=p[SAMPLE_ROW, ::16, :3].reshape(-1).tolist()))
        print(depth, name, frames[-1]["hits"], frames[-1]["shadowed"])
    return dict(depth=depth, color_tree_levels=T, top_bucket_bits=B, seed=workloads.SEED_SCENE, width=W, height=H,
                frames=frames)


def main():
    if len(sys.argv) > 2 and sys.argv[1] == "--depth":
        out = run(int(sys.argv[2]))
        with open(sys.argv[3], "w") as f:
            json.dump(out, f)
        return
    # one process per depth: the reference keeps its table in a static singleton
    import subprocess
    import tempfile
    scenes = []
    with tempfile.TemporaryDirectory() as tmp:
        for depth in (10, 12):
            path = os.path.join(tmp, f"d{depth}.json")
            subprocess.check_call([sys.executable, os.path.abspath(__file__), "--depth", str(depth), path])
            scenes.append(json.load(open(path)))
    with open(os.path.join(HERE, "ref_trace.json"), "w") as f:
        json.dump(dict(fp_mode=0, scenes=scenes), f)


if __name__ == "__main__":
    main()
