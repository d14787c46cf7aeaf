"""Generates tests/golden/replay_d10.csv and replay_d10.json with the
reference's own replay code (ReplayManager of replay.h, built into
oracle/_ref by oracle/build_ref.py).

    python tests/golden/make_golden_replay.py

A source replay in the reference's CSV format is written here: camera
moves (SetLocation / SetRotation of an orbit around the depth-10 shell
scene), sphere carves and fills, cube fills, a paint, copies in both the
10-cell and the 21-cell form, a flood fill, undo / redo and tool parameters,
positions and radii recorded at REPLAY_DEPTH 16.  (A negative integer cell
is written back as its uint32 value, which the reference's own stoi then
refuses to read, so the source has none.)
The reference's ReplayManager::load_csv reads it and write_csv writes it
back: that output is replay_d10.csv.  A second, fresh process reads
replay_d10.csv with load_csv and dumps every action's fields (as doubles)
into replay_d10.json with the frame count.
"""
import ctypes as C
import json
import math
import os
import shutil
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
DEPTH, REPLAY_DEPTH = 10, 16
TYPES = ["SetLocation", "SetRotation", "SetToolParameters", "EditSphere", "EditCube", "EditCopy", "EditFill",
         "EditPaint", "Undo", "Redo", "EndFrame"]


def load_ref():
    t, b = workloads.color_tree_levels(DEPTH), workloads.top_bucket_bits(DEPTH)
    R = C.CDLL(build_ref.build(DEPTH, t, b, colors=True))
    R.ref_replay_load.argtypes = [C.c_char_p]
    R.ref_replay_write.argtypes = [C.c_char_p]
    R.ref_replay_count.restype = C.c_uint64
    R.ref_replay_frames.restype = C.c_uint64
    R.ref_replay_action.restype = C.c_uint32
    R.ref_replay_action.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p]
    return R


def rotation_looking_at(pos, target):
    """CameraView rows: -right, up, forward (camera_view.h:15-27)."""
    f = np.asarray(target, float) - np.asarray(pos, float)
    f /= np.linalg.norm(f)
    r = np.cross(f, [0.0, 1.0, 0.0])
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    return list(-r) + list(u) + list(f)


def source_lines(rng):
    e = float(1 << DEPTH)
    scale = float(1 << REPLAY_DEPTH) / e
    T = workloads.color_tree_levels(DEPTH)
    t = po.Table(po.default_config(DEPTH, T))
    t.load_basic_dag(po.generate_basic_dag(workloads.SEED_SCENE, DEPTH, T, flags=po.SCENE_SHELL))

    def surface():
        while True:
            x, z = (int(v) for v in rng.integers(40, int(e) - 40, 2))
            for y in range(int(e) - 2, 1, -1):
                if t.get_value(x, y, z):
                    return np.array([x, y, z], float)

    lines = []
    world = 100.0  # the scene's DAGInfo spans [0, 100]^3 in world units

    def frame(k):
        a = 2 * math.pi * k / 7
        pos = [50 + 80 * math.cos(a), 70.0, 50 + 80 * math.sin(a)]
        lines.append("SetLocation," + ",".join(f"{v:.6f}" for v in pos))
        lines.append("SetRotation," + ",".join(f"{v:.6f}" for v in rotation_looking_at(pos, [world / 2] * 3)))
        lines.append("EndFrame")

    def at(p, jitter=0.37):
        return [float(v) * scale + jitter * scale * rng.uniform(-1, 1) for v in p]

    frame(0)
    lines.append("SetToolParameters,%d,%d,%d,%d,%d,%d,%d,%d,%d,%.6f,%d" % (
        *[int(v) for v in surface() * scale], 1000, 2000, 3000, 3500, 4000, 5000, 12.5 * scale, 1))
    kinds = ["sphere_remove", "sphere_add", "cube_add", "paint", "copy10", "sphere_remove", "copy21", "fill",
             "cube_remove", "undo", "redo", "paint"]
    for k, kind in enumerate(kinds):
        c = surface()
        r = float(rng.uniform(6, 24))
        if kind.startswith("sphere"):
            lines.append("EditSphere,%s,%.6f,%s" % (",".join(f"{v:.6f}" for v in at(c)), r * scale,
                                                    "true" if kind.endswith("add") else "false"))
        elif kind.startswith("cube"):
            lines.append("EditCube,%s,%.6f,%s" % (",".join(f"{v:.6f}" for v in at(c)), r * scale,
                                                  "TRUE" if kind.endswith("add") else "FALSE"))
        elif kind == "paint":
            lines.append("EditPaint,%s,%.6f" % (",".join(f"{v:.6f}" for v in at(c)), r * scale))
        elif kind == "fill":
            above = c + np.array([0.0, 3.0, 0.0])
            lines.append("EditFill,%s,%.6f" % (",".join(f"{v:.6f}" for v in at(above, 0.0)), 6.0 * scale))
        elif kind.startswith("copy"):
            src = c
            dst = src + rng.integers(-60, 61, 3)
            cells = [*at(src, 0.0), *(src * scale), *(dst * scale), float(int(r)) * scale]
            line = "EditCopy," + ",".join(f"{v:.6f}" for v in cells)
            if kind == "copy21":
                line += ",1.000000,0.000000,0.000000,0.000000,1.000000,0.000000,0.000000,0.000000,1.000000,false,1.0"
            lines.append(line)
        elif kind == "undo":
            lines.append("Undo")
        elif kind == "redo":
            lines.append("Redo,")  # an empty trailing cell is dropped
        frame(k + 1)
    return lines


def phase(tmp, what):
    R = load_ref()
    if what == "normalise":
        with Silence():
            R.ref_replay_load(os.path.join(tmp, "source.csv").encode())
            R.ref_replay_write(os.path.join(tmp, "replay.csv").encode())
        return
    with Silence():
        R.ref_replay_load(os.path.join(tmp, "replay.csv").encode())
    actions = []
    v = np.zeros(32, np.float64)
    n = C.c_uint32()
    for i in range(R.ref_replay_count()):
        t = R.ref_replay_action(i, v.ctypes.data_as(C.c_void_p), C.byref(n))
        actions.append(dict(type=TYPES[t], fields=[float(x) for x in v[:n.value]]))
    with open(os.path.join(tmp, "dump.json"), "w") as f:
        json.dump(dict(frames=int(R.ref_replay_frames()), actions=actions), f)


def main():
    if len(sys.argv) > 3 and sys.argv[1] == "--phase":
        phase(sys.argv[2], sys.argv[3])
        return
    tmp = tempfile.mkdtemp()
    try:
        with open(os.path.join(tmp, "source.csv"), "w", newline="\n") as f:
            f.write("\n".join(source_lines(np.random.default_rng(3))) + "\n")
        for what in ("normalise", "dump"):
            subprocess.check_call([sys.executable, os.path.abspath(__file__), "--phase", tmp, what])
        shutil.copy(os.path.join(tmp, "replay.csv"), os.path.join(HERE, "replay_d10.csv"))
        dump = json.load(open(os.path.join(tmp, "dump.json")))
        out = dict(depth=DEPTH, replay_depth=REPLAY_DEPTH, color_tree_levels=workloads.color_tree_levels(DEPTH),
                   seed=workloads.SEED_SCENE, color_seed=workloads.SEED_COLORS, shell=True,
                   world_min=[0.0, 0.0, 0.0], world_max=[100.0, 100.0, 100.0], **dump)
        with open(os.path.join(HERE, "replay_d10.json"), "w") as f:
            json.dump(out, f, indent=1)
        print("actions", len(dump["actions"]), "frames", dump["frames"])
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    main()
