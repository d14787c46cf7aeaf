"""Generates tests/golden/ref_colors_d10.json from the reference's own colour
code (oracle/_ref, built from the reference sources with
EDITS_ENABLE_COLORS=1 by oracle/build_ref.py).

    python tests/golden/make_golden_colors.py

Scene: the seeded shell scene (solid voxels with an empty face neighbour)
at depth 10, voxel colours from the colour field of seed 2 packed by the
reference's ColorLeafBuilder and imported with load_colors_from_DAG.  Then
an edit stream over all six tools (sphere carve / fill, box carve / fill,
sphere paint, copy) and one remove_stale_nodes.  After every step the
fixture pins the root, the edit counters, and DAGUtils::get_color of every
present voxel in boxes around the edits (digest plus a few raw values).
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
DEPTH, COLOR_SEED, HALF = 10, workloads.SEED_COLORS, 10
TOOLS = [4, 1, 0, 3, 2, 4, 5, 1, 4, 5, 0, 3, 4, 5]


def load_ref(depth):
    t, b = workloads.color_tree_levels(depth), workloads.top_bucket_bits(depth)
    R = C.CDLL(build_ref.build(depth, t, b, colors=True))
    R.ref_root.restype = C.c_uint32
    R.ref_get_value.argtypes = [C.c_uint32] * 3
    R.ref_get_color.argtypes = [C.c_uint32] * 3 + [C.c_void_p]
    R.ref_edit_colored.argtypes = [C.c_uint32, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    return R, t


def surface_points(get_value, depth, n, rng):
    e = 1 << depth
    pts = []
    while len(pts) < n:
        x, z = (int(v) for v in rng.integers(HALF + 1, e - HALF - 1, 2))
        for y in range(e - HALF - 2, HALF, -1):
            if get_value(x, y, z):
                pts.append((x, y, z))
                break
    return pts


def edit_stream(depth, rng, centers):
    edits = []
    for i, tool in enumerate(TOOLS):
        c = centers[i]
        r = float(np.float32(rng.uniform(6, 32)))
        e = dict(tool=tool, center=[c[0] + 0.5, c[1] + 0.5, c[2] + 0.5], radius=r, source=[0.0, 0.0, 0.0],
                 dest=[0.0, 0.0, 0.0])
        if tool == 5:
            s = centers[i + len(TOOLS)]
            e["center"] = [float(s[0]), float(s[1]), float(s[2])]
            e["radius"] = float(int(r))
            e["dest"] = [float(v) for v in rng.integers(-48, 49, 3)]
        edits.append(e)
    return edits


def color_state(get_value, get_color, boxes):
    rows = []
    for (cx, cy, cz) in boxes:
        for x in range(cx - HALF, cx + HALF):
            for y in range(cy - HALF, cy + HALF):
                for z in range(cz - HALF, cz + HALF):
                    if get_value(x, y, z):
                        rows.append((x, y, z) + tuple(get_color(x, y, z)))
    rows = sorted(set(rows))
    arr = np.array(rows, np.uint32).reshape(-1, 6)
    return dict(present=len(rows), digest=hashlib.sha256(arr.tobytes()).hexdigest(),
                first=[list(map(int, r)) for r in rows[:: max(1, len(rows) // 16)][:16]])


def main():
    R, T = load_ref(DEPTH)
    words = po.generate_basic_dag(workloads.SEED_SCENE, DEPTH, T, flags=po.SCENE_SHELL)
    with Silence():
        R.ref_load_colored(words.ctypes.data_as(C.c_void_p), C.c_uint64(words.size), C.c_uint32(1 << 20),
                           C.c_uint64(COLOR_SEED))

    def ref_color(x, y, z):
        out = np.zeros(3, np.uint32)
        R.ref_get_color(x, y, z, out.ctypes.data_as(C.c_void_p))
        return [int(v) for v in out]

    rng = np.random.default_rng(7)
    centers = surface_points(R.ref_get_value, DEPTH, 2 * len(TOOLS), rng)
    edits = edit_stream(DEPTH, rng, centers)
    boxes = [tuple(int(v) for v in c) for c in centers[:len(TOOLS)]]
    boxes += [tuple(int(c[k] + e["dest"][k]) for k in range(3)) for c, e in zip(centers[len(TOOLS):], edits)
              if e["tool"] == 5]
    out = dict(depth=DEPTH, color_tree_levels=T, seed=workloads.SEED_SCENE, color_seed=COLOR_SEED, shell=True,
               basic_dag_words=int(words.size), basic_dag_sha256=hashlib.sha256(words.tobytes()).hexdigest(),
               boxes=[list(b) for b in boxes], half=HALF, edits=edits, steps=[])
    out["steps"].append(dict(root=int(R.ref_root()), **color_state(R.ref_get_value, ref_color, boxes)))
    for e in edits:
        st = np.zeros(2, np.uint64)
        with Silence():
            R.ref_edit_colored(e["tool"], (C.c_float * 3)(*e["center"]), C.c_float(e["radius"]),
                               (C.c_float * 3)(*e["source"]), (C.c_float * 3)(*e["dest"]),
                               st.ctypes.data_as(C.c_void_p))
        out["steps"].append(dict(root=int(R.ref_root()), num_voxels=int(st[0]), num_nodes=int(st[1]),
                                 **color_state(R.ref_get_value, ref_color, boxes)))
    with Silence():
        R.ref_gc()
    out["gc"] = dict(root=int(R.ref_root()), **color_state(R.ref_get_value, ref_color, boxes))
    with open(os.path.join(HERE, "ref_colors_d10.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("steps", len(out["steps"]), "present", [s["present"] for s in out["steps"]])


if __name__ == "__main__":
    main()
