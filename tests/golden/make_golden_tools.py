"""Generates tests/golden/ref_tools_d10.json from the reference's own
SphereNoiseEditor and FillEditorColors (oracle/_ref, built from the
reference sources with EDITS_ENABLE_COLORS=1 by oracle/build_ref.py).

    python tests/golden/make_golden_tools.py

Scene: the seeded shell scene at depth 10 with the colour field of seed 2
(as tests/golden/make_golden_colors.py).  Edits: noise spheres that add and
that carve (the carving one changes nothing: BufferEditor::get_new_value
compares get_value's bool with EValues::Unknown, hash_dag_editors.h:211-220,
so a voxel set false keeps its old value), flood fills started in the air
just above the surface (integral and fractional centres and radii), and a
sphere carve between them.  After every step the fixture pins the root, the
edit counters and DAGUtils::get_color of every present voxel in boxes around
the edits.
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
from oracle import pyoracle as po  # noqa: E402
from tests.golden.make_golden import Silence  # noqa: E402
from tests.golden.make_golden_colors import load_ref  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
DEPTH, HALF = 10, 24
# (tool, radius, centre offset from a surface voxel)
STEPS = [(7, 9.0, (0.5, 0.5, 0.5)), (8, 6.0, (0.0, 4.0, 0.0)), (6, 8.0, (0.5, 0.5, 0.5)),
         (7, 13.5, (0.25, 0.75, 0.5)), (8, 7.25, (0.5, 5.5, 0.5)), (0, 6.0, (0.5, 0.5, 0.5)),
         (8, 5.0, (0.0, 3.0, 0.0)), (7, 5.0, (0.5, 0.5, 0.5))]


def surface_points(R, n, rng):
    e = 1 << DEPTH
    pts = []
    while len(pts) < n:
        x, z = (int(v) for v in rng.integers(HALF + 2, e - HALF - 2, 2))
        for y in range(e - HALF - 8, HALF, -1):
            if R.ref_get_value(x, y, z):
                pts.append((x, y, z))
                break
    return pts


def color_state(R, boxes):
    out = np.zeros(3, np.uint32)
    rows = []
    for (cx, cy, cz) in boxes:
        for x in range(cx - HALF, cx + HALF):
            for y in range(cy - HALF, cy + HALF):
                for z in range(cz - HALF, cz + HALF):
                    if R.ref_get_value(x, y, z):
                        R.ref_get_color(x, y, z, out.ctypes.data_as(C.c_void_p))
                        rows.append((x, y, z) + tuple(int(v) for v in out))
    rows = sorted(set(rows))
    arr = np.array(rows, np.uint32).reshape(-1, 6)
    return dict(present=len(rows), digest=hashlib.sha256(arr.tobytes()).hexdigest(),
                first=[list(map(int, r)) for r in rows[:: max(1, len(rows) // 16)][:16]])


def main():
    R, T = load_ref(DEPTH)
    words = po.generate_basic_dag(workloads.SEED_SCENE, DEPTH, T, flags=po.SCENE_SHELL)
    with Silence():
        R.ref_load_colored(words.ctypes.data_as(C.c_void_p), C.c_uint64(words.size), C.c_uint32(1 << 20),
                           C.c_uint64(workloads.SEED_COLORS))
    rng = np.random.default_rng(17)
    pts = surface_points(R, len(STEPS), rng)
    boxes = [tuple(int(v) for v in p) for p in pts]
    edits = []
    for (tool, r, off), p in zip(STEPS, pts):
        edits.append(dict(tool=tool, center=[float(p[k] + off[k]) for k in range(3)], radius=r,
                          source=[0.0, 0.0, 0.0], dest=[0.0, 0.0, 0.0]))
    out = dict(depth=DEPTH, color_tree_levels=T, seed=workloads.SEED_SCENE, color_seed=workloads.SEED_COLORS,
               shell=True, boxes=[list(b) for b in boxes], half=HALF, edits=edits, steps=[])
    out["steps"].append(dict(root=int(R.ref_root()), **color_state(R, boxes)))
    for e in edits:
        st = np.zeros(2, np.uint64)
        with Silence():
            rc = R.ref_edit_colored(e["tool"], (C.c_float * 3)(*e["center"]), C.c_float(e["radius"]),
                                    (C.c_float * 3)(0, 0, 0), (C.c_float * 3)(0, 0, 0),
                                    st.ctypes.data_as(C.c_void_p))
        assert rc == 0
        out["steps"].append(dict(root=int(R.ref_root()), num_voxels=int(st[0]), num_nodes=int(st[1]),
                                 **color_state(R, boxes)))
        print(e["tool"], out["steps"][-1]["root"], out["steps"][-1]["num_voxels"], out["steps"][-1]["present"])
    # FastNoise known answers (seed, frequency, octaves, x, y, z, value bits)
    R.ref_perlin_fractal.restype = C.c_float
    R.ref_perlin_fractal.argtypes = [C.c_int, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float]
    kat = []
    for k in range(96):
        seed = int(rng.integers(0, 1 << 30))
        freq = float(np.float32(1.0 / rng.uniform(2, 200)))
        xyz = [float(np.float32(v)) for v in rng.uniform(-300, 300, 3)]
        if k % 3 == 0:
            xyz = [float(int(v)) for v in rng.integers(0, 600, 3)]
        v = R.ref_perlin_fractal(seed, freq, 3, *xyz)
        kat.append([seed, freq, 3] + xyz + [int(np.float32(v).view(np.uint32))])
    out["perlin_kat"] = kat
    with open(os.path.join(HERE, "ref_tools_d10.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
