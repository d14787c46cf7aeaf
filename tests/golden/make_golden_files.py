"""Generates tests/golden/files_d9/ref_files_d9.json from the reference's own file code
(oracle/_ref, built from the reference sources with EDITS_ENABLE_COLORS=1 by
oracle/build_ref.py).

    python tests/golden/make_golden_files.py

Scene: the seeded shell scene at depth 9 with the colour field of seed 2
(as tests/golden/make_golden_colors.py).  One process loads it, writes the
BasicDAG file and the compressed-colour file with
BasicDAGFactory::save_dag_to_file / save_compressed_colors_to_file, applies
two edits (a sphere carve and a paint) and writes the hash-DAG file with
HashDAGFactory::save_dag_to_file; then it records the occupancy of boxes
around the edits, runs remove_stale_nodes, applies one more edit and records
the occupancy again.  A second, fresh process reads the two BasicDAG-side
files back with the reference's loaders (load_dag_from_file,
load_compressed_colors_from_file, load_from_DAG, load_colors_from_DAG) and
records the root and DAGUtils::get_color of every present voxel in the boxes.
Only the files' sizes and SHA-256 are kept: the tests rebuild the bytes from
the oracle (oracle/pyoracle.py) and check them against these.  The table
geometry has 2^7 buckets per level (BUCKETS_BITS_FOR_TOP_LEVELS = 7).
"""
import ctypes as C
import hashlib
import json
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
OUT = os.path.join(HERE, "files_d9")
# 2^7 buckets per level keep the hash-DAG file's pool (every touched bucket
# holds at least one page) close to the node data
DEPTH, HALF, POOL, TOP_BITS = 9, 10, 1 << 18, 7
EDITS = [dict(tool=0, radius=14.0), dict(tool=4, radius=18.0)]  # sphere carve, paint (blue)
EDIT_AFTER_GC = dict(tool=1, radius=9.0)


def load_ref():
    R = C.CDLL(build_ref.build(DEPTH, workloads.color_tree_levels(DEPTH), TOP_BITS, colors=True))
    R.ref_root.restype = C.c_uint32
    R.ref_get_value.argtypes = [C.c_uint32] * 3
    R.ref_get_color.argtypes = [C.c_uint32] * 3 + [C.c_void_p]
    R.ref_edit_colored.argtypes = [C.c_uint32, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    R.ref_save_files.argtypes = [C.c_char_p] * 3
    R.ref_load_files.argtypes = [C.c_char_p, C.c_char_p, C.c_uint32]
    return R


def boxes_of(centers):
    return [tuple(int(v) for v in c) for c in centers]


def occupancy(R, boxes):
    vals = []
    for (cx, cy, cz) in boxes:
        for x in range(cx - HALF, cx + HALF):
            for y in range(cy - HALF, cy + HALF):
                for z in range(cz - HALF, cz + HALF):
                    vals.append(R.ref_get_value(x, y, z))
    a = np.array(vals, np.uint8)
    return dict(present=int(a.sum()), digest=hashlib.sha256(a.tobytes()).hexdigest())


def colors(R, boxes):
    rows = []
    out = np.zeros(3, np.uint32)
    for (cx, cy, cz) in boxes:
        for x in range(cx - HALF, cx + HALF):
            for y in range(cy - HALF, cy + HALF):
                for z in range(cz - HALF, cz + HALF):
                    if R.ref_get_value(x, y, z):
                        R.ref_get_color(x, y, z, out.ctypes.data_as(C.c_void_p))
                        rows.append((x, y, z) + tuple(int(v) for v in out))
    arr = np.array(rows, np.uint32).reshape(-1, 6)
    return dict(present=len(rows), digest=hashlib.sha256(arr.tobytes()).hexdigest(),
                first=[list(map(int, r)) for r in rows[:: max(1, len(rows) // 8)][:8]])


def edit(R, e, center):
    st = np.zeros(2, np.uint64)
    c = [center[0] + 0.5, center[1] + 0.5, center[2] + 0.5]
    with Silence():
        R.ref_edit_colored(e["tool"], (C.c_float * 3)(*c), C.c_float(e["radius"]), (C.c_float * 3)(0, 0, 0),
                           (C.c_float * 3)(0, 0, 0), st.ctypes.data_as(C.c_void_p))
    return dict(tool=e["tool"], center=c, radius=e["radius"])


def phase_save(tmp):
    R = load_ref()
    T = workloads.color_tree_levels(DEPTH)
    words = po.generate_basic_dag(workloads.SEED_SCENE, DEPTH, T, flags=po.SCENE_SHELL)
    with Silence():
        R.ref_load_colored(words.ctypes.data_as(C.c_void_p), C.c_uint64(words.size), C.c_uint32(POOL),
                           C.c_uint64(workloads.SEED_COLORS))
    rng = np.random.default_rng(11)
    e = 1 << DEPTH
    centers = []
    while len(centers) < 3:
        x, z = (int(v) for v in rng.integers(HALF + 1, e - HALF - 1, 2))
        for y in range(e - HALF - 2, HALF, -1):
            if R.ref_get_value(x, y, z):
                centers.append((x, y, z))
                break
    boxes = boxes_of(centers)
    with Silence():
        R.ref_save_files(os.path.join(tmp, "scene.basic_dag.dag.bin").encode(),
                         os.path.join(tmp, "scene.basic_dag.compressed_colors.variable.bin").encode(), None)
    base = dict(root=int(R.ref_root()), **occupancy(R, boxes))
    edits = [edit(R, ed, centers[i]) for i, ed in enumerate(EDITS)]
    with Silence():
        R.ref_save_files(None, None, os.path.join(tmp, "scene.hash_dag.bin").encode())
    edited = dict(root=int(R.ref_root()), pool_top=int(R.ref_pool_top()), **occupancy(R, boxes))
    with Silence():
        R.ref_gc()
    after = edit(R, EDIT_AFTER_GC, centers[2])
    gc_edit = dict(edit=after, **occupancy(R, boxes))
    return dict(boxes=[list(b) for b in boxes], base=base, edits=edits, edited=edited, gc_then_edit=gc_edit)


def phase_load(tmp, boxes):
    R = load_ref()
    with Silence():
        R.ref_load_files(os.path.join(tmp, "scene.basic_dag.dag.bin").encode(),
                         os.path.join(tmp, "scene.basic_dag.compressed_colors.variable.bin").encode(), POOL)
    return dict(root=int(R.ref_root()), **colors(R, [tuple(b) for b in boxes]))


def main():
    if len(sys.argv) > 2 and sys.argv[1] == "--phase":
        tmp = sys.argv[2]
        if sys.argv[3] == "save":
            res = phase_save(tmp)
        else:
            res = phase_load(tmp, json.load(open(os.path.join(tmp, "save.json")))["boxes"])
        with open(os.path.join(tmp, sys.argv[3] + ".json"), "w") as f:
            json.dump(res, f)
        return
    tmp = tempfile.mkdtemp()
    try:
        for ph in ("save", "load"):
            subprocess.check_call([sys.executable, os.path.abspath(__file__), "--phase", tmp, ph])
        save = json.load(open(os.path.join(tmp, "save.json")))
        load = json.load(open(os.path.join(tmp, "load.json")))
        os.makedirs(OUT, exist_ok=True)
        files = {}
        for name in ("scene.basic_dag.dag.bin", "scene.basic_dag.compressed_colors.variable.bin",
                     "scene.hash_dag.bin"):
            raw = open(os.path.join(tmp, name), "rb").read()
            files[name] = dict(bytes=len(raw), sha256=hashlib.sha256(raw).hexdigest())
        out = dict(depth=DEPTH, color_tree_levels=workloads.color_tree_levels(DEPTH),
                   top_bucket_bits=TOP_BITS, seed=workloads.SEED_SCENE,
                   color_seed=workloads.SEED_COLORS, shell=True, pool_pages=POOL, half=HALF, files=files,
                   reference_load=load, **save)
        with open(os.path.join(OUT, "ref_files_d9.json"), "w") as f:
            json.dump(out, f, indent=1)
        print({k: v["bytes"] for k, v in files.items()}, "present", load["present"])
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    main()
