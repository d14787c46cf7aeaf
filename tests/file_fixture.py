"""Shared pieces of the file-format tests: the fixture of the reference's
own writers (tests/golden/make_golden_files.py) and the oracle's rebuild of
the files it wrote."""
import hashlib
import json
import os

import numpy as np

from oracle import pyoracle as po

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "files_d9")
NAMES = ("scene.basic_dag.dag.bin", "scene.basic_dag.compressed_colors.variable.bin", "scene.hash_dag.bin")


def fixture():
    with open(os.path.join(GOLDEN, "ref_files_d9.json")) as f:
        return json.load(f)


def info(fx):
    e = float(1 << fx["depth"])
    return (0.0, 0.0, 0.0), (e, e, e)


def config(fx):
    cfg = po.default_config(fx["depth"], fx["color_tree_levels"], fx["pool_pages"])
    cfg.top_bucket_bits = fx["top_bucket_bits"]
    return cfg


def rebuild(fx):
    """The three files' bytes as the oracle writes them: the BasicDAG and its
    compressed colours of the generated scene, and the hash-DAG file after the
    fixture's two edits."""
    D, T = fx["depth"], fx["color_tree_levels"]
    words = po.generate_basic_dag(fx["seed"], D, T, flags=po.SCENE_SHELL)
    t = po.Table(config(fx))
    t.load_basic_dag(words)
    col = po.Colors(t)
    col.from_scene(fx["color_seed"])
    for e in fx["edits"]:
        col.edit(e["tool"], e["center"], e["radius"])
    return {NAMES[0]: po.basic_dag_file(words, D, info(fx)),
            NAMES[1]: po.compressed_colors_file(words, D, T, fx["color_seed"]),
            NAMES[2]: po.hash_dag_file(t, info(fx), fx["pool_pages"])}


def sha(b):
    return hashlib.sha256(b).hexdigest()


def box_points(boxes, half):
    """Voxels of the boxes in the fixture's loop order (x, then y, then z)."""
    pts = []
    for (cx, cy, cz) in boxes:
        g = np.stack(np.meshgrid(np.arange(cx - half, cx + half), np.arange(cy - half, cy + half),
                                 np.arange(cz - half, cz + half), indexing="ij"), -1).reshape(-1, 3)
        pts.append(g)
    return np.concatenate(pts).astype(np.uint32)


def occupancy_digest(values):
    v = np.asarray(values, np.uint8)
    return int(v.sum()), sha(v.tobytes())


def colors_digest(points, values, colors):
    keep = np.asarray(values, bool)
    rows = np.concatenate([points[keep], np.asarray(colors, np.uint32)[keep]], axis=1).astype(np.uint32)
    return len(rows), sha(rows.tobytes())
