"""Pins the oracle (oracle/hd_oracle.c) to the reference's own code: the
golden fixtures in tests/golden/ were produced by the reference's host path
built from its sources (tests/golden/make_golden.py).  CPU only."""
import hashlib
import json
import os

import numpy as np
import pytest

from hashdag_gb300 import workloads
from oracle import pyoracle as po
from tests.helpers import table_digest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def test_hash_known_answers():
    kat = _load("hash_kat.json")
    for leaf, h in kat["leaf"]:
        assert po.lib().or_hash_leaf(leaf) == h
    for node, h in kat["interior"]:
        arr = np.array(node, np.uint32)
        assert po.lib().or_hash_interior(arr.size, arr) == h


@pytest.mark.parametrize("name", ["ref_d10.json", "ref_d12.json"])
def test_oracle_matches_reference(name):
    fx = _load(name)
    depth, bits = fx["depth"], fx["top_bucket_bits"]
    words = po.generate_basic_dag(fx["seed"], depth, fx["color_tree_levels"])
    assert words.size == fx["basic_dag_words"]
    assert hashlib.sha256(words.tobytes()).hexdigest() == fx["basic_dag_sha256"]
    cfg = po.default_config(depth, fx["color_tree_levels"])
    assert cfg.top_bucket_bits == bits
    t = po.Table(cfg)
    t.load_basic_dag(words)
    ex = t.export()
    assert t.root == fx["load"]["root"]
    assert t.pool_top == fx["load"]["pool_top"]
    assert [int(v) for v in ex["full_nodes"][1:depth - 1]] == fx["load"]["full_nodes"]
    assert table_digest(ex, depth, bits) == fx["load"]["digest"]
    for step in fx["edits"]:
        s = t.edit(step["tool"], step["center"], step["radius"])
        assert t.root == step["root"]
        assert s.num_voxels == step["num_voxels"]
        assert s.num_nodes == step["num_nodes"]
        assert t.pool_top == step["pool_top"]
        st = t.level_stats()
        assert [int(v) for v in st.words[:depth - 1]] == step["level_words"]
        assert table_digest(t.export(), depth, bits) == step["digest"]
    q = fx["queries"]
    vals = [t.get_value(*p) for p in q["xyz"]]
    assert vals == q["values"]
    # GC: the re-insertion order is canonical here and hash-set order in the
    # reference, so compare what does not depend on it.
    t.gc()
    g = fx["gc"]
    assert [int(v) for v in t.reachable_counts()] == g["reachable"]
    assert t.fingerprint() == g["fingerprint"]
    st = t.level_stats()
    nodes = [int(v) for v in st.nodes[:depth - 1]]
    assert nodes == [r + 1 for r in g["reachable"]]  # live nodes + the re-added full node


def test_scene_height_host_matches_oracle():
    from hashdag_gb300 import scene
    rng = np.random.default_rng(3)
    for depth in (8, 10, 15, 17):
        xs = rng.integers(0, 1 << depth, 300)
        zs = rng.integers(0, 1 << depth, 300)
        h = scene.height(1, depth, xs, zs)
        ref = [po.scene_height(1, depth, int(x), int(z)) for x, z in zip(xs, zs)]
        assert [int(v) for v in h] == ref
    sp = scene.spheres(1, 15)
    assert np.array_equal(sp, po.scene_spheres(1, 15))


def test_oracle_volume_matches_scene_function():
    depth = 8
    words = po.generate_basic_dag(1, depth, workloads.color_tree_levels(depth))
    t = po.Table(po.default_config(depth))
    t.load_basic_dag(words)
    rng = np.random.default_rng(0)
    e = 1 << depth
    for _ in range(2000):
        x, y, z = (int(v) for v in rng.integers(0, e, 3))
        assert t.get_value(x, y, z) == po.scene_solid(1, depth, x, y, z)


def _color_state(get_value, get_color, boxes, half):
    rows = []
    for (cx, cy, cz) in boxes:
        for x in range(cx - half, cx + half):
            for y in range(cy - half, cy + half):
                for z in range(cz - half, cz + half):
                    if get_value(x, y, z):
                        rows.append((x, y, z) + tuple(get_color(x, y, z)))
    rows = sorted(set(rows))
    arr = np.array(rows, np.uint32).reshape(-1, 6)
    return len(rows), hashlib.sha256(arr.tobytes()).hexdigest()


def test_oracle_colors_match_reference_fixture():
    """Shell scene with colours, an edit stream over all six tools and a GC:
    roots, edit counters and the colour of every present voxel in boxes
    around the edits equal what the reference computed (fixture made by
    tests/golden/make_golden_colors.py)."""
    fx = _load("ref_colors_d10.json")
    depth, T = fx["depth"], fx["color_tree_levels"]
    words = po.generate_basic_dag(fx["seed"], depth, T, flags=po.SCENE_SHELL)
    assert hashlib.sha256(words.tobytes()).hexdigest() == fx["basic_dag_sha256"]
    ot = po.Table(po.default_config(depth))
    ot.load_basic_dag(words)
    col = po.Colors(ot)
    col.from_scene(fx["color_seed"])
    boxes = [tuple(b) for b in fx["boxes"]]

    def state():
        return _color_state(ot.get_value, col.get_color, boxes, fx["half"])

    step = fx["steps"][0]
    assert ot.root == step["root"]
    assert state() == (step["present"], step["digest"])
    for i, (e, step) in enumerate(zip(fx["edits"], fx["steps"][1:])):
        s = col.edit(e["tool"], e["center"], e["radius"], source=e["source"], dest=e["dest"])
        assert ot.root == step["root"], i
        assert (s.num_voxels, s.num_nodes) == (step["num_voxels"], step["num_nodes"]), i
        assert state() == (step["present"], step["digest"]), i
    ot.gc()
    g = fx["gc"]
    assert state() == (g["present"], g["digest"])


def test_oracle_color_undo_redo_restores_state():
    """HashDAGUndoRedo semantics on the oracle: undo gives back the root and
    the colours before the edit, redo the ones after."""
    fx = _load("ref_colors_d10.json")
    depth, T = fx["depth"], fx["color_tree_levels"]
    ot = po.Table(po.default_config(depth))
    ot.load_basic_dag(po.generate_basic_dag(fx["seed"], depth, T, flags=po.SCENE_SHELL))
    col = po.Colors(ot)
    col.from_scene(fx["color_seed"])
    boxes = [tuple(b) for b in fx["boxes"][:4]]

    def state():
        return ot.root, _color_state(ot.get_value, col.get_color, boxes, fx["half"])

    states = [state()]
    for e in fx["edits"][:4]:
        col.edit(e["tool"], e["center"], e["radius"], source=e["source"], dest=e["dest"])
        states.append(state())
    for k in range(4, 0, -1):
        assert col.undo()
        assert state() == states[k - 1]
    assert not col.undo()
    for k in range(1, 5):
        assert col.redo()
        assert state() == states[k]
    assert not col.redo()
