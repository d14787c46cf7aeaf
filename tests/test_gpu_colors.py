"""GPU parity of shell scenes, colours, paint / copy and undo: against the
reference's own colour code (fixture ref_colors_d10.json, made by
tests/golden/make_golden_colors.py) and against the oracle."""
import hashlib
import json
import os

import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import workloads
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture():
    with open(os.path.join(GOLDEN, "ref_colors_d10.json")) as f:
        return json.load(f)


def _box_voxels(boxes, half):
    pts = []
    for (cx, cy, cz) in boxes:
        g = np.stack(np.meshgrid(np.arange(cx - half, cx + half), np.arange(cy - half, cy + half),
                                 np.arange(cz - half, cz + half), indexing="ij"), -1).reshape(-1, 3)
        pts.append(g)
    return np.unique(np.concatenate(pts), axis=0).astype(np.uint32)


def _editor(e):
    if e["tool"] == hd.TOOL_SPHERE_PAINT:
        return hd.SpherePaintEditor(e["center"], e["radius"])
    if e["tool"] == hd.TOOL_COPY:
        return hd.CopyEditor(e["center"], e["radius"], e["source"], e["dest"])
    return hd.editor_from_tuple((e["tool"], e["center"], e["radius"]))


def _state(d, pts):
    v = d.get_values(pts)
    p = pts[v != 0]
    cols = d.get_colors(p)
    rows = np.concatenate([p, cols.astype(np.uint32)], axis=1)
    rows = np.array(sorted(map(tuple, rows)), np.uint32).reshape(-1, 6)
    return len(rows), hashlib.sha256(rows.tobytes()).hexdigest()


@pytest.mark.parametrize("depth", [8, 10])
def test_shell_generator_matches_oracle(gpu, depth):
    T = workloads.color_tree_levels(depth)
    d = hd.HashDAG(depth)
    d.generate_scene(1, shell=True)
    want = po.generate_basic_dag(1, depth, T, flags=po.SCENE_SHELL)
    assert np.array_equal(d.export_basic_dag(), want)
    d.free()


def test_colors_and_edits_match_reference_fixture(gpu):
    """Colour import, then sphere / box / paint / copy edits and a GC: roots,
    counters and every present voxel's colour in boxes around the edits equal
    the reference's."""
    fx = _fixture()
    depth = fx["depth"]
    d = hd.HashDAG(depth)
    d.generate_scene(fx["seed"], shell=True)
    d.colors_from_scene(fx["color_seed"])
    pts = _box_voxels([tuple(b) for b in fx["boxes"]], fx["half"])
    step = fx["steps"][0]
    assert d.firstNodeIndex == step["root"]
    assert _state(d, pts) == (step["present"], step["digest"])
    for i, (e, step) in enumerate(zip(fx["edits"], fx["steps"][1:])):
        s = d.edit_threads(_editor(e))
        assert d.firstNodeIndex == step["root"], i
        assert (s.num_voxels, s.num_nodes) == (step["num_voxels"], step["num_nodes"]), i
        assert _state(d, pts) == (step["present"], step["digest"]), i
    d.remove_stale_nodes()
    g = fx["gc"]
    assert _state(d, pts) == (g["present"], g["digest"])
    d.free()


def test_color_import_matches_oracle_leaves(gpu):
    """Per-slot leaves: the same number of blocks and macro words as the
    oracle's ColorLeafBuilder, and every voxel's colour from the field."""
    depth = 10
    T = workloads.color_tree_levels(depth)
    d = hd.HashDAG(depth)
    d.generate_scene(1, shell=True)
    d.colors_from_scene(2)
    ot = po.Table(po.default_config(depth))
    ot.load_basic_dag(po.generate_basic_dag(1, depth, T, flags=po.SCENE_SHELL))
    col = po.Colors(ot)
    col.from_scene(2)
    a, b = d.color_stats(), col.stats()
    assert (a["nodes"], a["leaves"], a["blocks"], a["macro_words"]) == \
        (b["nodes"], b["leaves"], b["blocks"], b["macro_words"])
    rng = np.random.default_rng(2)
    q = rng.integers(0, 1 << depth, (200000, 3)).astype(np.uint32)
    v = d.get_values(q)
    p = q[v != 0]
    got = d.get_colors(p)
    want = np.array([po.voxel_color(2, *map(int, x)) for x in p], np.uint32).reshape(-1, 3)
    assert len(p) > 100 and np.array_equal(got, want)
    d.free()


def test_undo_redo_restores_roots_and_colors(gpu):
    fx = _fixture()
    depth = fx["depth"]
    d = hd.HashDAG(depth)
    d.generate_scene(fx["seed"], shell=True)
    d.colors_from_scene(fx["color_seed"])
    pts = _box_voxels([tuple(b) for b in fx["boxes"][:6]], fx["half"])
    states = [(d.firstNodeIndex, _state(d, pts))]
    for e in fx["edits"][:6]:
        d.edit_threads(_editor(e))
        states.append((d.firstNodeIndex, _state(d, pts)))
    assert d.history() == (6, 0)
    for k in range(6, 0, -1):
        assert d.undo()
        assert (d.firstNodeIndex, _state(d, pts)) == states[k - 1]
    assert not d.undo()
    for k in range(1, 7):
        assert d.redo()
        assert (d.firstNodeIndex, _state(d, pts)) == states[k]
    assert not d.redo()
    # history across a GC that keeps it: the undone state is still there
    d.remove_stale_nodes(keep_history=True)
    assert d.undo()
    assert _state(d, pts) == states[5][1]
    d.free()


def test_colored_edits_match_oracle_depth12(gpu):
    """A longer stream at depth 12 (paint with a non-default colour
    included) against the oracle: roots, counters, sampled colours."""
    depth = 12
    T = workloads.color_tree_levels(depth)
    d = hd.HashDAG(depth)
    d.generate_scene(1, shell=True)
    d.colors_from_scene(2)
    ot = po.Table(po.default_config(depth))
    ot.load_basic_dag(d.export_basic_dag())
    col = po.Colors(ot)
    col.from_scene(2)
    rng = np.random.default_rng(11)
    cs = [tuple(int(v) for v in c) for c in workloads._centres(depth, 24, rng)]
    boxes = []
    for i in range(16):
        c = cs[i]
        tool = [4, 1, 0, 3, 2, 5][i % 6]
        r = float(np.float32(rng.uniform(6, 40)))
        rgb = int(rng.integers(0, 1 << 24))
        src, dst = (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)
        center = (c[0] + 0.5, c[1] + 0.5, c[2] + 0.5)
        if tool == 5:
            center = tuple(float(v) for v in cs[i + 8])
            r = float(int(r))
            dst = tuple(float(v) for v in rng.integers(-64, 65, 3))
        if tool == 4:
            ed = hd.SpherePaintEditor(center, r, rgb)
        elif tool == 5:
            ed = hd.CopyEditor(center, r, src, dst)
        else:
            ed = hd.editor_from_tuple((tool, center, r))
        s = d.edit_threads(ed)
        os_ = col.edit(tool, center, r, rgb=rgb if tool == 4 else 0xFF0000, source=src, dest=dst)
        assert d.firstNodeIndex == ot.root, i
        assert (s.num_voxels, s.num_nodes) == (os_.num_voxels, os_.num_nodes), i
        boxes.append((c[0], c[1], c[2]))
    pts = _box_voxels(boxes, 12)
    v = d.get_values(pts)
    p = pts[v != 0]
    got = d.get_colors(p)
    want = np.array([col.get_color(*map(int, x)) for x in p], np.uint32).reshape(-1, 3)
    assert np.array_equal(got, want)
    d.free()
