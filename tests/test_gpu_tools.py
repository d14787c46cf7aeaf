"""GPU parity of the noise-sphere and flood-fill editors: against the
reference's own SphereNoiseEditor / FillEditorColors (fixture
ref_tools_d10.json, made by tests/golden/make_golden_tools.py) and against
the oracle on a second scene, with and without colours."""
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
    with open(os.path.join(GOLDEN, "ref_tools_d10.json")) as f:
        return json.load(f)


def _box_points(boxes, half):
    pts = [np.stack(np.meshgrid(np.arange(cx - half, cx + half), np.arange(cy - half, cy + half),
                                np.arange(cz - half, cz + half), indexing="ij"), -1).reshape(-1, 3)
           for (cx, cy, cz) in boxes]
    return np.unique(np.concatenate(pts), axis=0).astype(np.uint32)


def _digest(dag, pts):
    vals = dag.get_values(pts).astype(bool)
    rows = np.concatenate([pts[vals], dag.get_colors(pts[vals])], axis=1).astype(np.uint32)
    return len(rows), hashlib.sha256(rows.tobytes()).hexdigest()


def test_noise_and_fill_match_reference(gpu):
    fx = _fixture()
    dag = hd.HashDAG(fx["depth"])
    dag.generate_scene(fx["seed"], shell=True)
    dag.colors_from_scene(fx["color_seed"])
    pts = _box_points(fx["boxes"], fx["half"])
    assert dag.firstNodeIndex == fx["steps"][0]["root"]
    for e, want in zip(fx["edits"], fx["steps"][1:]):
        st = dag.edit_threads(hd.editor_from_tuple((e["tool"], e["center"], e["radius"])))
        assert dag.firstNodeIndex == want["root"], e
        assert (st.num_voxels, st.num_nodes) == (want["num_voxels"], want["num_nodes"]), e
        assert _digest(dag, pts) == (want["present"], want["digest"]), e
    dag.free()


@pytest.mark.parametrize("colors", [False, True])
def test_noise_and_fill_match_oracle_d12(gpu, colors):
    depth = 12
    T = workloads.color_tree_levels(depth)
    dag = hd.HashDAG(depth)
    dag.generate_scene(workloads.SEED_SCENE, shell=colors)
    ot = po.Table(po.default_config(depth, T))
    ot.load_basic_dag(po.generate_basic_dag(workloads.SEED_SCENE, depth, T, flags=po.SCENE_SHELL if colors else 0))
    col = None
    if colors:
        dag.colors_from_scene(workloads.SEED_COLORS)
        col = po.Colors(ot)
        col.from_scene(workloads.SEED_COLORS)
    rng = np.random.default_rng(23)
    e = 1 << depth
    pts_all = []
    for k in range(6):
        x, z = (int(v) for v in rng.integers(64, e - 64, 2))
        y = next(y for y in range(e - 2, 0, -1) if ot.get_value(x, y, z))
        tool = [hd.TOOL_NOISE_ADD, hd.TOOL_FILL, hd.TOOL_NOISE_REMOVE][k % 3]
        r = float(rng.uniform(6, 20))
        c = [x + 0.5, y + (3.0 if tool == hd.TOOL_FILL else 0.5), z + 0.5]
        st = dag.edit_threads(hd.editor_from_tuple((tool, c, r)))
        ost = col.edit(tool, c, r) if colors else ot.edit(tool, c, r)
        assert dag.firstNodeIndex == ot.root, (tool, c, r)
        assert (st.num_voxels, st.num_nodes) == (ost.num_voxels, ost.num_nodes)
        pts_all.append((x, y, z))
    pts = _box_points(pts_all, 28)
    got = dag.get_values(pts)
    want = np.array([ot.get_value(*p) for p in pts], np.uint8)
    assert np.array_equal(got, want)
    if colors:
        gc = dag.get_colors(pts[got.astype(bool)])
        oc = np.array([col.get_color(*p) for p in pts[got.astype(bool)]], np.uint32).reshape(-1, 3)
        assert np.array_equal(gc, oc)
    dag.free()
