"""The oracle's noise and flood-fill editors against the reference's own
SphereNoiseEditor / FillEditorColors (fixture ref_tools_d10.json, made by
tests/golden/make_golden_tools.py): FastNoise known answers, then the edit
stream's roots, counters and the colour of every present voxel in boxes
around the edits."""
import hashlib
import json
import os

import numpy as np

from oracle import pyoracle as po

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture():
    with open(os.path.join(GOLDEN, "ref_tools_d10.json")) as f:
        return json.load(f)


def _colors(t, col, boxes, half):
    rows = []
    for (cx, cy, cz) in boxes:
        for x in range(cx - half, cx + half):
            for y in range(cy - half, cy + half):
                for z in range(cz - half, cz + half):
                    if t.get_value(x, y, z):
                        rows.append((x, y, z) + tuple(col.get_color(x, y, z)))
    rows = sorted(set(rows))
    arr = np.array(rows, np.uint32).reshape(-1, 6)
    return len(rows), hashlib.sha256(arr.tobytes()).hexdigest()


def test_perlin_fractal_known_answers():
    for seed, freq, octaves, x, y, z, bits in _fixture()["perlin_kat"]:
        v = np.float32(po.perlin_fractal(seed, freq, octaves, x, y, z))
        assert int(v.view(np.uint32)) == bits, (seed, freq, x, y, z)


def test_noise_and_fill_edits_match_reference():
    fx = _fixture()
    D, T = fx["depth"], fx["color_tree_levels"]
    t = po.Table(po.default_config(D, T))
    t.load_basic_dag(po.generate_basic_dag(fx["seed"], D, T, flags=po.SCENE_SHELL))
    col = po.Colors(t)
    col.from_scene(fx["color_seed"])
    boxes = [tuple(b) for b in fx["boxes"]]
    assert t.root == fx["steps"][0]["root"]
    for e, want in zip(fx["edits"], fx["steps"][1:]):
        st = col.edit(e["tool"], e["center"], e["radius"])
        assert t.root == want["root"], e
        assert (st.num_voxels, st.num_nodes) == (want["num_voxels"], want["num_nodes"]), e
        assert _colors(t, col, boxes, fx["half"]) == (want["present"], want["digest"]), e
