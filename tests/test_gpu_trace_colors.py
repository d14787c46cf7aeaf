"""Tracer::trace_colors on the GPU against the oracle: every EDebugColors
view, the Index view at several levels, and the ToolInfo overlay of each
tool shape, on a coloured scene after noise, fill, paint and carve edits."""
import os

import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import _capi, workloads
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
W, H = 320, 180


def _params(debug=0, level=0, tool=None):
    q = _capi.TraceColorsParams()
    q.debug_colors, q.debug_level = debug, level
    if tool is not None:
        kind, pos, radius, src, dst = tool
        q.overlay.enabled, q.overlay.tool, q.overlay.radius = 1, kind, radius
        q.overlay.position[:] = pos
        q.overlay.copy_source[:] = src
        q.overlay.copy_dest[:] = dst
    return q


def test_trace_colors_views_match_oracle(gpu):
    depth = 10
    T = workloads.color_tree_levels(depth)
    dag = hd.HashDAG(depth)
    dag.generate_scene(workloads.SEED_SCENE, shell=True)
    dag.colors_from_scene(workloads.SEED_COLORS)
    ot = po.Table(po.default_config(depth, T))
    ot.load_basic_dag(po.generate_basic_dag(workloads.SEED_SCENE, depth, T, flags=po.SCENE_SHELL))
    col = po.Colors(ot)
    col.from_scene(workloads.SEED_COLORS)
    cam = workloads.orbit_camera(depth, W, H)
    tr = hd.DAGTracer(W, H)
    tr.resolve_paths(cam, dag)
    paths = tr.get_paths().reshape(H, W, 4)
    hits = paths[..., :3][np.any(paths[..., :3] != 0, axis=-1)]
    rng = np.random.default_rng(4)
    for k, tool in enumerate([hd.TOOL_NOISE_ADD, hd.TOOL_SPHERE_PAINT, hd.TOOL_FILL, hd.TOOL_SPHERE_REMOVE]):
        p = hits[rng.integers(0, len(hits))]
        c = [float(p[0]) + 0.5, float(p[1]) + (3.0 if tool == hd.TOOL_FILL else 0.5), float(p[2]) + 0.5]
        r = float(rng.uniform(10, 30))
        dag.edit_threads(hd.editor_from_tuple((tool, c, r)))
        col.edit(tool, c, r)
    assert dag.firstNodeIndex == ot.root
    tr.resolve_paths(cam, dag)
    paths = tr.get_paths()
    centre = [int(v) for v in hits[len(hits) // 2]]
    views = [(d, 0, None) for d in range(8)]
    views += [(hd.DEBUG_INDEX, lv, None) for lv in (1, 3, T, depth - 2)]
    views += [(hd.DEBUG_NONE, 0, (hd.OVERLAY_SPHERE, centre, 40.0, (0, 0, 0), (0, 0, 0))),
              (hd.DEBUG_WEIGHT, 0, (hd.OVERLAY_CUBE, centre, 25.0, (0, 0, 0), (0, 0, 0))),
              (hd.DEBUG_NONE, 0, (hd.OVERLAY_CUBE_COPY, centre, 30.0, [v + 9 for v in centre], [v - 9 for v in centre]))]
    for debug, level, tool in views:
        got = tr.resolve_colors(dag, debug, level, tool).reshape(-1)
        want = col.trace_colors(paths, _params(debug, level, tool))
        bad = np.nonzero(got != want)[0]
        assert bad.size == 0, (debug, level, tool, bad[:5], got[bad[:5]], want[bad[:5]])
    # the plain entry point is the plain view
    got = tr.resolve_colors(dag)
    assert np.array_equal(got.reshape(-1), col.trace_colors(paths))
    # misses are the sky
    sky = np.all(paths.reshape(-1, 4)[:, :3] == 0, axis=1)
    assert sky.any() and np.all(got.reshape(-1)[sky] == po.lib().or_f3_to_rgb888(187 / 255, 242 / 255, 250 / 255))
    dag.free()


def test_trace_colors_equal_reference(gpu, tmp_path):
    """Every colour view of a 1920 x 1080 frame equals the reference's own
    Tracer::trace_colors (tests/golden/ref_trace_colors_d10.json): the scene
    read from the reference's BasicDAG and compressed-colour files (one
    shared main colour leaf, the files rebuilt here and checked against the
    reference's bytes), a paint, a fill and a carve, paths at fp_mode 0."""
    import hashlib
    import json
    fx = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                     "ref_trace_colors_d10.json")))
    D, T = fx["depth"], fx["color_tree_levels"]
    words = po.generate_basic_dag(fx["seed"], D, T, flags=po.SCENE_SHELL)
    e = float(1 << D)
    data = {"scene.basic_dag.dag.bin": po.basic_dag_file(words, D, ((0.0, 0.0, 0.0), (e, e, e))),
            "scene.basic_dag.compressed_colors.variable.bin": po.compressed_colors_file(words, D, T,
                                                                                      fx["color_seed"])}
    paths_on_disk = {}
    for name, raw in data.items():
        assert hashlib.sha256(raw).hexdigest() == fx["files"][name]["sha256"], name
        p = tmp_path / name
        p.write_bytes(raw)
        paths_on_disk[name] = str(p)
    dag = hd.HashDAG(D)
    dag.load_dag_from_file(paths_on_disk["scene.basic_dag.dag.bin"])
    dag.load_compressed_colors_from_file(paths_on_disk["scene.basic_dag.compressed_colors.variable.bin"])
    for ed in fx["edits"]:
        if ed["tool"] == hd.TOOL_SPHERE_PAINT:
            dag.edit_threads(hd.SpherePaintEditor(ed["center"], ed["radius"]))
        else:
            dag.edit_threads(hd.editor_from_tuple((ed["tool"], ed["center"], ed["radius"])))
    assert dag.firstNodeIndex == fx["root"]
    W, H = fx["width"], fx["height"]
    dag.set_fp_mode(0)
    tr = hd.DAGTracer(W, H)
    tr.resolve_paths(fx["camera"], dag)
    dag.set_fp_mode(0)
    assert hashlib.sha256(np.ascontiguousarray(tr.get_paths()).tobytes()).hexdigest() == fx["paths_sha256"]
    for v in fx["views"]:
        t = v["tool"]
        tool = None if t is None else (t["kind"], t["pos"], t["radius"], t["src"], t["dst"])
        got = np.ascontiguousarray(tr.resolve_colors(dag, v["debug"], v["level"], tool))
        row = got.reshape(H, W)[fx["sample_row"], ::64].tolist()
        assert row == v["row"], (v["debug"], v["level"], t)
        assert hashlib.sha256(got.tobytes()).hexdigest() == v["sha256"], (v["debug"], v["level"], t)
    dag.free()
