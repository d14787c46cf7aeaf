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
