"""GPU replay of the reference's replay CSV (tests/golden/replay_d10.csv,
written by the reference's own ReplayManager): frame by frame, the edits,
undo / redo and the view applied through hd_replay_frame equal the same
actions applied to the oracle (positions and radii scaled from depth 16 to
10 in float), the frame cameras equal get_trace_params of the view, and a
frame traced from one equals the oracle's."""
import json
import math
import os

import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import workloads
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
W, H = 320, 180


def _trace_params(pos, rot, levels, lo, hi):
    """get_trace_params (dag_tracer.cu:71-113) with a 60 degree FOV."""
    right, up, fwd = [-rot[0], -rot[1], -rot[2]], rot[3:6], rot[6:9]
    fov = 60.0 / 2.0 * (math.pi / 180.0)
    aspect = W / H
    out = dict(position=[], ray_min=[], ray_ddx=[], ray_ddy=[])
    for a in range(3):
        X, Y, Z = right[a] * math.sin(fov) * aspect, up[a] * math.sin(fov), fwd[a] * math.cos(fov)
        bl, br, tl = pos[a] + Z - Y - X, pos[a] + Z - Y + X, pos[a] + Z + Y - X
        s = float(1 << levels) / (hi[a] - lo[a])
        fp, fbl, ftl, fbr = (pos[a] - lo[a]) * s, (bl - lo[a]) * s, (tl - lo[a]) * s, (br - lo[a]) * s
        out["position"].append(fp)
        out["ray_min"].append(fbl)
        out["ray_ddx"].append((fbr - fbl) * (1.0 / W))
        out["ray_ddy"].append((ftl - fbl) * (1.0 / H))
    return out


def test_replay_matches_oracle(gpu):
    with open(os.path.join(GOLDEN, "replay_d10.json")) as f:
        fx = json.load(f)
    depth, rdepth = fx["depth"], fx["replay_depth"]
    T = fx["color_tree_levels"]
    info = (tuple(fx["world_min"]), tuple(fx["world_max"]))
    dag = hd.HashDAG(depth)
    dag.generate_scene(fx["seed"], shell=True)
    dag.colors_from_scene(fx["color_seed"])
    ot = po.Table(po.default_config(depth, T))
    ot.load_basic_dag(po.generate_basic_dag(fx["seed"], depth, T, flags=po.SCENE_SHELL))
    col = po.Colors(ot)
    col.from_scene(fx["color_seed"])
    r = hd.ReplayManager(os.path.join(GOLDEN, "replay_d10.csv"))
    scale = np.float32(np.float32(1 << depth) / np.float32(1 << rdepth))
    f32 = lambda v: float(np.float32(v) * scale)  # noqa: E731
    pos, rot = [0.0, 0.0, 0.0], [1, 0, 0, 0, 1, 0, 0, 0, 1]
    action, frames = 0, 0
    tools = {"EditSphere": (hd.TOOL_SPHERE_REMOVE, hd.TOOL_SPHERE_ADD), "EditCube": (hd.TOOL_BOX_REMOVE, hd.TOOL_BOX_ADD)}
    last_cam = None
    while not r.at_end():
        cam, n_edits = r.replay_frame(dag, rdepth, W, H, info)
        applied = 0
        while True:
            t, fl, ints, flag = r.action(action)
            action += 1
            if t == "SetLocation":
                pos = [float(v) for v in fl]
            elif t == "SetRotation":
                rot = [float(v) for v in fl]
            elif t in tools:
                col.edit(tools[t][int(flag)], [f32(v) for v in fl[:3]], f32(fl[3]))
                applied += 1
            elif t == "EditPaint":
                col.edit(hd.TOOL_SPHERE_PAINT, [f32(v) for v in fl[:3]], f32(fl[3]))
                applied += 1
            elif t == "EditFill":
                col.edit(hd.TOOL_FILL, [f32(v) for v in fl[:3]], f32(fl[3]))
                applied += 1
            elif t == "EditCopy":
                col.edit(hd.TOOL_COPY, [f32(v) for v in fl[:3]], f32(fl[9]), source=[f32(v) for v in fl[3:6]],
                         dest=[f32(v) for v in fl[6:9]])
                applied += 1
            elif t == "Undo":
                col.undo()
            elif t == "Redo":
                col.redo()
            if t == "EndFrame" or action == len(r):
                break
        frames += 1
        assert n_edits == applied
        assert dag.firstNodeIndex == ot.root, f"frame {frames}"
        want = _trace_params(pos, rot, depth, *info)
        for k in want:
            assert np.allclose(cam[k], want[k], rtol=1e-13, atol=1e-9), (frames, k)
        last_cam = cam
    assert frames == fx["frames"]
    # the last frame, traced from its camera
    tr = hd.DAGTracer(W, H)
    tr.resolve_paths(last_cam, dag)
    opaths, _ = ot.trace_frame(last_cam, W, H, (0.3, 1.0, 0.2), 1.0, fp_mode=0, threads=os.cpu_count() or 4)
    assert np.array_equal(tr.get_paths(), opaths)
    dag.free()
