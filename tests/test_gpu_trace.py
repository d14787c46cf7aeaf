"""GPU parity of scene ingest and traversal against the oracle and the
reference fixtures (tests/golden)."""
import hashlib
import json
import os

import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import scene, workloads
from oracle import pyoracle as po
from tests.helpers import table_digest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LIGHT_REF = (0.3, 1.0, 0.5)   # the reference's hard-coded sun (tracer.cu:546-549)
LIGHT_BENCH = (0.3, 1.0, 0.2)


def _fixture(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


_cache = {}


def gpu_dag(depth):
    if depth not in _cache:
        d = hd.HashDAG(depth)
        d.generate_scene(workloads.SEED_SCENE)
        _cache[depth] = d
    return _cache[depth]


def oracle_table(depth):
    key = ("oracle", depth)
    if key not in _cache:
        t = po.Table(po.default_config(depth))
        t.load_basic_dag(po.generate_basic_dag(workloads.SEED_SCENE, depth, workloads.color_tree_levels(depth)))
        _cache[key] = t
    return _cache[key]


@pytest.mark.parametrize("depth", [8, 10, 12])
def test_generator_matches_oracle(gpu, depth):
    d = gpu_dag(depth)
    words = d.export_basic_dag()
    ref = po.generate_basic_dag(workloads.SEED_SCENE, depth, workloads.color_tree_levels(depth))
    assert words.size == ref.size
    assert np.array_equal(words, ref)


@pytest.mark.parametrize("name", ["ref_d10.json", "ref_d12.json"])
def test_ingest_matches_reference_fixture(gpu, name):
    fx = _fixture(name)
    depth = fx["depth"]
    d = gpu_dag(depth)
    assert hashlib.sha256(d.export_basic_dag().tobytes()).hexdigest() == fx["basic_dag_sha256"]
    t = d.export_table()
    assert int(t["root"]) == fx["load"]["root"]
    assert [int(v) for v in t["full_nodes"][1:depth - 1]] == fx["load"]["full_nodes"]
    assert table_digest(t, depth, fx["top_bucket_bits"]) == fx["load"]["digest"]
    st = d.level_stats()
    assert [int(v) for v in st.words[:depth - 1]] == fx["load"]["level_words"]
    assert st.pages_used + 1 == fx["load"]["pool_top"]


def test_load_from_host_basic_dag(gpu):
    depth = 10
    words = po.generate_basic_dag(workloads.SEED_SCENE, depth, workloads.color_tree_levels(depth))
    d = hd.HashDAG(depth)
    d.load_from_DAG(words)
    fx = _fixture("ref_d10.json")
    assert table_digest(d.export_table(), depth, 10) == fx["load"]["digest"]
    d.free()


@pytest.mark.parametrize("fp_mode", [0, 1])
def test_primary_and_shadow_match_oracle_1080p(gpu, fp_mode):
    depth, W, H = 10, 1920, 1080
    d = gpu_dag(depth)
    d.set_fp_mode(fp_mode)
    cam = workloads.orbit_camera(depth, W, H)
    tr = hd.DAGTracer(W, H)
    tr.resolve_paths(cam, d)
    tr.resolve_shadows(cam, d, 1.0, LIGHT_REF)
    paths, shadows = tr.get_paths(), tr.get_shadows()
    ot = oracle_table(depth)
    opaths, omask = ot.trace_frame(cam, W, H, LIGHT_REF, 1.0, fp_mode=fp_mode, threads=os.cpu_count() or 4)
    hits = int((paths[..., :3] != 0).any(-1).sum())
    assert hits > W * H // 50
    assert np.array_equal(paths, opaths)
    assert np.array_equal(shadows, omask)
    d.set_fp_mode(0)


def test_get_values_match_scene_function(gpu):
    depth = 12
    d = gpu_dag(depth)
    rng = np.random.default_rng(21)
    e = 1 << depth
    q = rng.integers(0, e, (20000, 3))
    q[:, 1] = np.clip(scene.height(1, depth, q[:, 0], q[:, 2]) + rng.integers(-64, 64, len(q)), 0, e - 1)
    got = d.get_values(q)
    want = scene.solid(1, depth, q[:, 0], q[:, 1], q[:, 2]).astype(np.uint8)
    assert np.array_equal(got, want)


def test_scene_depth15_properties(gpu):
    depth = 15
    d = gpu_dag(depth)
    st = d.level_stats()
    assert st.nodes[depth - 2] > 1000
    rng = np.random.default_rng(5)
    e = 1 << depth
    q = rng.integers(0, e, (50000, 3))
    q[:, 1] = np.clip(scene.height(1, depth, q[:, 0], q[:, 2]) + rng.integers(-8, 8, len(q)), 0, e - 1)
    got = d.get_values(q)
    want = scene.solid(1, depth, q[:, 0], q[:, 1], q[:, 2]).astype(np.uint8)
    assert np.array_equal(got, want)


def test_trace_depth15_rows_match_oracle(gpu):
    """4K frame of the 2^15 scene on the GPU; a band of rows re-traced by the
    oracle on the exported table."""
    depth, W, H = 15, 3840, 2160
    d = gpu_dag(depth)
    cam = workloads.catmull_rom_path(depth, 64, W, H)[5]
    tr = hd.DAGTracer(W, H)
    tr.resolve_paths(cam, d)
    tr.resolve_shadows(cam, d, 1.0, LIGHT_BENCH)
    paths, shadows = tr.get_paths(), tr.get_shadows()
    t = d.export_table()
    cfg = po.default_config(depth, pool_pages=int(t["pool"].size // 512) + 16)
    ot = po.Table(cfg)
    ot.import_(t)
    rows = (1000, 1064)  # pixel rows; output rows H-1-y
    opaths, omask = ot.trace_frame(cam, W, H, LIGHT_BENCH, 1.0, fp_mode=0, threads=os.cpu_count() or 4,
                                   rows=rows)
    out_rows = slice(H - rows[1], H - rows[0])
    assert np.array_equal(paths[out_rows], opaths[out_rows])
    assert np.array_equal(shadows[out_rows], omask[out_rows])


def test_trace_views_equals_single_views(gpu):
    """hd_trace_views (several views per launch) gives each view the paths
    and shadow mask of hd_trace_primary / hd_trace_shadow."""
    import ctypes as C
    import torch
    from hashdag_gb300 import _capi
    depth, W, H, V = 12, 640, 360, 5
    d = hd.HashDAG(depth)
    d.generate_scene(1)
    poses = workloads.catmull_rom_path(depth, V, W, H)
    cams = (_capi.Camera * V)(*[_capi.Camera.from_params(p) for p in poses])
    paths = torch.zeros(V * W * H * 4, dtype=torch.int32, device="cuda")
    mask = torch.zeros(V * W * H, dtype=torch.uint8, device="cuda")
    light = (C.c_float * 3)(0.3, 1.0, 0.2)
    ms = (C.c_float * 2)()
    d._check(_capi.lib().hd_trace_views(d.handle, cams, V, W, H, paths.data_ptr(), light, 1.0, mask.data_ptr(), ms))
    tr = hd.DAGTracer(W, H)
    for v in range(V):
        tr.resolve_paths(poses[v], d)
        tr.resolve_shadows(poses[v], d)
        got_p = paths[v * W * H * 4:(v + 1) * W * H * 4].cpu().numpy().view(np.uint32).reshape(H, W, 4)
        got_m = mask[v * W * H:(v + 1) * W * H].cpu().numpy().reshape(H, W)
        assert np.array_equal(got_p, tr.get_paths().reshape(H, W, 4)), v
        assert np.array_equal(got_m, tr.get_shadows()), v
    assert ms[0] > 0 and ms[1] > 0
    d.free()


@pytest.mark.parametrize("chunk,V", [(0, 5), (1, 5), (3, 5), (0, 14), (0, 8)])
def test_trace_views_host_equals_device_views(gpu, chunk, V):
    """hd_trace_views_host (chunks of views, copies to host memory on a
    second stream; or, chunk 0, paths written straight into the pinned
    buffer, views 5-7 of every 8 copied there during the shadow launch)
    gives every view's paths and mask exactly as hd_trace_views does on
    device buffers."""
    import ctypes as C

    import torch
    depth, W, H = 10, 160, 96
    dag = hd.HashDAG(depth)
    dag.generate_scene(workloads.SEED_SCENE)
    poses = workloads.catmull_rom_path(depth, V, W, H)
    cams = (hd._capi.Camera * V)(*[hd._capi.Camera.from_params(p) for p in poses])
    light = (C.c_float * 3)(*LIGHT_BENCH)
    L = hd._capi.lib()
    d_paths = torch.zeros(V * W * H * 4, dtype=torch.int32, device="cuda")
    d_mask = torch.zeros(V * W * H, dtype=torch.uint8, device="cuda")
    ms = (C.c_float * 2)()
    dag._check(L.hd_trace_views(dag.handle, cams, V, W, H, d_paths.data_ptr(), light, 1.0, d_mask.data_ptr(), ms))
    h_paths = torch.full((V * W * H * 4,), -1, dtype=torch.int32, pin_memory=True)
    h_mask = torch.full((V * W * H,), 7, dtype=torch.uint8, pin_memory=True)
    dag._check(L.hd_trace_views_host(dag.handle, cams, V, W, H, h_paths.data_ptr(), light, 1.0, h_mask.data_ptr(),
                                     chunk, None))
    assert torch.equal(h_paths, d_paths.cpu())
    assert torch.equal(h_mask, d_mask.cpu())
    dag.free()


_REF_TRACE = json.load(open(os.path.join(GOLDEN, "ref_trace.json")))
_REF_CASES = [(s["depth"], f["name"]) for s in _REF_TRACE["scenes"] for f in s["frames"]]


@pytest.mark.parametrize("depth,name", _REF_CASES)
def test_trace_equals_reference_tracer(gpu, depth, name):
    """Paths and shadow masks of whole 1920 x 1080 frames equal the
    reference's own trace_paths / trace_shadows hit test (fp_mode 0)."""
    s = next(s for s in _REF_TRACE["scenes"] if s["depth"] == depth)
    f = next(f for f in s["frames"] if f["name"] == name)
    W, H = s["width"], s["height"]
    d = gpu_dag(depth)
    d.set_fp_mode(0)
    try:
        tr = hd.DAGTracer(W, H)
        tr.resolve_paths(f["camera"], d)
        tr.resolve_shadows(f["camera"], d, f["bias"], tuple(f["light"]))
        paths, mask = np.ascontiguousarray(tr.get_paths()), np.ascontiguousarray(tr.get_shadows())
    finally:
        d.set_fp_mode(0)
    assert int((paths[..., :3] != 0).any(-1).sum()) == f["hits"]
    assert hashlib.sha256(paths.tobytes()).hexdigest() == f["paths_sha256"]
    assert hashlib.sha256(mask.tobytes()).hexdigest() == f["mask_sha256"]


def test_trace_views_equal_reference_tracer(gpu):
    """Every frame of a scene in one hd_trace_views launch (fp_mode 0), per
    view equal to the reference's frames."""
    import ctypes as C
    import torch
    from hashdag_gb300 import _capi
    s = next(s for s in _REF_TRACE["scenes"] if s["depth"] == 10)
    frames = [f for f in s["frames"] if f["light"] == s["frames"][0]["light"]]
    W, H, V = s["width"], s["height"], len(frames)
    d = gpu_dag(10)
    d.set_fp_mode(0)
    try:
        cams = (_capi.Camera * V)(*[_capi.Camera.from_params(f["camera"]) for f in frames])
        paths = torch.zeros(V * W * H * 4, dtype=torch.int32, device="cuda")
        mask = torch.zeros(V * W * H, dtype=torch.uint8, device="cuda")
        light = (C.c_float * 3)(*frames[0]["light"])
        d._check(_capi.lib().hd_trace_views(d.handle, cams, V, W, H, paths.data_ptr(), light, 1.0, mask.data_ptr(),
                                            None))
        paths, mask = paths.cpu().numpy().view(np.uint32), mask.cpu().numpy()
    finally:
        d.set_fp_mode(0)
    for v, f in enumerate(frames):
        assert hashlib.sha256(paths[v * W * H * 4:(v + 1) * W * H * 4].tobytes()).hexdigest() == f["paths_sha256"]
        assert hashlib.sha256(mask[v * W * H:(v + 1) * W * H].tobytes()).hexdigest() == f["mask_sha256"], f["name"]
