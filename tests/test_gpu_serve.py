"""The serving loop: in the continuous mix (renders in flight on their own
streams while edits run, GCs in between) every render equals the same render
made alone on the same state, and the edits leave the same scene as applying
them one by one."""
import ctypes as C

import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import workloads

pytestmark = pytest.mark.gpu


def _requests(trace, zero_time=False):
    out = []
    for kind, t, p in trace:
        t = 0.0 if zero_time else t
        if kind == "edit":
            tool, centre, radius, rgb = p
            ed = hd.SpherePaintEditor(centre, radius, rgb) if tool == 4 else hd.editor_from_tuple((tool, centre, radius))
            out.append(hd.edit_request(t, ed))
        else:
            w, h, cam = p
            out.append(hd.render_request(t, w, h, cam))
    return out


def _scene(depth, pool_pages=0):
    cfg = hd.default_config(depth)
    if pool_pages:
        cfg.pool_pages = pool_pages
    d = hd.HashDAG(config=cfg)
    d.generate_scene(1, shell=True)
    d.colors_from_scene(2)
    return d


def _digest(d, pts):
    v = d.get_values(pts)
    p = pts[v != 0]
    return v.tobytes(), d.get_colors(p).tobytes()


def _sample(trace, depth, rng):
    pts = []
    for kind, _, p in trace:
        if kind == "edit":
            c = np.array(p[1], np.int64)
            pts.append(np.clip(c + rng.integers(-48, 49, (400, 3)), 0, (1 << depth) - 1))
    return np.concatenate(pts).astype(np.uint32)


@pytest.mark.parametrize("gc_fraction", [0.0, 0.98])
def test_mix_equals_alone(gpu, gc_fraction):
    depth = 10
    trace = workloads.serving_trace(depth, 48, 2000.0, r_range=(4.0, 64.0),
                                    resolutions=((320, 180), (640, 360), (1280, 720)))
    d = _scene(depth)
    if gc_fraction:
        # a pool a little larger than the scene: free words stay below the
        # threshold, so the loop collects before every edit
        used = d.level_stats().pages_used
        d.free()
        d = _scene(depth, pool_pages=used + 4096)
    reqs = _requests(trace)
    res, st = d.serve(reqs, continuous=True, max_renders=3, realtime=False, gc_free_fraction=gc_fraction)
    assert st.edits + st.renders == len(reqs)
    assert (st.gcs > 0) == (gc_fraction > 0)
    # replay one at a time: every render at the state it saw in the mix
    edits = [i for i, r in enumerate(reqs) if r.kind == 0]
    renders = sorted((i for i, r in enumerate(reqs) if r.kind == 1), key=lambda i: (res[i].edits_before, i))
    order, k = [], 0
    for n_done in range(len(edits) + 1):
        while k < len(renders) and res[renders[k]].edits_before == n_done:
            order.append(renders[k])
            k += 1
        if n_done < len(edits):
            order.append(edits[n_done])
    assert sorted(order) == list(range(len(reqs)))
    alone = _requests([trace[i] for i in order], zero_time=True)
    d2 = _scene(depth)
    res2, _ = d2.serve(alone, continuous=False, realtime=False, gc_free_fraction=0.0)
    for pos, i in enumerate(order):
        assert res2[pos].checksum == res[i].checksum, (pos, i)
    pts = _sample(trace, depth, np.random.default_rng(0))
    assert _digest(d, pts) == _digest(d2, pts)
    d.free()
    d2.free()


def test_realtime_trace_reports_latencies(gpu):
    depth = 10
    trace = workloads.serving_trace(depth, 30, 400.0, r_range=(4.0, 48.0),
                                    resolutions=((640, 360), (1280, 720)))
    d = _scene(depth)
    res, st = d.serve(_requests(trace), continuous=True, realtime=True)
    assert st.edits + st.renders == 30 and st.edit_p99_ms >= st.edit_p50_ms >= 0
    assert all(r.end_ms >= t - 1e-3 for r, (_, t, _) in zip(res, trace))
    d.free()


def _geometry_requests(depth, n, rate, seed=5, r_range=(4.0, 64.0)):
    trace = workloads.serving_trace(depth, n, rate, seed=seed, r_range=r_range,
                                    resolutions=((320, 180), (640, 360)))
    # no colours: paints become fills
    return [(k, t, ((1 if p[0] == 4 else p[0]),) + tuple(p[1:])) if k == "edit" else (k, t, p)
            for k, t, p in trace]


def test_batched_mix_equals_alone(gpu):
    """Continuous policy on a scene without colours: the edits queued at a
    moment run as one persistent batch while renders are in flight; every
    render equals the same render alone on the state it saw, the scene
    equals one-by-one application."""
    depth = 10
    trace = _geometry_requests(depth, 64, 4000.0)
    d = hd.HashDAG(depth)
    d.generate_scene(1)
    reqs = _requests(trace)
    res, st = d.serve(reqs, continuous=True, max_renders=2, realtime=False, gc_free_fraction=0.0, batch_edits=True)
    assert st.edits + st.renders == len(reqs) and st.refused == 0
    edits = [i for i, r in enumerate(reqs) if r.kind == 0]
    renders = sorted((i for i, r in enumerate(reqs) if r.kind == 1), key=lambda i: (res[i].edits_before, i))
    order, k = [], 0
    for n_done in range(len(edits) + 1):
        while k < len(renders) and res[renders[k]].edits_before == n_done:
            order.append(renders[k])
            k += 1
        if n_done < len(edits):
            order.append(edits[n_done])
    alone = _requests([trace[i] for i in order], zero_time=True)
    d2 = hd.HashDAG(depth)
    d2.generate_scene(1)
    res2, _ = d2.serve(alone, continuous=False, realtime=False, gc_free_fraction=0.0)
    for pos, i in enumerate(order):
        assert res2[pos].checksum == res[i].checksum, (pos, i)
    assert d.firstNodeIndex == d2.firstNodeIndex
    d.free()
    d2.free()


def test_pool_gated_admission_with_page_release(gpu):
    """A pool too small for the trace without page reuse: without GCs the
    loop refuses edits once the pool is full; with the page-releasing GC
    (below 5 % free pages, and on a full pool before a retry) it takes every
    edit and ends on the same voxels.  The undo history is kept to 8 frames:
    the GC keeps every state the history can return to, so a longer history
    than the pool's slack would keep the garbage alive."""
    depth = 10
    trace = [x for x in _geometry_requests(depth, 120, 4000.0, seed=9, r_range=(16.0, 96.0)) if x[0] == "edit"]
    probe = hd.HashDAG(depth)
    probe.generate_scene(1)
    res0, _ = probe.serve(_requests(trace), continuous=False, realtime=False, gc_free_fraction=0.0)
    total = probe.level_stats().pages_used
    probe.remove_stale_nodes(release_pages=True)
    live = probe.level_stats().pages_used
    probe.free()
    pool = live + 1 + (total - live) // 3
    outcomes = {}
    for gc_free, release in ((0.0, False), (0.05, True)):
        d = hd.HashDAG(config=hd.default_config(depth, pool_pages=pool))
        d.generate_scene(1)
        d.set_undo_capacity(8)
        res, st = d.serve(_requests(trace), continuous=True, realtime=False, gc_free_fraction=gc_free,
                          release_pages=release, batch_edits=False)
        outcomes[release] = (st.refused, st.gcs)
        if release:
            assert [r.num_voxels for r in res] == [r.num_voxels for r in res0]
            q = np.random.default_rng(3).integers(0, 1 << depth, (40000, 3)).astype(np.uint32)
            probe = hd.HashDAG(depth)
            probe.generate_scene(1)
            for e in trace:
                probe.edit_threads(hd.editor_from_tuple(e[2][:3]))
            assert np.array_equal(d.get_values(q), probe.get_values(q))
            probe.free()
        d.free()
    assert outcomes[False][0] > 0          # the pool ran out without page reuse
    assert outcomes[True][0] == 0 and outcomes[True][1] > 0
