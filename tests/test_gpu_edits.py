"""GPU parity of the edit pipeline and GC against the reference fixtures and
the oracle."""
import json
import os

import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import workloads
from oracle import pyoracle as po
from tests.helpers import table_digest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def _oracle_of(t, depth, spare_pages=64):
    ot = po.Table(po.default_config(depth, pool_pages=int(t["pool"].size // 512) + spare_pages))
    ot.import_(t)
    return ot


@pytest.mark.parametrize("name", ["ref_d10.json", "ref_d12.json"])
def test_edits_match_reference_fixture(gpu, name):
    fx = _fixture(name)
    depth, bits = fx["depth"], fx["top_bucket_bits"]
    d = hd.HashDAG(depth)
    d.generate_scene(fx["seed"])
    for i, step in enumerate(fx["edits"]):
        s = d.edit_threads(hd.editor_from_tuple((step["tool"], step["center"], step["radius"])))
        assert d.firstNodeIndex == step["root"], i
        assert s.num_voxels == step["num_voxels"], i
        assert s.num_nodes == step["num_nodes"], i
        st = d.level_stats()
        assert st.pages_used + 1 == step["pool_top"], i
        assert [int(v) for v in st.words[:depth - 1]] == step["level_words"], i
        assert table_digest(d.export_table(), depth, bits) == step["digest"], i
    q = fx["queries"]
    assert [int(v) for v in d.get_values(np.array(q["xyz"]))] == q["values"]
    d.remove_stale_nodes()
    g = fx["gc"]
    ot = _oracle_of(d.export_table(), depth)
    assert [int(v) for v in ot.reachable_counts()] == g["reachable"]
    assert ot.fingerprint() == g["fingerprint"]
    st = d.level_stats()
    assert [int(v) for v in st.nodes[:depth - 1]] == [r + 1 for r in g["reachable"]]
    # Post-GC words per level = the full node + the reachable nodes' words +
    # padding at page ends.  The first two are the same on both sides; the
    # padding depends on the re-append order (the reference's hash-set
    # iteration order, here increasing old address), so it is reported
    # beside the reference's and bounded: a node never straddles a page, so
    # at most 8 words (the largest node, 9 words, less one) go unused at the
    # end of each page.  The order also decides each node's new address, so
    # its parent (whose words hold that address) hashes into another bucket:
    # the buckets' sizes, and with them the pages the rebuild maps (pool_top),
    # differ by a few per cent of the pages the GC maps.
    live = [int(v) for v in ot.reachable_words()]
    full = [9] * (depth - 2) + [2]
    ours = [int(v) for v in st.words[:depth - 1]]
    pad_ref = [w - l - f for w, l, f in zip(g["level_words"], live, full)]
    pad_ours = [w - l - f for w, l, f in zip(ours, live, full)]
    sizes = np.asarray(d.export_table()["bucket_sizes"], np.int64)
    print(f"\n{name} post-GC padding words per level: reference {pad_ref}, ours {pad_ours}; "
          f"pool_top reference {g['pool_top']}, ours {st.pages_used + 1}")
    for level in range(depth - 1):
        pages = int(np.ceil(g["level_words"][level] / 512)) + int((sizes > 0).sum())
        assert 0 <= pad_ref[level] <= 8 * pages and 0 <= pad_ours[level] <= 8 * pages, level
    assert [int(v) for v in st.words[:depth - 1]] == g["level_words"]
    gc_pages = g["pool_top"] - fx["edits"][-1]["pool_top"]
    assert abs(st.pages_used + 1 - g["pool_top"]) <= max(8, gc_pages // 20)
    d.free()


def test_gc_and_later_edits_match_oracle(gpu):
    """Canonical GC order on both sides: the rebuilt tables are identical,
    and so are edits made afterwards (whose bucket scans walk the pages as
    GC left them)."""
    depth = 10
    d = hd.HashDAG(depth)
    d.generate_scene(1)
    ot = po.Table(po.default_config(depth))
    ot.load_basic_dag(po.generate_basic_dag(1, depth, workloads.color_tree_levels(depth)))
    edits = workloads.mixed_edits(depth, 24, (4.0, 80.0), seed=17)
    for e in edits[:12]:
        d.edit_threads(hd.editor_from_tuple(e))
        ot.edit(*e)
    assert d.firstNodeIndex == ot.root
    d.remove_stale_nodes()
    ot.gc()
    assert d.firstNodeIndex == ot.root
    assert table_digest(d.export_table(), depth) == table_digest(ot.export(), depth)
    for i, e in enumerate(edits[12:]):
        s = d.edit_threads(hd.editor_from_tuple(e))
        os_ = ot.edit(*e)
        assert d.firstNodeIndex == ot.root, i
        assert (s.num_voxels, s.find_or_add_calls, s.nodes_added) == \
            (os_.num_voxels, os_.find_or_add_calls, os_.nodes_added), i
    assert table_digest(d.export_table(), depth) == table_digest(ot.export(), depth)
    d.free()


def test_gc_keeps_extra_roots(gpu):
    depth = 10
    d = hd.HashDAG(depth)
    d.generate_scene(1)
    fp0 = _oracle_of(d.export_table(), depth).fingerprint()
    r0 = d.firstNodeIndex
    for e in workloads.carve_edits(depth, 4, seed=23):
        d.edit_threads(hd.editor_from_tuple(e))
    fp1 = _oracle_of(d.export_table(), depth).fingerprint()
    (r0_new,) = d.remove_stale_nodes(extra_roots=[r0])
    t = d.export_table()
    ot = _oracle_of(t, depth)
    assert ot.fingerprint() == fp1
    assert ot.fingerprint(r0_new) == fp0
    d.free()


def test_batch_equals_sequential(gpu):
    depth = 10
    edits = workloads.mixed_edits(depth, 16, (4.0, 64.0), seed=31)
    a = hd.HashDAG(depth)
    a.generate_scene(1)
    for e in edits:
        a.edit_threads(hd.editor_from_tuple(e))
    b = hd.HashDAG(depth)
    b.generate_scene(1)
    b.edit_batch([hd.editor_from_tuple(e) for e in edits])
    assert a.firstNodeIndex == b.firstNodeIndex
    assert table_digest(a.export_table(), depth) == table_digest(b.export_table(), depth)
    a.free()
    b.free()


def test_edit_depth15_matches_oracle_sample(gpu):
    """A large carve and fill on the 2^15 scene: occupancy of sampled voxels
    and the edit counters match the oracle run on the exported table."""
    depth = 15
    d = hd.HashDAG(depth)
    d.generate_scene(1)
    ot = _oracle_of(d.export_table(), depth, spare_pages=1 << 18)
    edits = workloads.mixed_edits(depth, 3, (128.0, 384.0), seed=41)
    for e in edits:
        s = d.edit_threads(hd.editor_from_tuple(e))
        os_ = ot.edit(*e)
        assert d.firstNodeIndex == ot.root
        assert s.num_voxels == os_.num_voxels and s.nodes_added == os_.nodes_added
    rng = np.random.default_rng(3)
    c = np.array([e[1] for e in edits])
    q = (c[rng.integers(0, len(c), 20000)] + rng.integers(-400, 400, (20000, 3))).clip(0, (1 << depth) - 1)
    q = q.astype(np.uint32)
    got = d.get_values(q)
    want = np.array([ot.get_value(*map(int, p)) for p in q], np.uint8)
    assert np.array_equal(got, want)
    d.free()


def _stats_tuple(s):
    return (s.num_voxels, s.num_nodes, s.find_or_add_calls, s.nodes_added, s.words_scanned)


@pytest.mark.parametrize("tuning", [(4, 4, 304, 0), (2, 1, 1216, 0), (8, 2, 608, 0), (4, 4, 304, 1), (4, 1, 304, 1),
                                    (4, 2, 304, 1)])
def test_batch_launch_shapes_agree(gpu, tuning):
    """Every launch shape of the batched path, graph per edit (mode 0) or one
    persistent launch (mode 1), gives the plain path's table and per-edit
    counters (depth 12, uneven radii)."""
    depth = 12
    edits = workloads.mixed_edits(depth, 24, (2.0, 200.0), seed=37)
    a = hd.HashDAG(depth)
    a.generate_scene(1)
    plain = [a.edit_threads(hd.editor_from_tuple(e)) for e in edits]
    b = hd.HashDAG(depth)
    b.generate_scene(1)
    b.batch_tuning = tuning
    total, per = b.edit_batch([hd.editor_from_tuple(e) for e in edits], per_edit=True)
    assert [_stats_tuple(s) for s in per] == [_stats_tuple(s) for s in plain]
    assert a.firstNodeIndex == b.firstNodeIndex
    assert table_digest(a.export_table(), depth) == table_digest(b.export_table(), depth)
    assert b.batch_fallbacks() == 0
    ends = [s.host_ms for s in per]
    assert all(x <= y for x, y in zip(ends, ends[1:]))
    a.free()
    b.free()


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_depth15_matches_plain(gpu, mode):
    """A batch of 64 edits of radius 4..512 on the 2^15 scene: same roots,
    per-level words and nodes, counters and sampled occupancy as the
    one-edit path, in both batch modes."""
    depth = 15
    edits = workloads.mixed_edits(depth, 64, (4.0, 512.0), seed=3)
    a = hd.HashDAG(depth)
    a.generate_scene(1)
    plain = [a.edit_threads(hd.editor_from_tuple(e)) for e in edits]
    b = hd.HashDAG(depth)
    b.generate_scene(1)
    b.batch_tuning = (4, 4, 304, mode)
    total, per = b.edit_batch([hd.editor_from_tuple(e) for e in edits], per_edit=True)
    assert [_stats_tuple(s) for s in per] == [_stats_tuple(s) for s in plain]
    assert a.firstNodeIndex == b.firstNodeIndex
    sa, sb = a.level_stats(), b.level_stats()
    assert list(sa.words[:depth]) == list(sb.words[:depth])
    assert list(sa.nodes[:depth]) == list(sb.nodes[:depth])
    assert sa.pages_used == sb.pages_used
    assert b.batch_fallbacks() == 0
    rng = np.random.default_rng(5)
    q = rng.integers(0, 1 << depth, (50000, 3)).astype(np.uint32)
    assert np.array_equal(a.get_values(q), b.get_values(q))
    a.free()
    b.free()


def test_autotune_leaves_table_unchanged(gpu):
    depth = 12
    d = hd.HashDAG(depth)
    d.generate_scene(1)
    before = table_digest(d.export_table(), depth)
    r0 = d.firstNodeIndex
    edits = [hd.editor_from_tuple(e) for e in workloads.mixed_edits(depth, 8, (2.0, 100.0), seed=41)]
    t, ms = d.autotune_batch(edits)
    assert t.foa_warps in (2, 4, 8) and t.probe_words in (1, 2, 4) and ms > 0
    assert d.firstNodeIndex == r0
    assert table_digest(d.export_table(), depth) == before
    cur = d.batch_tuning
    assert (cur.foa_warps, cur.probe_words, cur.grid_blocks, cur.mode) == \
        (t.foa_warps, t.probe_words, t.grid_blocks, t.mode)
    d.free()
