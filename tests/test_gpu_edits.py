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
