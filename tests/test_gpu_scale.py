"""Parity at the benchmark's own scale (the 2^15 scenes) against the oracle.

* The batched-edit workload: 256 edits (50 % sphere carve, 30 % sphere
  fill, 20 % box fill, radii log-uniform in [4, 512]) through the batched
  form in one call, against the oracle applying them one by one as the
  reference's edit_threads does (hash_dag.h:255-405): per-edit counters,
  the root, per-level words and nodes, the pages in use, the whole table by
  virtual address and voxels sampled around every edit.
* The colour workload, scaled down in count (32 paints, radius
  log-uniform in [8, 256], 4 copies of 256^3 regions moved by up to 2048
  voxels) but not in size, on the coloured 2^15 shell scene, then a GC:
  roots and counters per edit, occupancy and colours of voxels sampled
  around every edit, and after the GC the root, per-level words and nodes,
  the pages in use and the whole table (remove_stale_nodes,
  hash_dag.h:407-547; colours, variable_weight_size_colors.h:557-689).

Both scenes are generated on both sides; the oracle's threaded generator
builds the same words as the GPU's (checked first).  Each test takes one to
two minutes of host time for the oracle.
"""
import os

import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import workloads
from oracle import pyoracle as po
from tests.helpers import table_digest

pytestmark = pytest.mark.gpu
DEPTH = 15
THREADS = os.cpu_count() or 4


def _oracle_scene(d, shell):
    """The oracle's table of the same scene, its words checked against the
    GPU's BasicDAG export, in a pool as large as the GPU context's."""
    ctl = workloads.color_tree_levels(DEPTH)
    words = po.generate_basic_dag(workloads.SEED_SCENE, DEPTH, ctl, flags=po.SCENE_SHELL if shell else 0,
                                  threads=THREADS)
    assert np.array_equal(d.export_basic_dag(), words)
    ot = po.Table(po.default_config(DEPTH, pool_pages=int(d.config.pool_pages)))
    ot.load_basic_dag(words)
    del words
    assert d.firstNodeIndex == ot.root
    return ot


def _samples(edits, n, seed):
    rng = np.random.default_rng(seed)
    c = np.array([e[1] for e in edits], np.float64)
    r = np.array([e[2] for e in edits], np.float64)
    k = rng.integers(0, len(edits), n)
    off = rng.uniform(-1.0, 1.0, (n, 3)) * (r[k, None] + 8.0)
    return np.clip(np.floor(c[k] + off), 0, (1 << DEPTH) - 1).astype(np.uint32)


def _same_tables(d, ot):
    gs, os_ = d.level_stats(), ot.level_stats()
    assert d.firstNodeIndex == ot.root
    assert list(gs.words[:DEPTH]) == list(os_.words[:DEPTH])
    assert list(gs.nodes[:DEPTH]) == list(os_.nodes[:DEPTH])
    assert gs.pages_used + 1 == ot.pool_top
    bits = workloads.top_bucket_bits(DEPTH)
    assert table_digest(d.export_table(), DEPTH, bits) == table_digest(ot.export(), DEPTH, bits)


def test_batch_of_256_edits_depth15_matches_oracle(gpu):
    d = hd.HashDAG(DEPTH)
    d.generate_scene(workloads.SEED_SCENE)
    ot = _oracle_scene(d, shell=False)
    edits = workloads.mixed_edits(DEPTH, 256, (4.0, 512.0))
    total, per = d.edit_batch([hd.editor_from_tuple(e) for e in edits], per_edit=True)
    vox = 0
    for i, e in enumerate(edits):
        s = ot.edit(*e)
        assert (per[i].num_voxels, per[i].num_nodes, per[i].find_or_add_calls, per[i].nodes_added) == \
            (s.num_voxels, s.num_nodes, s.find_or_add_calls, s.nodes_added), i
        vox += s.num_voxels
    assert total.num_voxels == vox
    _same_tables(d, ot)
    q = _samples(edits, 50000, 5)
    want = np.array([ot.get_value(*map(int, p)) for p in q], np.uint8)
    assert np.array_equal(d.get_values(q), want)
    assert 0 < int(want.sum()) < len(q)
    d.free()


def test_paints_copies_gc_depth15_matches_oracle(gpu):
    d = hd.HashDAG(DEPTH)
    d.generate_scene(workloads.SEED_SCENE, shell=True)
    d.colors_from_scene(workloads.SEED_COLORS)
    ot = _oracle_scene(d, shell=True)
    col = po.Colors(ot)
    col.from_scene(workloads.SEED_COLORS, threads=THREADS)
    edits = workloads.paint_copy_edits(DEPTH, n_paint=32, n_copy=4)
    assert [e[0] for e in edits].count(5) == 4 and max(e[2] for e in edits if e[0] == 5) == 128.0
    for i, e in enumerate(edits):
        s = d.edit_threads(hd.editor_from_tuple(e))
        if e[0] == 4:
            os_ = col.edit(4, e[1], e[2], rgb=e[3])
        else:
            os_ = col.edit(5, e[1], e[2], source=e[3], dest=e[4])
        assert d.firstNodeIndex == ot.root, i
        assert (s.num_voxels, s.num_nodes) == (os_.num_voxels, os_.num_nodes), i
    # the 12^3 voxels around every paint's centre (a surface voxel) and
    # around both ends of every copy, plus voxels anywhere in the edits
    ends = [e[1] for e in edits] + [tuple(e[1][k] + e[4][k] for k in range(3)) for e in edits if e[0] == 5]
    g = np.stack(np.meshgrid(*[np.arange(-6, 6)] * 3, indexing="ij"), -1).reshape(-1, 3)
    boxes = (np.floor(np.array(ends))[:, None, :] + g[None]).reshape(-1, 3)
    q = np.concatenate([np.clip(boxes, 0, (1 << DEPTH) - 1).astype(np.uint32),
                        _samples([(e[0], e[1], e[2]) for e in edits], 20000, 9)])

    def state():
        v = d.get_values(q)
        want = np.array([ot.get_value(*map(int, p)) for p in q], np.uint8)
        assert np.array_equal(v, want)
        p = q[v != 0]
        assert len(p) > 1000
        got = d.get_colors(p)
        wc = np.array([col.get_color(*map(int, x)) for x in p], np.uint32).reshape(-1, 3)
        assert np.array_equal(got, wc)
        return v, got

    before = state()
    d.remove_stale_nodes()
    ot.gc()
    _same_tables(d, ot)
    after = state()
    assert all(np.array_equal(a, b) for a, b in zip(before, after))
    d.free()
