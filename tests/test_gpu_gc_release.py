"""The page-releasing GC (HD_GC_RELEASE_PAGES), which has no reference
counterpart (the reference's poolTop only grows, hash_table.h:794-809).

After it, every bucket holds what the default GC leaves (same sizes, same
words at the same virtual addresses, same root), fewer pages are in use, and
the freed pages serve later edits, which land exactly where they land after
the default GC.  A pool too small for a stream of edits without page reuse
takes the whole stream when a releasing GC runs between the edits.
"""
import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import _capi, workloads
from tests.helpers import table_digest

pytestmark = pytest.mark.gpu
DEPTH = 12


def _edited(edits, depth=DEPTH, **cfg):
    d = hd.HashDAG(config=hd.default_config(depth, **cfg))
    d.generate_scene(workloads.SEED_SCENE)
    for e in edits:
        d.edit_threads(hd.editor_from_tuple(e))
    return d


def test_release_gc_keeps_buckets_and_frees_pages(gpu):
    edits = workloads.mixed_edits(DEPTH, 32, (8.0, 200.0), seed=17)
    a, b = _edited(edits), _edited(edits)
    a.remove_stale_nodes()
    before = b.level_stats().pages_used
    b.remove_stale_nodes(release_pages=True)
    sa, sb = a.level_stats(), b.level_stats()
    assert a.firstNodeIndex == b.firstNodeIndex
    assert list(sa.words[:DEPTH]) == list(sb.words[:DEPTH])
    ta, tb = a.export_table(), b.export_table()
    assert table_digest(ta, DEPTH, 12) == table_digest(tb, DEPTH, 12)
    # (the default GC can claim a few pages: its order pads pages differently)
    assert sb.pages_used < sa.pages_used and sb.pages_used < before
    # later edits draw on the freed pages and land where they land after the
    # default GC
    more = workloads.mixed_edits(DEPTH, 16, (8.0, 200.0), seed=18)
    for e in more:
        ra = a.edit_threads(hd.editor_from_tuple(e))
        rb = b.edit_threads(hd.editor_from_tuple(e))
        assert a.firstNodeIndex == b.firstNodeIndex
        assert (ra.num_voxels, ra.nodes_added) == (rb.num_voxels, rb.nodes_added)
    assert table_digest(a.export_table(), DEPTH, 12) == table_digest(b.export_table(), DEPTH, 12)
    assert b.level_stats().pages_used < a.level_stats().pages_used
    a.free()
    b.free()


def test_release_gc_lets_a_small_pool_take_an_edit_stream(gpu):
    depth = 10
    edits = workloads.mixed_edits(depth, 64, (16.0, 160.0), seed=23)
    # the stream without a GC: pages each edit claims, pages at the end
    ref = _edited([], depth)
    scene_pages = ref.level_stats().pages_used
    step = []
    for e in edits:
        before = ref.level_stats().pages_used
        ref.edit_threads(hd.editor_from_tuple(e))
        step.append(ref.level_stats().pages_used - before)
    total = ref.level_stats().pages_used
    live = hd.HashDAG(depth)
    live.import_table(ref.export_table())
    live.remove_stale_nodes(release_pages=True)
    live_pages = live.level_stats().pages_used
    live.free()
    # free pages to keep: an edit's worth twice over, and room for the GC's
    # rebuild (its order pads pages differently from the edits')
    need = 2 * max(step) + total // 16 + 64
    pool = live_pages + 1 + 2 * need
    assert pool - 1 < total, "the stream must not fit the pool without page reuse"
    # without page reuse the pool runs out partway through the stream
    plain = hd.HashDAG(config=hd.default_config(depth, pool_pages=pool))
    plain.generate_scene(workloads.SEED_SCENE)
    refused = 0
    for e in edits:
        try:
            plain.edit_threads(hd.editor_from_tuple(e))
        except hd.HashDagError as err:
            assert err.status == _capi.HD_ERR_POOL_FULL
            refused += 1
    assert refused > 0
    plain.free()
    # with a releasing GC whenever fewer than `need` pages are free, every
    # edit lands and the scene equals the unconstrained one
    d = hd.HashDAG(config=hd.default_config(depth, pool_pages=pool))
    d.generate_scene(workloads.SEED_SCENE)
    gcs = 0
    for e in edits:
        if pool - 1 - d.level_stats().pages_used < need:
            d.remove_stale_nodes(release_pages=True)
            gcs += 1
        d.edit_threads(hd.editor_from_tuple(e))
    assert gcs > 0 and scene_pages < pool
    q = np.random.default_rng(7).integers(0, 1 << depth, (40000, 3)).astype(np.uint32)
    assert np.array_equal(d.get_values(q), ref.get_values(q))
    d.free()
    ref.free()


def test_gc_refuses_when_its_rebuild_does_not_fit(gpu):
    """The GC first runs its rebuild dry (same order, same addresses) and
    counts the pages it would map; when they are not free it refuses before
    it changes anything (HD_ERR_POOL_FULL) and the table stays as it was.
    Here: an edited table imported into a pool with no free page."""
    depth = 10
    edits = workloads.mixed_edits(depth, 16, (16.0, 96.0), seed=29)
    src = _edited(edits, depth)
    t = src.export_table()
    src.free()
    d = hd.HashDAG(config=hd.default_config(depth, pool_pages=int(t["pool"].size // 512)))
    d.import_table(t)
    root = d.firstNodeIndex
    before = table_digest(d.export_table(), depth, 10)
    with pytest.raises(hd.HashDagError) as ei:
        d.remove_stale_nodes()
    assert ei.value.status == _capi.HD_ERR_POOL_FULL and "unchanged" in str(ei.value), str(ei.value)
    assert d.firstNodeIndex == root and table_digest(d.export_table(), depth, 10) == before
    d.free()
