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
from oracle import pyoracle as po
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


def _stream(depth, n):
    """n edits of a seeded stream, and the pages in use after each of them
    without a GC (the scene's first)."""
    edits = workloads.mixed_edits(depth, n, (16.0, 96.0), seed=23)
    ref = _edited([], depth)
    pages = [ref.level_stats().pages_used]
    for e in edits:
        ref.edit_threads(hd.editor_from_tuple(e))
        pages.append(ref.level_stats().pages_used)
    return edits, pages, ref


def test_release_gc_lets_a_small_pool_take_an_edit_stream(gpu):
    """A pool too small for an edit stream without page reuse takes the whole
    stream when every edit that finds it full is retried after a releasing
    GC.  The GC's rebuild re-hashes the interior levels (children
    remapped), so a bucket can need a page it never had: a page reserve
    (hd_set_page_reserve) keeps room for it once edits have filled the
    pool."""
    depth, reserve = 10, 64
    n = 64
    while True:  # enough edits that the stream's garbage dwarfs one edit
        edits, pages, ref = _stream(depth, n)
        live = hd.HashDAG(depth)
        live.import_table(ref.export_table())
        live.remove_stale_nodes(release_pages=True)
        live_pages = live.level_stats().pages_used
        live.free()
        step = max(b - a for a, b in zip(pages, pages[1:]))
        pool = live_pages + 1 + reserve + 4 * step
        if pool - 1 < pages[-1] - 4 * step or n >= 512:
            break
        ref.free()
        n *= 2
    assert pool - 1 < pages[-1], "the stream must not fit the pool without page reuse"
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
    # edits stop at the reserve; a releasing GC then frees the garbage and
    # the edit lands on the retry
    d = hd.HashDAG(config=hd.default_config(depth, pool_pages=pool))
    d.generate_scene(workloads.SEED_SCENE)
    d.set_page_reserve(reserve)
    gcs = 0
    for e in edits:
        try:
            d.edit_threads(hd.editor_from_tuple(e))
        except hd.HashDagError as err:
            assert err.status == _capi.HD_ERR_POOL_FULL and "reserve" in str(err), str(err)
            assert d.level_stats().pages_used + 1 <= pool - reserve
            d.remove_stale_nodes(release_pages=True)
            gcs += 1
            d.edit_threads(hd.editor_from_tuple(e))
    assert gcs > 0
    q = np.random.default_rng(7).integers(0, 1 << depth, (40000, 3)).astype(np.uint32)
    assert np.array_equal(d.get_values(q), ref.get_values(q))
    # the same voxels everywhere (the GCs moved nodes, so addresses differ,
    # and with them which equal nodes the scans' visibility rule duplicates)
    fp = []
    for x in (d, ref):
        t = x.export_table()
        ot = po.Table(po.default_config(depth, pool_pages=int(t["pool"].size // 512) + 8))
        ot.import_(t)
        fp.append(ot.fingerprint())
    assert fp[0] == fp[1]
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
