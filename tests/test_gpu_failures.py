"""Edits that run out of room: a pool without free pages, a bucket at its
capacity.

The reference does not check either in release builds: allocate_page
(hash_table.h:794-809) takes poolTop++ past the pool, and add_leaf_node /
add_interior_node (hash_table.h:359-468) write past the bucket
(checks only under ENABLE_CHECKS, hash_table.h:393, :461).  The library
refuses the edit instead: HD_ERR_POOL_FULL / HD_ERR_BUCKET_FULL with a
message, the root left as it was, poolTop never past the pool, no node built
over an unresolved child.  Nodes the failed edit appended before it stopped
stay in their buckets, unreachable; a GC removes them, after which the table
equals the GC of the same scene without the failed edit.  The oracle (the
reference's algorithm with the same checks) fails on the same edit.
"""
import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import _capi, workloads
from oracle import pyoracle as po
from tests.helpers import table_digest

pytestmark = pytest.mark.gpu
DEPTH = 10
W, H = 320, 180


def _words():
    return po.generate_basic_dag(workloads.SEED_SCENE, DEPTH, workloads.color_tree_levels(DEPTH))


def _frame(d):
    cam = workloads.orbit_camera(DEPTH, W, H)
    tr = hd.DAGTracer(W, H)
    tr.resolve_paths(cam, d)
    tr.resolve_shadows(cam, d, 1.0, (0.3, 1.0, 0.2))
    return np.ascontiguousarray(tr.get_paths()).copy(), np.ascontiguousarray(tr.get_shadows()).copy()


def _oracle(cfg_kw, words):
    cfg = po.default_config(DEPTH)
    for k, v in cfg_kw.items():
        setattr(cfg, k, v)
    t = po.Table(cfg)
    t.load_basic_dag(words)
    return t


def test_pool_full_edit_is_refused_and_table_stays_usable(gpu):
    words = _words()
    top = _oracle({}, words).pool_top           # pages the scene needs (+ the null page)
    edit = hd.SphereEditor((512.0, 512.0, 512.0), 16.0, adding=True)
    # the oracle: 8 spare pages do not hold this edit
    small = _oracle({"pool_pages": top + 8}, words)
    with pytest.raises(RuntimeError):
        small.edit(1, (512.0, 512.0, 512.0), 16.0)
    assert small.error == _capi.HD_ERR_POOL_FULL

    d = hd.HashDAG(config=hd.default_config(DEPTH, pool_pages=top + 8))
    d.load_from_DAG(words)
    root0, frame0 = d.firstNodeIndex, _frame(d)
    assert d.level_stats().pages_used + 1 == top
    for _ in range(2):  # refused again the same way: nothing was left half-claimed
        with pytest.raises(hd.HashDagError) as ei:
            d.edit_threads(edit)
        assert ei.value.status == _capi.HD_ERR_POOL_FULL
        assert "pool is full" in str(ei.value), str(ei.value)
        assert d.firstNodeIndex == root0
        assert d.level_stats().pages_used + 1 <= top + 8
        p, m = _frame(d)
        assert np.array_equal(p, frame0[0]) and np.array_equal(m, frame0[1])
    # the table is consistent: imported into a context with room, a GC
    # drops what the failed edit appended and leaves the GC of the untouched
    # scene, read by virtual address
    big = hd.HashDAG(DEPTH)
    big.import_table(d.export_table())
    big.remove_stale_nodes()
    clean = hd.HashDAG(DEPTH)
    clean.load_from_DAG(words)
    clean.remove_stale_nodes()
    t_failed, t_clean = big.export_table(), clean.export_table()
    assert int(t_failed["root"]) == int(t_clean["root"])
    assert table_digest(t_failed, DEPTH, 10) == table_digest(t_clean, DEPTH, 10)
    big.free()
    # with room, the same edit lands where the oracle puts it
    clean.edit_threads(edit)
    ot = _oracle({}, words)
    ot.gc()
    ost = ot.edit(1, (512.0, 512.0, 512.0), 16.0)
    assert clean.firstNodeIndex == ot.root and ost.num_voxels > 0
    assert table_digest(clean.export_table(), DEPTH, 10) == table_digest(ot.export(), DEPTH, 10)
    d.free()
    clean.free()


def _bucket_case():
    """2^9 top-level buckets: the scene fits (largest bucket 744 of 1024
    words) and the sixth of these edits overflows a level-7 bucket."""
    return {"top_bucket_bits": 9}, workloads.mixed_edits(DEPTH, 40, (64.0, 400.0), seed=7)[:6]


@pytest.mark.parametrize("batched", [False, True])
def test_bucket_full_edit_is_refused(gpu, batched):
    words = _words()
    kw, edits = _bucket_case()
    ot = _oracle(kw, words)
    roots = []
    for e in edits[:5]:
        ot.edit(*e)
        roots.append(ot.root)
    with pytest.raises(RuntimeError):
        ot.edit(*edits[5])
    assert ot.error == _capi.HD_ERR_BUCKET_FULL and ot.root == roots[-1]

    d = hd.HashDAG(config=hd.default_config(DEPTH, **kw))
    d.load_from_DAG(words)
    eds = [hd.editor_from_tuple(e) for e in edits]
    if batched:
        with pytest.raises(hd.HashDagError) as ei:
            d.edit_batch(eds)
    else:
        for k, e in enumerate(eds[:5]):
            d.edit_threads(e)
            assert d.firstNodeIndex == roots[k], k
        with pytest.raises(hd.HashDagError) as ei:
            d.edit_threads(eds[5])
    assert ei.value.status == _capi.HD_ERR_BUCKET_FULL
    assert "is full" in str(ei.value), str(ei.value)
    # the edits before it stay applied, the failed one left no trace in the root
    assert d.firstNodeIndex == roots[-1]
    frame = _frame(d)
    ot2 = _oracle(kw, words)
    for e in edits[:5]:
        ot2.edit(*e)
    op, om = ot2.trace_frame(workloads.orbit_camera(DEPTH, W, H), W, H, (0.3, 1.0, 0.2), 1.0, fp_mode=0, threads=4)
    assert np.array_equal(frame[0], op) and np.array_equal(frame[1], om)
    # after a GC the table holds what a GC of the five applied edits holds,
    # at the same virtual addresses: the failed edit left nothing reachable
    d.remove_stale_nodes()
    ot2.gc()
    assert d.firstNodeIndex == ot2.root
    assert table_digest(d.export_table(), DEPTH, 9) == table_digest(ot2.export(), DEPTH, 9)
    d.free()


def test_persistent_barrier_timeout_is_reported_and_context_stays_usable(gpu):
    """The persistent batch's grid barriers are bounded waits.  A test hook
    makes one CTA return without ever arriving (a barrier nothing completes):
    the other CTAs' waits run out after 50 ms, the call returns
    HD_ERR_TIMEOUT with where it stopped, the root is that of the last edit
    the launch finished, and the context keeps working: the remaining edits
    applied afterwards leave the same voxels as applying all of them one by
    one."""
    edits = workloads.mixed_edits(DEPTH, 12, (8.0, 96.0), seed=13)
    eds = [hd.editor_from_tuple(e) for e in edits]
    ref = hd.HashDAG(DEPTH)
    ref.load_from_DAG(_words())
    roots = [ref.firstNodeIndex]
    for e in eds:
        ref.edit_threads(e)
        roots.append(ref.firstNodeIndex)
    d = hd.HashDAG(DEPTH)
    d.load_from_DAG(_words())
    d.batch_tuning = hd.BatchTuning(4, 4, 304, 1)  # the persistent launch
    d.set_test_barrier_skip(5, 50)
    with pytest.raises(hd.HashDagError) as ei:
        d.edit_batch(eds)
    assert ei.value.status == _capi.HD_ERR_TIMEOUT and "ran out of time" in str(ei.value), str(ei.value)
    # the edits the launch finished (CTA 0 finishes the first edit before the
    # grid meets) are applied, in order
    k = roots.index(d.firstNodeIndex)
    assert k <= 1
    # the hook is gone: the rest of the batch runs
    d.edit_batch(eds[k:])
    q = np.random.default_rng(5).integers(0, 1 << DEPTH, (60000, 3)).astype(np.uint32)
    c = np.array([e[1] for e in edits], np.float64)
    near = (c[np.arange(20000) % len(c)] + np.random.default_rng(6).uniform(-100, 100, (20000, 3)))
    q = np.concatenate([q, np.clip(near, 0, (1 << DEPTH) - 1).astype(np.uint32)])
    assert np.array_equal(d.get_values(q), ref.get_values(q))
    fp = []
    for x in (d, ref):
        t = x.export_table()
        ot = po.Table(po.default_config(DEPTH, pool_pages=int(t["pool"].size // 512) + 8))
        ot.import_(t)
        fp.append(ot.fingerprint())
    assert fp[0] == fp[1]
    d.free()
    ref.free()
