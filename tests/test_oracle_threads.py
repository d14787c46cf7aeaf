"""The oracle's threaded edit (the reference's edit_threads with
THREADED_EDITS: level-T tasks on a thread pool, the hash table under
per-bucket locks, hash_dag.h:255-405), which the edit path's CPU baseline
times: the same voxels and counters as the single-threaded editor."""
from hashdag_gb300 import workloads
from oracle import pyoracle as po


def test_threaded_edits_keep_voxels_and_counters():
    depth = 10
    words = po.generate_basic_dag(workloads.SEED_SCENE, depth, workloads.color_tree_levels(depth))
    one, many = po.Table(po.default_config(depth)), po.Table(po.default_config(depth))
    one.load_basic_dag(words)
    many.load_basic_dag(words)
    for e in workloads.mixed_edits(depth, 16, (4.0, 160.0), seed=9):
        a, b = one.edit(*e), many.edit(*e, threads=4)
        assert (a.num_voxels, a.num_nodes, a.find_or_add_calls) == (b.num_voxels, b.num_nodes, b.find_or_add_calls)
        assert one.fingerprint() == many.fingerprint()
    assert many.error == 0
