"""The oracle's threaded scene generator builds the same BasicDAG words as
its single-threaded one (subtrees built in parallel, merged with
content deduplication), for solid and shell scenes."""
import numpy as np
import pytest

from hashdag_gb300 import workloads
from oracle import pyoracle as po


@pytest.mark.parametrize("depth,flags", [(8, 0), (10, 0), (10, po.SCENE_SHELL), (11, 0)])
def test_threaded_generator_equals_single_threaded(depth, flags):
    ctl = workloads.color_tree_levels(depth)
    one = po.generate_basic_dag(workloads.SEED_SCENE, depth, ctl, flags)
    for threads in (2, 5):
        many = po.generate_basic_dag(workloads.SEED_SCENE, depth, ctl, flags, threads=threads)
        assert many.size == one.size and np.array_equal(many, one), (depth, flags, threads)
