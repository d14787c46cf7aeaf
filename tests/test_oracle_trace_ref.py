"""The oracle's tracer against the reference's own traversal code
(tests/golden/ref_trace.json: Tracer::trace_paths and the hit test of
Tracer::trace_shadows compiled for the host from tracer.cu, 1920 x 1080
frames of the seeded scene at depths 10 and 12, fp_mode 0)."""
import hashlib
import json
import os

import numpy as np
import pytest

from hashdag_gb300 import workloads
from oracle import pyoracle as po

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_trace.json")
FIXTURE = json.load(open(GOLDEN))
_tables = {}


def _table(depth):
    if depth not in _tables:
        t = po.Table(po.default_config(depth))
        t.load_basic_dag(po.generate_basic_dag(workloads.SEED_SCENE, depth, workloads.color_tree_levels(depth)))
        _tables[depth] = t
    return _tables[depth]


CASES = [(s["depth"], f["name"]) for s in FIXTURE["scenes"] for f in s["frames"]]


def frame(depth, name):
    s = next(s for s in FIXTURE["scenes"] if s["depth"] == depth)
    return s, next(f for f in s["frames"] if f["name"] == name)


@pytest.mark.parametrize("depth,name", CASES)
def test_oracle_tracer_equals_reference_tracer(depth, name):
    s, f = frame(depth, name)
    W, H = s["width"], s["height"]
    paths, mask = _table(depth).trace_frame(f["camera"], W, H, tuple(f["light"]), f["bias"], fp_mode=0,
                                            threads=os.cpu_count() or 4)
    assert np.array_equal(paths[f["sample_row"], ::16, :3].reshape(-1), np.array(f["row"], np.uint32))
    assert int((paths[..., :3] != 0).any(-1).sum()) == f["hits"]
    assert int((mask == 1).sum()) == f["shadowed"]
    assert hashlib.sha256(np.ascontiguousarray(paths).tobytes()).hexdigest() == f["paths_sha256"]
    assert hashlib.sha256(np.ascontiguousarray(mask).tobytes()).hexdigest() == f["mask_sha256"]
