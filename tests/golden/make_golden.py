"""Generates the golden fixtures of tests/golden/ from the reference's own
code (oracle/_ref, built from the reference sources by oracle/build_ref.py).

    python tests/golden/make_golden.py

Each fixture pins, on a seeded scene, what the reference computes:
load_from_DAG's table, the table after each edit of a seeded stream (tasks in
depth-first order), and the state after remove_stale_nodes; plus hash
known-answer vectors.  Needs the reference sources; the fixtures it writes
are small JSON files checked into the repository.
"""
import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from hashdag_gb300 import workloads  # noqa: E402
from oracle import build_ref, pyoracle as po  # noqa: E402
from tests.helpers import table_digest  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


class Silence:
    """Swallows the reference's printf output."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        self.null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.null, 1)

    def __exit__(self, *a):
        os.dup2(self.saved, 1)
        os.close(self.null)
        os.close(self.saved)


def load_ref(depth):
    t = workloads.color_tree_levels(depth)
    b = workloads.top_bucket_bits(depth)
    R = C.CDLL(build_ref.build(depth, t, b))
    for f in ("ref_root", "ref_pool_top", "ref_total_buckets", "ref_total_pages", "ref_level_size", "ref_depth",
              "ref_color_tree_levels", "ref_hash_leaf", "ref_hash_interior"):
        getattr(R, f).restype = C.c_uint32
    R.ref_edit.argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p]
    R.ref_hash_leaf.argtypes = [C.c_uint64]
    R.ref_hash_interior.argtypes = [C.c_uint32, C.c_void_p]
    R.ref_get_value.argtypes = [C.c_uint32] * 3
    return R, t, b


def ref_table(R, depth):
    nb, nv = R.ref_total_buckets(), R.ref_total_pages()
    bs = np.zeros(nb, np.uint32)
    pt = np.zeros(nv, np.uint32)
    pool = np.zeros(R.ref_pool_top() * 512, np.uint32)
    full = np.zeros(depth, np.uint32)
    R.ref_export(bs.ctypes.data_as(C.c_void_p), pt.ctypes.data_as(C.c_void_p), pool.ctypes.data_as(C.c_void_p),
                 C.c_uint64(pool.size), full.ctypes.data_as(C.c_void_p))
    return dict(bucket_sizes=bs, page_table=pt, pool=pool, full_nodes=full, root=R.ref_root())


def fixture(depth, edits):
    R, T, bits = load_ref(depth)
    words = po.generate_basic_dag(workloads.SEED_SCENE, depth, T)
    out = dict(depth=depth, color_tree_levels=T, top_bucket_bits=bits, seed=workloads.SEED_SCENE,
               basic_dag_words=int(words.size), basic_dag_sha256=hashlib.sha256(words.tobytes()).hexdigest())
    with Silence():
        R.ref_load(words.ctypes.data_as(C.c_void_p), C.c_uint64(words.size), C.c_uint32(1 << 20))
    tab = ref_table(R, depth)
    out["load"] = dict(root=int(tab["root"]), pool_top=R.ref_pool_top(),
                       full_nodes=[int(v) for v in tab["full_nodes"][1:depth - 1]],
                       level_words=[R.ref_level_size(l) for l in range(depth - 1)],
                       digest=table_digest(tab, depth, bits))
    steps = []
    for tool, c, r in edits:
        st = (C.c_uint64 * 2)()
        with Silence():
            R.ref_edit(tool, C.c_float(c[0]), C.c_float(c[1]), C.c_float(c[2]), C.c_float(r), st)
        tab = ref_table(R, depth)
        steps.append(dict(tool=tool, center=list(c), radius=r, root=int(tab["root"]), num_voxels=int(st[0]),
                          num_nodes=int(st[1]), pool_top=R.ref_pool_top(),
                          level_words=[R.ref_level_size(l) for l in range(depth - 1)],
                          digest=table_digest(tab, depth, bits)))
    out["edits"] = steps
    # point queries on the edited volume
    rng = np.random.default_rng(11)
    e = 1 << depth
    q = rng.integers(0, e, (2000, 3))
    from hashdag_gb300 import scene
    q[:, 1] = np.clip(scene.height(workloads.SEED_SCENE, depth, q[:, 0], q[:, 2]) + rng.integers(-40, 40, 2000),
                      0, e - 1)
    out["queries"] = dict(xyz=q.tolist(), values=[R.ref_get_value(*(int(v) for v in p)) for p in q])
    # garbage collection (remove_stale_nodes keeps firstNodeIndex at the old
    # address; the in-place child remap keeps that address valid)
    with Silence():
        R.ref_gc()
    tab = ref_table(R, depth)
    t2 = po.Table(po.default_config(depth))
    t2.import_(tab)
    out["gc"] = dict(root=int(tab["root"]), pool_top=R.ref_pool_top(),
                     level_words=[R.ref_level_size(l) for l in range(depth - 1)],
                     reachable=[int(v) for v in t2.reachable_counts()],
                     fingerprint=int(t2.fingerprint()))
    return out, R


def main():
    d10_edits = workloads.carve_edits(10, 16) + workloads.mixed_edits(10, 16, (4.0, 64.0), seed=7)
    f10, R = fixture(10, d10_edits)
    # hash known-answer vectors from the reference's HashDagUtils
    rng = np.random.default_rng(5)
    leaves = [int(v) for v in rng.integers(0, 2 ** 63, 64, dtype=np.int64)] + [0, 2 ** 64 - 1, 1, 2 ** 63]
    kat_leaf = [[v, R.ref_hash_leaf(C.c_uint64(v))] for v in leaves]
    kat_int = []
    for n in range(2, 10):
        for _ in range(6):
            node = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
            kat_int.append([[int(v) for v in node], R.ref_hash_interior(n, node.ctypes.data_as(C.c_void_p))])
    with open(os.path.join(HERE, "hash_kat.json"), "w") as f:
        json.dump(dict(leaf=kat_leaf, interior=kat_int), f)
    with open(os.path.join(HERE, "ref_d10.json"), "w") as f:
        json.dump(f10, f)
    d12_edits = workloads.carve_edits(12, 8, (32.0, 96.0)) + workloads.mixed_edits(12, 8, (4.0, 128.0), seed=9)
    f12, _ = fixture(12, d12_edits)
    with open(os.path.join(HERE, "ref_d12.json"), "w") as f:
        json.dump(f12, f)
    print("fixtures written")


if __name__ == "__main__":
    main()
