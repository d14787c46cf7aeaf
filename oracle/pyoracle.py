"""ORACLE — test infrastructure only.

ctypes bindings of oracle/hd_oracle.c (the plain-C restatement of the
reference's hashed-DAG hot path).  Imported only by tests/, the smoke check of
__graft_entry__ and bench.py's CPU-baseline leg, always as the checker.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_HERE = os.path.dirname(os.path.abspath(__file__))


class HdConfig(C.Structure):
    _fields_ = [("depth", C.c_uint32), ("color_tree_levels", C.c_uint32), ("top_levels", C.c_uint32),
                ("top_bucket_bits", C.c_uint32), ("low_bucket_bits", C.c_uint32),
                ("top_bucket_size", C.c_uint32), ("low_bucket_size", C.c_uint32),
                ("pool_pages", C.c_uint32)]


class HdCamera(C.Structure):
    _fields_ = [("position", C.c_double * 3), ("ray_min", C.c_double * 3), ("ray_ddx", C.c_double * 3),
                ("ray_ddy", C.c_double * 3)]


class HdEdit(C.Structure):
    _fields_ = [("tool", C.c_uint32), ("center", C.c_float * 3), ("radius", C.c_float), ("rgb", C.c_uint32),
                ("source", C.c_float * 3), ("dest", C.c_float * 3)]


class HdColor(C.Structure):
    _fields_ = [("color_bits", C.c_uint32), ("weight", C.c_uint8), ("bits_per_weight", C.c_uint8),
                ("reserved", C.c_uint16)]

    def tuple(self):
        return (self.color_bits, self.weight, self.bits_per_weight)


class HdEditStats(C.Structure):
    _fields_ = [("num_voxels", C.c_uint64), ("num_nodes", C.c_uint64), ("find_or_add_calls", C.c_uint64),
                ("nodes_added", C.c_uint64), ("words_scanned", C.c_uint64), ("device_ms", C.c_float),
                ("host_ms", C.c_float)]


class HdLevelStats(C.Structure):
    _fields_ = [("words", C.c_uint64 * 20), ("nodes", C.c_uint64 * 20), ("pages_used", C.c_uint64),
                ("root", C.c_uint32), ("levels", C.c_uint32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        P = C.c_void_p
        u32, u64, f32 = C.c_uint32, C.c_uint64, C.c_float
        pu32 = np.ctypeslib.ndpointer(np.uint32, flags="C")
        pu8 = np.ctypeslib.ndpointer(np.uint8, flags="C")
        L.or_table_create.restype = P
        L.or_table_create.argtypes = [C.POINTER(HdConfig)]
        L.or_table_destroy.argtypes = [P]
        L.or_table_error.argtypes = [P]
        L.or_table_root.restype = u32
        L.or_table_root.argtypes = [P]
        L.or_table_set_root.argtypes = [P, u32]
        L.or_table_pool_top.restype = u32
        L.or_table_pool_top.argtypes = [P]
        L.or_table_full_nodes.restype = C.POINTER(u32)
        L.or_table_full_nodes.argtypes = [P]
        L.or_table_export.argtypes = [P, P, P, P, u64, P]
        L.or_table_import.argtypes = [P, P, P, P, u64, P, u32]
        L.or_level_stats.argtypes = [P, C.POINTER(HdLevelStats)]
        L.or_total_buckets.restype = u64
        L.or_total_buckets.argtypes = [C.POINTER(HdConfig)]
        L.or_total_virtual_pages.restype = u64
        L.or_total_virtual_pages.argtypes = [C.POINTER(HdConfig)]
        L.or_make_ptr.restype = u32
        L.or_make_ptr.argtypes = [C.POINTER(HdConfig), u32, u32, u32]
        L.or_hash_leaf.restype = u32
        L.or_hash_leaf.argtypes = [u64]
        L.or_hash_interior.restype = u32
        L.or_hash_interior.argtypes = [u32, pu32]
        L.or_murmurhash32.restype = u32
        L.or_murmurhash32.argtypes = [u32]
        L.or_murmurhash64.restype = u64
        L.or_murmurhash64.argtypes = [u64]
        L.or_find_or_add_leaf.restype = u32
        L.or_find_or_add_leaf.argtypes = [P, u64]
        L.or_find_or_add_interior.restype = u32
        L.or_find_or_add_interior.argtypes = [P, u32, u32, pu32]
        L.or_read_word.restype = u32
        L.or_read_word.argtypes = [P, u32]
        L.or_scene_height.restype = C.c_int32
        L.or_scene_height.argtypes = [u64, u32, u32, u32]
        L.or_scene_solid.restype = C.c_int
        L.or_scene_solid.argtypes = [u64, u32, u32, u32, u32]
        L.or_scene_spheres.argtypes = [u64, u32, np.ctypeslib.ndpointer(np.int64, flags="C")]
        L.or_generate_basic_dag.restype = C.POINTER(u32)
        L.or_generate_basic_dag.argtypes = [u64, u32, u32, C.POINTER(u64)]
        L.or_generate_basic_dag_ex.restype = C.POINTER(u32)
        L.or_generate_basic_dag_ex.argtypes = [u64, u32, u32, u32, C.POINTER(u64)]
        L.or_generate_basic_dag_mt.restype = C.POINTER(u32)
        L.or_generate_basic_dag_mt.argtypes = [u64, u32, u32, u32, u32, C.POINTER(u64)]
        L.or_scene_shell.restype = C.c_int
        L.or_scene_shell.argtypes = [u64, u32, u32, u32, u32]
        L.or_free.argtypes = [P]
        L.or_load_basic_dag.argtypes = [P, pu32, u64]
        L.or_get_value.argtypes = [P, u32, u32, u32]
        L.or_occupancy_fingerprint.restype = u64
        L.or_occupancy_fingerprint.argtypes = [P, u32]
        L.or_trace_primary.argtypes = [P, C.POINTER(HdCamera), u32, u32, u32, pu32, u32, u32, P]
        L.or_trace_shadow.argtypes = [P, C.POINTER(HdCamera), u32, u32, u32, pu32,
                                      np.ctypeslib.ndpointer(np.float32, flags="C"), f32, pu8, u32, u32, P]
        L.or_trace_frame_mt.argtypes = [P, C.POINTER(HdCamera), u32, u32, u32,
                                        np.ctypeslib.ndpointer(np.float32, flags="C"), f32, pu32, pu8, u32,
                                        u32, u32]
        L.or_reachable_counts.argtypes = [P, u32, np.ctypeslib.ndpointer(np.uint64, flags="C")]
        L.or_reachable_words.argtypes = [P, u32, np.ctypeslib.ndpointer(np.uint64, flags="C"),
                                         np.ctypeslib.ndpointer(np.uint64, flags="C")]
        L.or_edit.argtypes = [P, C.POINTER(HdEdit), C.POINTER(HdEditStats)]
        L.or_edit_mt.argtypes = [P, C.POINTER(HdEdit), C.POINTER(HdEditStats), u32]
        L.or_gc.argtypes = [P, P, u32]
        L.or_set_foa_log.argtypes = [C.c_char_p]
        L.or_colors_create.restype = P
        L.or_colors_destroy.argtypes = [P]
        L.or_colors_from_scene.argtypes = [P, P, u64]
        L.or_colors_from_scene_mt.argtypes = [P, P, u64, u32]
        L.or_get_color.restype = HdColor
        L.or_get_color.argtypes = [P, P, u32, u32, u32]
        L.or_edit_colored.argtypes = [P, P, C.POINTER(HdEdit), C.POINTER(HdEditStats)]
        L.or_undo.argtypes = [P, P]
        L.or_redo.argtypes = [P, P]
        L.or_colors_stats.argtypes = [P, np.ctypeslib.ndpointer(np.uint64, flags="C")]
        L.or_color_rgb8.restype = u32
        L.or_color_rgb8.argtypes = [u64, u32, u32, u32]
        L.or_voxel_color.restype = HdColor
        L.or_voxel_color.argtypes = [u64, u32, u32, u32]
        L.or_color_rgb888.restype = u32
        L.or_color_rgb888.argtypes = [HdColor]
        L.or_f3_to_rgb888.restype = u32
        L.or_f3_to_rgb888.argtypes = [C.c_float, C.c_float, C.c_float]
        L.or_trace_colors.argtypes = [P, P, pu32, u64, P, np.ctypeslib.ndpointer(np.uint32, flags="C")]
        L.or_perlin_fractal.restype = C.c_float
        L.or_perlin_fractal.argtypes = [C.c_int, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float]
        PP = C.POINTER(C.c_void_p)
        L.or_main_leaf.argtypes = [pu32, u64, u32, u32, u64, PP, C.POINTER(u64), PP, C.POINTER(u64), PP,
                                   C.POINTER(u64), PP, C.POINTER(u64)]
        _lib = L
    return _lib


def default_config(depth, color_tree_levels=None, pool_pages=None):
    """The reference's default bucket geometry (typedefs.h:201-239); scenes
    of depth 11 and more take 2^12 top-level buckets (BUCKETS_BITS_FOR_TOP_LEVELS)
    because their level 8 holds over 10^5 nodes."""
    if color_tree_levels is None:
        color_tree_levels = min(10, depth - 5)
    if pool_pages is None:
        pool_pages = 1 << 20
    top_bits = 10 if depth <= 10 else (12 if depth <= 15 else 14)
    return HdConfig(depth, color_tree_levels, 9, top_bits, 16 if depth <= 15 else 17, 1024, 4096, pool_pages)


def camera(cam):
    """Accepts an HdCamera-like object with the four double[3] fields."""
    if isinstance(cam, HdCamera):
        return cam
    c = HdCamera()
    for f in ("position", "ray_min", "ray_ddx", "ray_ddy"):
        getattr(c, f)[:] = [float(v) for v in getattr(cam, f) if True] if not isinstance(cam, dict) else cam[f]
    return c


SCENE_SHELL = 1


def generate_basic_dag(seed, depth, color_tree_levels, flags=0, threads=1):
    """BasicDAG words of the seeded scene; threads > 1 (0: every core)
    builds subtrees in parallel, with the same words."""
    n = C.c_uint64(0)
    p = lib().or_generate_basic_dag_mt(seed, depth, color_tree_levels, flags, threads, C.byref(n))
    if not p:
        raise RuntimeError("scene generation failed")
    words = np.ctypeslib.as_array(p, shape=(n.value,)).copy()
    lib().or_free(p)
    return words


def scene_height(seed, depth, x, z):
    return lib().or_scene_height(seed, depth, x, z)


def scene_solid(seed, depth, x, y, z):
    return lib().or_scene_solid(seed, depth, x, y, z)


def scene_shell(seed, depth, x, y, z):
    return lib().or_scene_shell(seed, depth, x, y, z)


def scene_spheres(seed, depth):
    out = np.zeros(256, np.int64)
    lib().or_scene_spheres(seed, depth, out)
    return out.reshape(64, 4)


class Table:
    """The oracle's paged hash table (HashTable + HashDAG root)."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.h = lib().or_table_create(C.byref(cfg))
        if not self.h:
            raise RuntimeError("or_table_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_table_destroy(self.h)
            self.h = None

    @property
    def error(self):
        return lib().or_table_error(self.h)

    @property
    def root(self):
        return lib().or_table_root(self.h)

    @root.setter
    def root(self, v):
        lib().or_table_set_root(self.h, v)

    @property
    def pool_top(self):
        return lib().or_table_pool_top(self.h)

    def full_nodes(self):
        p = lib().or_table_full_nodes(self.h)
        return np.array([p[i] for i in range(self.cfg.depth)], np.uint32)

    def load_basic_dag(self, words):
        words = np.ascontiguousarray(words, np.uint32)
        r = lib().or_load_basic_dag(self.h, words, words.size)
        if r:
            raise RuntimeError(f"load_basic_dag failed: {r}")

    def level_stats(self):
        s = HdLevelStats()
        lib().or_level_stats(self.h, C.byref(s))
        return s

    def export(self):
        nb = lib().or_total_buckets(C.byref(self.cfg))
        nv = lib().or_total_virtual_pages(C.byref(self.cfg))
        bs = np.zeros(nb, np.uint32)
        pt = np.zeros(nv, np.uint32)
        pool = np.zeros(self.pool_top * 512, np.uint32)
        full = np.zeros(self.cfg.depth, np.uint32)
        lib().or_table_export(self.h, bs.ctypes.data, pt.ctypes.data, pool.ctypes.data, pool.size,
                              full.ctypes.data)
        return dict(bucket_sizes=bs, page_table=pt, pool=pool, full_nodes=full, root=self.root)

    def import_(self, t):
        r = lib().or_table_import(self.h, t["bucket_sizes"].ctypes.data, t["page_table"].ctypes.data,
                                  t["pool"].ctypes.data, t["pool"].size, t["full_nodes"].ctypes.data,
                                  int(t["root"]))
        if r:
            raise RuntimeError(f"import failed {r}")

    def get_value(self, x, y, z):
        return lib().or_get_value(self.h, x, y, z)

    def fingerprint(self, root=None):
        return lib().or_occupancy_fingerprint(self.h, self.root if root is None else root)

    def reachable_counts(self, root=None):
        out = np.zeros(20, np.uint64)
        lib().or_reachable_counts(self.h, self.root if root is None else root, out)
        return out[:self.cfg.depth - 1]

    def reachable_words(self, root=None):
        """Words of the nodes reachable from root, per level."""
        out, words = np.zeros(20, np.uint64), np.zeros(20, np.uint64)
        lib().or_reachable_words(self.h, self.root if root is None else root, out, words)
        return words[:self.cfg.depth - 1]

    def trace_primary(self, cam, w, h, fp_mode=0, rows=None):
        paths = np.zeros(w * h * 4, np.uint32)
        r0, r1 = (0, h) if rows is None else rows
        lib().or_trace_primary(self.h, C.byref(camera(cam)), w, h, fp_mode, paths, r0, r1, None)
        return paths.reshape(h, w, 4)

    def trace_shadow(self, cam, w, h, paths, light, bias, fp_mode=0, rows=None):
        mask = np.zeros(w * h, np.uint8)
        r0, r1 = (0, h) if rows is None else rows
        lib().or_trace_shadow(self.h, C.byref(camera(cam)), w, h, fp_mode,
                              np.ascontiguousarray(paths, np.uint32).reshape(-1),
                              np.asarray(light, np.float32), bias, mask, r0, r1, None)
        return mask.reshape(h, w)

    def trace_frame(self, cam, w, h, light, bias, fp_mode=0, threads=1, rows=None):
        paths = np.zeros(w * h * 4, np.uint32)
        mask = np.zeros(w * h, np.uint8)
        r0, r1 = (0, h) if rows is None else rows
        lib().or_trace_frame_mt(self.h, C.byref(camera(cam)), w, h, fp_mode, np.asarray(light, np.float32),
                                bias, paths, mask, threads, r0, r1)
        return paths.reshape(h, w, 4), mask.reshape(h, w)

    def edit(self, tool, center, radius, threads=1):
        """One edit; threads > 1 (0: every core) runs the level-T tasks on
        that many threads (same voxels, node order may differ)."""
        e = make_edit(tool, center, radius)
        s = HdEditStats()
        if threads == 1:
            r = lib().or_edit(self.h, C.byref(e), C.byref(s))
        else:
            r = lib().or_edit_mt(self.h, C.byref(e), C.byref(s), threads)
        if r:
            raise RuntimeError(f"edit failed {r}")
        return s

    def gc(self, extra_roots=()):
        arr = np.array(list(extra_roots) + [0], np.uint32)
        r = lib().or_gc(self.h, arr.ctypes.data, len(extra_roots))
        if r:
            raise RuntimeError(f"gc failed {r}")
        return [int(v) for v in arr[:len(extra_roots)]]


def make_edit(tool, center, radius, rgb=0xFF0000, source=(0.0, 0.0, 0.0), dest=(0.0, 0.0, 0.0)):
    return HdEdit(tool, (C.c_float * 3)(*center), radius, rgb, (C.c_float * 3)(*source), (C.c_float * 3)(*dest))


class Colors:
    """HashDAGColors of a Table: colour tree, leaves, undo/redo frames."""

    def __init__(self, table):
        self.t = table
        self.h = lib().or_colors_create()

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_colors_destroy(self.h)
            self.h = None

    def from_scene(self, color_seed, threads=1):
        """threads > 1 (0: every core) builds the leaves in parallel, with the
        same result."""
        r = (lib().or_colors_from_scene(self.h, self.t.h, color_seed) if threads == 1 else
             lib().or_colors_from_scene_mt(self.h, self.t.h, color_seed, threads))
        if r:
            raise RuntimeError("colour import failed")

    def get_color(self, x, y, z):
        return lib().or_get_color(self.t.h, self.h, x, y, z).tuple()

    def edit(self, tool, center, radius, rgb=0xFF0000, source=(0.0, 0.0, 0.0), dest=(0.0, 0.0, 0.0)):
        e = make_edit(tool, center, radius, rgb, source, dest)
        s = HdEditStats()
        r = lib().or_edit_colored(self.t.h, self.h, C.byref(e), C.byref(s))
        if r:
            raise RuntimeError(f"edit failed {r}")
        return s

    def trace_colors(self, paths, params=None):
        """Tracer::trace_colors of a paths image (h x w x 4 uint32);
        params: a ctypes hd_trace_colors_params (or None: the plain view)."""
        p = np.ascontiguousarray(paths, np.uint32).reshape(-1, 4)
        out = np.zeros(len(p), np.uint32)
        lib().or_trace_colors(self.t.h, self.h, p.reshape(-1), len(p), C.byref(params) if params is not None else None,
                              out)
        return out

    def undo(self):
        return bool(lib().or_undo(self.t.h, self.h))

    def redo(self):
        return bool(lib().or_redo(self.t.h, self.h))

    def stats(self):
        out = np.zeros(5, np.uint64)
        lib().or_colors_stats(self.h, out)
        return dict(zip(("nodes", "leaves", "blocks", "weight_words", "macro_words"), (int(v) for v in out)))


def voxel_color(seed, x, y, z):
    return lib().or_voxel_color(seed, x, y, z).tuple()


def color_rgb888(color_bits, weight=0, bits_per_weight=0):
    return lib().or_color_rgb888(HdColor(color_bits, weight, bits_per_weight, 0))


# ---- on-disk formats (FileWriter, serializer.h:11-121) ------------------------
# Raw little-endian values; an array is its uint64 element count, then its
# elements; a DAGInfo is six doubles (AABB min, then max).

def _array(a, dtype):
    a = np.ascontiguousarray(a, dtype)
    return np.uint64(a.size).tobytes() + a.tobytes()


def _info(info):
    lo, hi = info
    return np.array(list(lo) + list(hi), np.float64).tobytes()


def basic_dag_file(words, depth, info):
    """BasicDAGFactory::save_dag_to_file (basic_dag.cpp:94-103): DAGInfo,
    uint32 levels, the node words."""
    return _info(info) + np.uint32(depth).tobytes() + _array(words, np.uint32)


def main_leaf(words, depth, top_levels, seed):
    """enclosedLeaves and the main leaf (blocks, macro words, weights in the
    leaf's in-memory order) of the colour field of `seed` on a BasicDAG."""
    words = np.ascontiguousarray(words, np.uint32)
    ptr = [C.c_void_p() for _ in range(4)]
    cnt = [C.c_uint64() for _ in range(4)]
    r = lib().or_main_leaf(words, words.size, depth, top_levels, seed, C.byref(ptr[0]), C.byref(cnt[0]),
                           C.byref(ptr[1]), C.byref(cnt[1]), C.byref(ptr[2]), C.byref(cnt[2]),
                           C.byref(ptr[3]), C.byref(cnt[3]))
    if r:
        raise RuntimeError(f"main leaf failed: {r}")
    out = []
    for (p_, n_), dt in zip(zip(ptr, cnt), (np.uint64, np.uint64, np.uint64, np.uint32)):
        arr = np.ctypeslib.as_array(C.cast(p_, C.POINTER(C.c_uint64 if dt == np.uint64 else C.c_uint32)),
                                    shape=(max(1, n_.value),))[:n_.value].copy()
        lib().or_free(p_)
        out.append(arr.astype(dt))
    enclosed, blocks, macros, weights = out
    return dict(enclosed=enclosed, blocks=blocks, macros=macros, weights=weights)


def swap_bytes(words):
    """ColorUtils::swap_byte_order (color_utils.h:85-105) of uint32 words."""
    return np.ascontiguousarray(words, np.uint32).byteswap()


def compressed_colors_file(words, depth, top_levels, seed):
    """BasicDAGFactory::save_compressed_colors_to_file (basic_dag.cpp:34-47):
    uint32 topLevels, enclosedLeaves (uint64), the weights swapped back to
    file order, blocks, macro blocks."""
    m = main_leaf(words, depth, top_levels, seed)
    return (np.uint32(top_levels).tobytes() + _array(m["enclosed"], np.uint64) +
            _array(swap_bytes(m["weights"]), np.uint32) + _array(m["blocks"], np.uint64) +
            _array(m["macros"], np.uint64))


def hash_dag_file(table, info, pool_max):
    """HashDAGFactory::save_dag_to_file (hash_dag_factory.cpp:199-222):
    DAGInfo, uint32 levels, firstNodeIndex, poolMaxSize, pageTableSize,
    poolTop, the pool's first poolTop pages, the page table."""
    t = table.export()
    head = np.array([table.cfg.depth, t["root"], pool_max, t["page_table"].size, table.pool_top], np.uint32)
    return _info(info) + head.tobytes() + t["pool"].tobytes() + t["page_table"].tobytes()


def perlin_fractal(seed, frequency, octaves, x, y, z):
    """FastNoise's GetPerlinFractal (FBM, quintic, lacunarity 2, gain 0.5)."""
    return lib().or_perlin_fractal(seed, frequency, octaves, x, y, z)
