"""hashdag_gb300 — GB300-native hashed sparse voxel DAG hot path.

Host-side mirror of the reference's interfaces (Phyronnaz/HashDAG) over the
C ABI of libhashdag_gb300.so:

* HashDAG        — HashDAG (hash_dag.h:214-636) with the device-resident
                   HashTable; load_from_DAG (hash_dag_factory.cpp:152-184),
                   edit_threads (hash_dag.h:255-405), remove_stale_nodes
                   (hash_dag.h:407-547).
* DAGTracer      — DAGTracer (dag_tracer.h:9-42), headless: resolve_paths /
                   resolve_shadows return kernel milliseconds and keep their
                   results in device buffers.
* SphereEditor / BoxEditor — the editors (hash_dag_editors.h:223-313).

Every call runs sm_103a kernels; there is no CPU path.
"""
import ctypes as C
import os

import numpy as np

from . import _capi
from ._capi import (BatchTuning, Camera, Config, Edit, EditStats, HashDagError, LevelStats, Request, RequestResult,
                    ServeConfig, ServeStats, lib)

__all__ = ["HashDAG", "DAGTracer", "SphereEditor", "BoxEditor", "SpherePaintEditor", "CopyEditor",
           "SphereNoiseEditor", "FillEditorColors", "ReplayManager", "BatchTuning",
           "Request", "RequestResult", "ServeConfig", "ServeStats", "edit_request", "render_request", "Camera", "Config", "EditStats", "LevelStats",
           "HashDagError", "default_config"]

TOOL_SPHERE_REMOVE, TOOL_SPHERE_ADD, TOOL_BOX_REMOVE, TOOL_BOX_ADD, TOOL_SPHERE_PAINT, TOOL_COPY, \
    TOOL_NOISE_REMOVE, TOOL_NOISE_ADD, TOOL_FILL = range(9)
SCENE_SHELL = 1
GC_KEEP_HISTORY = 1
GC_RELEASE_PAGES = 2
# EDebugColors (tracer.h:7-17) and the overlay's ETool (tracer.h:21-29)
DEBUG_NONE, DEBUG_INDEX, DEBUG_POSITION, DEBUG_COLOR_TREE, DEBUG_COLOR_BITS, DEBUG_MIN_COLOR, DEBUG_MAX_COLOR, \
    DEBUG_WEIGHT = range(8)
OVERLAY_SPHERE, OVERLAY_SPHERE_PAINT, OVERLAY_SPHERE_NOISE, OVERLAY_CUBE, OVERLAY_CUBE_COPY, OVERLAY_CUBE_FILL = range(6)


def default_config(depth, **overrides):
    cfg = Config()
    lib().hd_default_config(depth, C.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise HashDagError(_capi.HD_ERR_STATE, "no CUDA device")
    return torch


class _Editor:
    tool = None
    rgb = 0xFF0000
    source = (0.0, 0.0, 0.0)
    dest = (0.0, 0.0, 0.0)

    def __init__(self, center, radius):
        self.center = tuple(float(np.float32(v)) for v in center)
        self.radius = float(np.float32(radius))

    def to_edit(self):
        return Edit(self.tool, (C.c_float * 3)(*self.center), self.radius, self.rgb,
                    (C.c_float * 3)(*self.source), (C.c_float * 3)(*self.dest))


class SphereEditor(_Editor):
    """SphereEditor<isAdding> (hash_dag_editors.h:272-313)."""

    def __init__(self, center, radius, adding):
        super().__init__(center, radius)
        self.tool = TOOL_SPHERE_ADD if adding else TOOL_SPHERE_REMOVE


class BoxEditor(_Editor):
    """BoxEditor<isAdding> (hash_dag_editors.h:223-270); radius is the half
    extent."""

    def __init__(self, center, radius, adding):
        super().__init__(center, radius)
        self.tool = TOOL_BOX_ADD if adding else TOOL_BOX_REMOVE


class SpherePaintEditor(_Editor):
    """SpherePaintEditor (hash_dag_editors.h:315-330): voxels in the sphere
    move their colour toward rgb (r | g << 8 | b << 16; the reference paints
    blue, 0xFF0000) by clamp(1 - distance / radius, 0, 0.1)."""
    tool = TOOL_SPHERE_PAINT

    def __init__(self, center, radius, rgb=0xFF0000):
        super().__init__(center, radius)
        self.rgb = int(rgb)


class CopyEditor(_Editor):
    """The copy tool (CopyEditorWithDecompression, hash_dag_editors.h:437-609):
    the region center +- radius, read before the edit, is OR-ed into the
    region moved by dest - source, with its colours."""
    tool = TOOL_COPY

    def __init__(self, center, radius, source, dest):
        super().__init__(center, radius)
        self.source = tuple(float(np.float32(v)) for v in source)
        self.dest = tuple(float(np.float32(v)) for v in dest)


class SphereNoiseEditor(_Editor):
    """SphereNoiseEditor (hash_dag_editors.h:712-760): a sphere roughened by
    FastNoise's Perlin FBM, in a buffer of 1.5 radius.  Carving (adding =
    False) changes no voxel, as in the reference (BufferEditor::get_new_value
    reads a voxel set false as its old value)."""

    def __init__(self, center, radius, adding):
        super().__init__(center, radius)
        self.tool = TOOL_NOISE_ADD if adding else TOOL_NOISE_REMOVE


class FillEditorColors(_Editor):
    """FillEditorColors (hash_dag_editors.h:624-710): flood fill of the empty
    voxels connected to the centre within center +- radius, each filled voxel
    taking the colour of the last solid boundary voxel before it in x, y, z
    order."""
    tool = TOOL_FILL


def edit_request(arrival_ms, editor):
    return Request(0, 0, 0, 0, float(arrival_ms), editor.to_edit(), Camera())


def render_request(arrival_ms, width, height, camera):
    cam = camera if isinstance(camera, Camera) else Camera.from_params(camera)
    return Request(1, int(width), int(height), 0, float(arrival_ms), Edit(), cam)


def editor_from_tuple(t):
    tool, center, radius = t[:3]
    if tool in (TOOL_SPHERE_REMOVE, TOOL_SPHERE_ADD):
        return SphereEditor(center, radius, tool == TOOL_SPHERE_ADD)
    if tool == TOOL_SPHERE_PAINT:
        return SpherePaintEditor(center, radius, *(t[3:4] or ()))
    if tool == TOOL_COPY:
        return CopyEditor(center, radius, t[3], t[4])
    if tool in (TOOL_NOISE_REMOVE, TOOL_NOISE_ADD):
        return SphereNoiseEditor(center, radius, tool == TOOL_NOISE_ADD)
    if tool == TOOL_FILL:
        return FillEditorColors(center, radius)
    return BoxEditor(center, radius, tool == TOOL_BOX_ADD)


REPLAY_TYPES = ("SetLocation", "SetRotation", "SetToolParameters", "EditSphere", "EditCube", "EditCopy",
                "EditFill", "EditPaint", "Undo", "Redo", "EndFrame")


class ReplayManager:
    """ReplayManager (replay.h:462-635) over hd_replay: load_csv, write_csv,
    replay_frame on a HashDAG (edits, undo / redo, the view), the frame's
    camera back."""

    def __init__(self, path=None, text=None):
        self._h = C.c_void_p()
        if path is not None:
            st = lib().hd_replay_load(os.fsencode(path), C.byref(self._h))
        else:
            data = text.encode() if isinstance(text, str) else bytes(text)
            st = lib().hd_replay_load_text(data, len(data), C.byref(self._h))
        if st != _capi.HD_OK:
            raise HashDagError(st, f"cannot load the replay {path if path is not None else '(text)'}")

    def free(self):
        if self._h:
            lib().hd_replay_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def _info(self):
        a, f, n = C.c_uint64(), C.c_uint64(), C.c_uint64()
        lib().hd_replay_info(self._h, C.byref(a), C.byref(f), C.byref(n))
        return a.value, f.value, n.value

    def num_frames(self):
        return self._info()[1]

    def __len__(self):
        return self._info()[0]

    def at_end(self):
        a, _, n = self._info()
        return n == a

    def action(self, i):
        """(type name, float cells, integer cells, boolean cell)."""
        a = _capi.ReplayAction()
        st = lib().hd_replay_get_action(self._h, i, C.byref(a))
        if st != _capi.HD_OK:
            raise HashDagError(st, f"no action {i}")
        return (REPLAY_TYPES[a.type], [float(v) for v in a.floats[:a.n_floats]], [int(v) for v in a.ints[:a.n_ints]],
                bool(a.flag))

    def write_csv(self, path):
        st = lib().hd_replay_write(self._h, os.fsencode(path))
        if st != _capi.HD_OK:
            raise HashDagError(st, f"cannot write {path}")

    def reset_replay(self):
        lib().hd_replay_reset(self._h)

    def replay_frame(self, dag, replay_depth, width, height, info):
        """Applies the next frame's actions to dag; returns (camera params
        dict, edits applied)."""
        cfg = _capi.ReplayConfig()
        cfg.replay_depth, cfg.width, cfg.height = replay_depth, width, height
        lo, hi = info
        cfg.info.aabb_min[:] = [float(v) for v in lo]
        cfg.info.aabb_max[:] = [float(v) for v in hi]
        cam = Camera()
        n = C.c_uint32()
        _capi.check(dag.handle, lib().hd_replay_frame(dag.handle, self._h, C.byref(cfg), C.byref(cam), C.byref(n)))
        return dict(position=list(cam.position), ray_min=list(cam.ray_min), ray_ddx=list(cam.ray_ddx),
                    ray_ddy=list(cam.ray_ddy)), n.value


class HashDAG:
    """A device-resident hash DAG (one hd_ctx)."""

    def __init__(self, depth=None, config=None):
        if config is None:
            config = default_config(depth)
        self.config = config
        self._h = C.c_void_p()
        st = lib().hd_create(C.byref(config), C.byref(self._h))
        if st != _capi.HD_OK:
            raise HashDagError(st, "hd_create failed")

    # -- lifetime ----------------------------------------------------------
    def free(self):
        if self._h:
            lib().hd_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def _check(self, st):
        _capi.check(self._h, st)

    @property
    def handle(self):
        return self._h

    @property
    def levels(self):
        return self.config.depth

    def leaf_level(self):
        return self.config.depth - 2

    # -- ingest ------------------------------------------------------------
    def load_from_DAG(self, words):
        """HashDAGFactory::load_from_DAG on BasicDAG words (host array)."""
        words = np.ascontiguousarray(words, np.uint32)
        self._check(lib().hd_load_basic_dag(self._h, words.ctypes.data, words.size))

    def generate_scene(self, seed, shell=False):
        """The seeded scene; shell=True keeps its surface shell (the form the
        coloured scenes use)."""
        self._check(lib().hd_generate_scene_ex(self._h, seed, SCENE_SHELL if shell else 0))

    # -- colours -------------------------------------------------------------
    def colors_from_scene(self, color_seed):
        """HashDAGColors of the current scene from the seeded colour field."""
        self._check(lib().hd_colors_from_scene(self._h, color_seed))

    def get_colors(self, xyz):
        """DAGUtils::get_color for n x 3 voxels: n x 3 array of (colour bits,
        weight, bits per weight)."""
        torch = _torch()
        xyz = np.ascontiguousarray(xyz, np.uint32).reshape(-1, 3)
        d_in = torch.from_numpy(xyz.view(np.int32)).cuda()
        d_out = torch.empty(len(xyz) * 2, dtype=torch.int32, device="cuda")
        self._check(lib().hd_get_colors(self._h, d_in.data_ptr(), len(xyz), d_out.data_ptr()))
        raw = d_out.cpu().numpy().view(np.uint32).reshape(-1, 2)
        return np.stack([raw[:, 0], raw[:, 1] & 0xFF, (raw[:, 1] >> 8) & 0xFF], axis=1)

    def memory_stats(self):
        out = (C.c_uint64 * 4)()
        self._check(lib().hd_memory_stats(self._h, out))
        return dict(zip(("table", "colors", "scratch", "generation_peak"), (int(v) for v in out)))

    def color_stats(self):
        out = (C.c_uint64 * 5)()
        self._check(lib().hd_color_stats(self._h, out))
        return dict(zip(("nodes", "leaves", "blocks", "macro_words", "weight_words"), (int(v) for v in out)))

    # -- undo / redo ---------------------------------------------------------
    def undo(self):
        """HashDAGUndoRedo::undo; False when there is nothing to undo."""
        st = lib().hd_undo(self._h)
        if st == _capi.HD_ERR_STATE:
            return False
        self._check(st)
        return True

    def redo(self):
        st = lib().hd_redo(self._h)
        if st == _capi.HD_ERR_STATE:
            return False
        self._check(st)
        return True

    def history(self):
        u, r = C.c_uint32(), C.c_uint32()
        self._check(lib().hd_history(self._h, C.byref(u), C.byref(r)))
        return u.value, r.value

    def set_undo_capacity(self, frames):
        self._check(lib().hd_set_undo_capacity(self._h, int(frames)))

    # -- files (serializer.h) ------------------------------------------------
    @staticmethod
    def _info(info):
        if info is None:
            return None
        if isinstance(info, _capi.DagInfo):
            return C.byref(info)
        lo, hi = info
        d = _capi.DagInfo()
        d.aabb_min[:] = [float(v) for v in lo]
        d.aabb_max[:] = [float(v) for v in hi]
        return C.byref(d)

    @staticmethod
    def _info_tuple(d):
        return tuple(d.aabb_min), tuple(d.aabb_max)

    def load_dag_from_file(self, path):
        """BasicDAGFactory::load_dag_from_file + load_from_DAG; returns the
        file's DAGInfo as ((min), (max))."""
        d = _capi.DagInfo()
        self._check(lib().hd_load_basic_dag_file(self._h, os.fsencode(path), C.byref(d)))
        return self._info_tuple(d)

    def save_dag_to_file(self, path, info=None):
        """BasicDAGFactory::save_dag_to_file of the last imported or
        generated BasicDAG."""
        self._check(lib().hd_save_basic_dag_file(self._h, os.fsencode(path), self._info(info)))

    def load_compressed_colors_from_file(self, path, enclosed_leaves_compat32=False):
        """BasicDAGFactory::load_compressed_colors_from_file +
        HashDAGFactory::load_colors_from_DAG on the loaded scene."""
        flags = _capi.COLORS_ENCLOSED_32 if enclosed_leaves_compat32 else 0
        self._check(lib().hd_load_colors_file(self._h, os.fsencode(path), flags))

    def save_snapshot(self, path, info=None):
        """The table (and colours) in the reference's hash-DAG file format
        plus bucket sizes, full nodes and colours."""
        self._check(lib().hd_save_snapshot(self._h, os.fsencode(path), self._info(info)))

    def load_snapshot(self, path):
        """A snapshot, or a hash-DAG file the reference wrote (then edits wait
        for remove_stale_nodes); returns the DAGInfo."""
        d = _capi.DagInfo()
        self._check(lib().hd_load_snapshot(self._h, os.fsencode(path), C.byref(d)))
        return self._info_tuple(d)

    def export_basic_dag(self):
        n = C.c_uint64()
        self._check(lib().hd_export_basic_dag(self._h, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.uint32)
        self._check(lib().hd_export_basic_dag(self._h, out.ctypes.data, out.size, C.byref(n)))
        return out

    # -- state -------------------------------------------------------------
    @property
    def firstNodeIndex(self):
        v = C.c_uint32()
        self._check(lib().hd_get_root(self._h, C.byref(v)))
        return v.value

    @firstNodeIndex.setter
    def firstNodeIndex(self, v):
        self._check(lib().hd_set_root(self._h, int(v)))

    def level_stats(self):
        s = LevelStats()
        self._check(lib().hd_get_level_stats(self._h, C.byref(s)))
        return s

    def export_table(self):
        nb, nv, npu = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._check(lib().hd_table_sizes(self._h, C.byref(nb), C.byref(nv), C.byref(npu)))
        bs = np.zeros(nb.value, np.uint32)
        pt = np.zeros(nv.value, np.uint32)
        pool = np.zeros((npu.value + 1) * 512, np.uint32)
        full = np.zeros(self.config.depth, np.uint32)
        self._check(lib().hd_export_table(self._h, bs.ctypes.data, pt.ctypes.data, pool.ctypes.data, pool.size,
                                          full.ctypes.data))
        return dict(bucket_sizes=bs, page_table=pt, pool=pool, full_nodes=full, root=self.firstNodeIndex)

    def import_table(self, t):
        self._check(lib().hd_import_table(self._h, t["bucket_sizes"].ctypes.data, t["page_table"].ctypes.data,
                                          t["pool"].ctypes.data, t["pool"].size, t["full_nodes"].ctypes.data,
                                          int(t["root"])))

    def device_table(self):
        pool, pt, bs = C.c_void_p(), C.c_void_p(), C.c_void_p()
        self._check(lib().hd_device_table(self._h, C.byref(pool), C.byref(pt), C.byref(bs)))
        return pool.value, pt.value, bs.value

    def sync(self):
        self._check(lib().hd_sync(self._h))

    # -- queries -----------------------------------------------------------
    def get_values(self, xyz):
        """DAGUtils::get_value for n x 3 voxel coordinates (host array)."""
        torch = _torch()
        xyz = np.ascontiguousarray(xyz, np.uint32).reshape(-1, 3)
        d_in = torch.from_numpy(xyz.view(np.int32)).cuda()
        d_out = torch.empty(len(xyz), dtype=torch.uint8, device="cuda")
        self._check(lib().hd_get_values(self._h, d_in.data_ptr(), len(xyz), d_out.data_ptr()))
        self.sync()
        return d_out.cpu().numpy()

    # -- edits and GC --------------------------------------------------------
    def edit_threads(self, editor):
        """HashDAG::edit_threads(editor, ...): one edit; returns EditStats."""
        s = EditStats()
        e = editor.to_edit()
        self._check(lib().hd_edit_apply(self._h, C.byref(e), C.byref(s)))
        return s

    def edit_batch(self, editors, per_edit=False):
        """The batched form: the edits in order, one captured CUDA graph per
        edit launched back to back.  Returns the total EditStats, and with
        per_edit=True also the list of per-edit EditStats (device_ms = the
        edit's device time, host_ms = its completion time since the batch
        started)."""
        arr = (Edit * len(editors))(*[e.to_edit() for e in editors])
        s = EditStats()
        per = (EditStats * max(1, len(editors)))()
        self._check(lib().hd_edit_batch_ex(self._h, arr, len(editors), per if per_edit else None, C.byref(s)))
        return (s, list(per)[:len(editors)]) if per_edit else s

    @property
    def batch_tuning(self):
        t = BatchTuning()
        self._check(lib().hd_get_batch_tuning(self._h, C.byref(t)))
        return t

    @batch_tuning.setter
    def batch_tuning(self, t):
        if not isinstance(t, BatchTuning):
            t = BatchTuning(*t)
        self._check(lib().hd_set_batch_tuning(self._h, C.byref(t)))

    def autotune_batch(self, editors):
        """Times every launch shape of the batched path on a device copy of
        the table with these sample edits; keeps and returns the fastest
        (BatchTuning, device ms of the sample)."""
        arr = (Edit * len(editors))(*[e.to_edit() for e in editors])
        t, ms = BatchTuning(), C.c_float()
        self._check(lib().hd_autotune_batch(self._h, arr, len(editors), C.byref(t), C.byref(ms)))
        return t, ms.value

    def batch_fallbacks(self):
        v = C.c_uint64()
        self._check(lib().hd_batch_fallbacks(self._h, C.byref(v)))
        return v.value

    def remove_stale_nodes(self, extra_roots=(), keep_history=False, release_pages=False):
        """HashDAG::remove_stale_nodes(levels - 2), marking from the root and
        from extra_roots; returns the remapped extra roots.  The undo / redo
        history is dropped (as the reference's engine does) unless
        keep_history, which keeps its states alive.  release_pages: pages
        past every bucket's new size go back to a free list."""
        arr = np.array(list(extra_roots) + [0], np.uint32)
        flags = (GC_KEEP_HISTORY if keep_history else 0) | (GC_RELEASE_PAGES if release_pages else 0)
        self._check(lib().hd_gc_ex(self._h, arr.ctypes.data, len(extra_roots), flags))
        return [int(v) for v in arr[:len(extra_roots)]]

    # -- serving loop ----------------------------------------------------------
    def serve(self, requests, continuous=True, max_renders=3, realtime=True, gc_free_fraction=0.1,
              light=(0.3, 1.0, 0.2), shadow_bias=1.0, release_pages=True, batch_edits=True):
        """Runs a request trace (a list of Request, arrival times
        non-decreasing); returns (list of RequestResult, ServeStats)."""
        arr = (Request * max(1, len(requests)))(*requests)
        cfg = ServeConfig(int(continuous), int(max_renders), int(realtime), float(gc_free_fraction),
                          (C.c_float * 3)(*light), float(shadow_bias), int(release_pages), int(batch_edits))
        res = (RequestResult * max(1, len(requests)))()
        st = ServeStats()
        self._check(lib().hd_serve(self._h, arr, len(requests), C.byref(cfg), res, C.byref(st)))
        return list(res)[:len(requests)], st

    def set_fp_mode(self, mode):
        self._check(lib().hd_set_fp_mode(self._h, int(mode)))

    def set_test_barrier_skip(self, cta_plus_one, wait_ms=50):
        """Test hook (hd_set_test_barrier_skip): the next persistent batch
        launch leaves one CTA out of its grid barriers, so the others' waits
        run out after wait_ms and the call fails with HD_ERR_TIMEOUT."""
        self._check(lib().hd_set_test_barrier_skip(self._h, int(cta_plus_one), int(wait_ms)))

    def set_page_reserve(self, pages):
        """Keeps `pages` pool pages back from edits for the GC's rebuild
        (hd_set_page_reserve)."""
        self._check(lib().hd_set_page_reserve(self._h, int(pages)))


class DAGTracer:
    """Headless DAGTracer: results in device buffers (torch tensors)."""

    def __init__(self, width, height):
        torch = _torch()
        self.width, self.height = int(width), int(height)
        self.paths = torch.zeros((self.height, self.width, 4), dtype=torch.int32, device="cuda")
        self.shadows = torch.zeros((self.height, self.width), dtype=torch.uint8, device="cuda")

    def resolve_paths(self, camera, dag):
        """Tracer::trace_paths; returns kernel ms."""
        cam = camera if isinstance(camera, Camera) else Camera.from_params(camera)
        ms = C.c_float()
        dag._check(lib().hd_trace_primary(dag.handle, C.byref(cam), self.width, self.height,
                                          self.paths.data_ptr(), C.byref(ms)))
        return ms.value

    def resolve_shadows(self, camera, dag, shadow_bias=1.0, light=(0.3, 1.0, 0.2)):
        """trace_shadows' hit test from the paths of resolve_paths; returns ms."""
        cam = camera if isinstance(camera, Camera) else Camera.from_params(camera)
        ms = C.c_float()
        lt = (C.c_float * 3)(*light)
        dag._check(lib().hd_trace_shadow(dag.handle, C.byref(cam), self.width, self.height,
                                         self.paths.data_ptr(), lt, float(shadow_bias),
                                         self.shadows.data_ptr(), C.byref(ms)))
        return ms.value

    def resolve_colors(self, dag, debug_colors=DEBUG_NONE, debug_level=0, tool=None):
        """Tracer::trace_colors on the last paths: uint32 RGBA8 per pixel,
        kept in self.colors.  debug_colors: an EDebugColors view (DEBUG_*);
        tool: the ToolInfo overlay as (overlay tool, position, radius,
        copy source, copy dest), or None."""
        torch = _torch()
        if getattr(self, "colors", None) is None:
            self.colors = torch.zeros((self.height, self.width), dtype=torch.int32, device="cuda")
        q = _capi.TraceColorsParams()
        q.debug_colors, q.debug_level = int(debug_colors), int(debug_level)
        if tool is not None:
            kind, pos, radius = tool[:3]
            src, dst = (tool[3], tool[4]) if len(tool) > 3 else ((0, 0, 0), (0, 0, 0))
            q.overlay.enabled, q.overlay.tool, q.overlay.radius = 1, int(kind), float(radius)
            q.overlay.position[:] = [int(v) for v in pos]
            q.overlay.copy_source[:] = [int(v) for v in src]
            q.overlay.copy_dest[:] = [int(v) for v in dst]
        dag._check(lib().hd_trace_colors_ex(dag.handle, self.paths.data_ptr(), self.width, self.height,
                                            self.colors.data_ptr(), C.byref(q)))
        return self.colors.cpu().numpy().view(np.uint32)

    def get_paths(self):
        return self.paths.cpu().numpy().view(np.uint32)

    def get_shadows(self):
        return self.shadows.cpu().numpy()

    def get_path(self, x, y):
        return tuple(int(v) for v in self.paths[y, x, :3].cpu().numpy().view(np.uint32))
