"""ctypes bindings of the C ABI (include/hashdag_gb300.h) over the in-tree
libhashdag_gb300.so.  There is no fallback: importing the bindings without
the built library raises."""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhashdag_gb300.so")

HD_OK, HD_ERR_INVALID, HD_ERR_CUDA, HD_ERR_POOL_FULL, HD_ERR_BUCKET_FULL, HD_ERR_TIMEOUT, HD_ERR_OOM, \
    HD_ERR_STATE, HD_ERR_IO = range(9)
STATUS_NAMES = {0: "HD_OK", 1: "HD_ERR_INVALID", 2: "HD_ERR_CUDA", 3: "HD_ERR_POOL_FULL", 4: "HD_ERR_BUCKET_FULL",
                5: "HD_ERR_TIMEOUT", 6: "HD_ERR_OOM", 7: "HD_ERR_STATE", 8: "HD_ERR_IO"}
COLORS_ENCLOSED_32 = 1
MAX_DEPTH = 20
INVALID_NODE = 0xDFFFFFF


class Config(C.Structure):
    _fields_ = [("depth", C.c_uint32), ("color_tree_levels", C.c_uint32), ("top_levels", C.c_uint32),
                ("top_bucket_bits", C.c_uint32), ("low_bucket_bits", C.c_uint32),
                ("top_bucket_size", C.c_uint32), ("low_bucket_size", C.c_uint32),
                ("pool_pages", C.c_uint32)]


class DagInfo(C.Structure):
    """DAGInfo (dag_info.h:6-10): the scene's bounding box."""
    _fields_ = [("aabb_min", C.c_double * 3), ("aabb_max", C.c_double * 3)]


class ReplayAction(C.Structure):
    _fields_ = [("type", C.c_uint32), ("flag", C.c_uint32), ("n_floats", C.c_uint32), ("n_ints", C.c_uint32),
                ("floats", C.c_float * 20), ("ints", C.c_uint32 * 10)]


class ReplayConfig(C.Structure):
    _fields_ = [("replay_depth", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("reserved", C.c_uint32), ("info", DagInfo)]


class ToolOverlay(C.Structure):
    _fields_ = [("enabled", C.c_uint32), ("tool", C.c_uint32), ("position", C.c_uint32 * 3), ("radius", C.c_float),
                ("copy_source", C.c_uint32 * 3), ("copy_dest", C.c_uint32 * 3)]


class TraceColorsParams(C.Structure):
    _fields_ = [("debug_colors", C.c_uint32), ("debug_level", C.c_uint32), ("overlay", ToolOverlay)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_double * 3), ("ray_min", C.c_double * 3), ("ray_ddx", C.c_double * 3),
                ("ray_ddy", C.c_double * 3)]

    @classmethod
    def from_params(cls, p):
        c = cls()
        for f in ("position", "ray_min", "ray_ddx", "ray_ddy"):
            getattr(c, f)[:] = [float(v) for v in (p[f] if isinstance(p, dict) else getattr(p, f))]
        return c


class Edit(C.Structure):
    _fields_ = [("tool", C.c_uint32), ("center", C.c_float * 3), ("radius", C.c_float), ("rgb", C.c_uint32),
                ("source", C.c_float * 3), ("dest", C.c_float * 3)]


class Color(C.Structure):
    _fields_ = [("color_bits", C.c_uint32), ("weight", C.c_uint8), ("bits_per_weight", C.c_uint8),
                ("reserved", C.c_uint16)]


class EditStats(C.Structure):
    _fields_ = [("num_voxels", C.c_uint64), ("num_nodes", C.c_uint64), ("find_or_add_calls", C.c_uint64),
                ("nodes_added", C.c_uint64), ("words_scanned", C.c_uint64), ("device_ms", C.c_float),
                ("host_ms", C.c_float)]


class BatchTuning(C.Structure):
    _fields_ = [("foa_warps", C.c_uint32), ("probe_words", C.c_uint32), ("grid_blocks", C.c_uint32),
                ("mode", C.c_uint32)]

    def __repr__(self):
        return (f"BatchTuning(foa_warps={self.foa_warps}, probe_words={self.probe_words}, "
                f"grid_blocks={self.grid_blocks}, mode={self.mode})")


class Request(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32), ("reserved", C.c_uint32),
                ("arrival_ms", C.c_double), ("edit", Edit), ("camera", Camera)]


class ServeConfig(C.Structure):
    _fields_ = [("continuous", C.c_uint32), ("max_renders", C.c_uint32), ("realtime", C.c_uint32),
                ("gc_free_fraction", C.c_float), ("light", C.c_float * 3), ("shadow_bias", C.c_float),
                ("release_pages", C.c_uint32), ("batch_edits", C.c_uint32)]


class RequestResult(C.Structure):
    _fields_ = [("start_ms", C.c_double), ("end_ms", C.c_double), ("root", C.c_uint32), ("status", C.c_uint32),
                ("edits_before", C.c_uint32), ("reserved", C.c_uint32), ("checksum", C.c_uint64),
                ("num_voxels", C.c_uint64)]


class ServeStats(C.Structure):
    _fields_ = [("wall_ms", C.c_double), ("edits", C.c_uint32), ("renders", C.c_uint32), ("gcs", C.c_uint32),
                ("refused", C.c_uint32), ("edit_p50_ms", C.c_double), ("edit_p99_ms", C.c_double),
                ("frame_p50_ms", C.c_double), ("frame_p99_ms", C.c_double), ("voxels_per_s", C.c_double),
                ("num_voxels", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class LevelStats(C.Structure):
    _fields_ = [("words", C.c_uint64 * MAX_DEPTH), ("nodes", C.c_uint64 * MAX_DEPTH), ("pages_used", C.c_uint64),
                ("root", C.c_uint32), ("levels", C.c_uint32)]


class HashDagError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


# (name, restype, argtypes) of every exported entry point
_P = C.c_void_p
_u32, _u64, _f32 = C.c_uint32, C.c_uint64, C.c_float
SIGNATURES = [
    ("hd_abi_version", _u32, []),
    ("hd_default_config", None, [_u32, C.POINTER(Config)]),
    ("hd_create", C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
    ("hd_destroy", C.c_int, [_P]),
    ("hd_last_error", C.c_char_p, [_P]),
    ("hd_set_stream", C.c_int, [_P, _P]),
    ("hd_sync", C.c_int, [_P]),
    ("hd_load_basic_dag", C.c_int, [_P, _P, _u64]),
    ("hd_generate_scene", C.c_int, [_P, _u64]),
    ("hd_generate_scene_ex", C.c_int, [_P, _u64, _u32]),
    ("hd_colors_from_scene", C.c_int, [_P, _u64]),
    ("hd_get_colors", C.c_int, [_P, _P, _u64, _P]),
    ("hd_trace_colors", C.c_int, [_P, _P, _u32, _u32, _P]),
    ("hd_trace_colors_ex", C.c_int, [_P, _P, _u32, _u32, _P, C.POINTER(TraceColorsParams)]),
    ("hd_color_stats", C.c_int, [_P, C.POINTER(_u64)]),
    ("hd_memory_stats", C.c_int, [_P, C.POINTER(_u64)]),
    ("hd_undo", C.c_int, [_P]),
    ("hd_redo", C.c_int, [_P]),
    ("hd_set_undo_capacity", C.c_int, [_P, _u32]),
    ("hd_history", C.c_int, [_P, C.POINTER(_u32), C.POINTER(_u32)]),
    ("hd_gc_ex", C.c_int, [_P, _P, _u32, _u32]),
    ("hd_serve", C.c_int, [_P, C.POINTER(Request), _u32, C.POINTER(ServeConfig), C.POINTER(RequestResult),
                           C.POINTER(ServeStats)]),
    ("hd_export_basic_dag", C.c_int, [_P, _P, _u64, C.POINTER(_u64)]),
    ("hd_load_basic_dag_file", C.c_int, [_P, C.c_char_p, C.POINTER(DagInfo)]),
    ("hd_save_basic_dag_file", C.c_int, [_P, C.c_char_p, C.POINTER(DagInfo)]),
    ("hd_load_colors_file", C.c_int, [_P, C.c_char_p, _u32]),
    ("hd_save_snapshot", C.c_int, [_P, C.c_char_p, C.POINTER(DagInfo)]),
    ("hd_camera_from_view", C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double, _u32,
                                      C.POINTER(DagInfo), _u32, _u32, C.POINTER(Camera)]),
    ("hd_replay_load", C.c_int, [C.c_char_p, C.POINTER(_P)]),
    ("hd_replay_load_text", C.c_int, [C.c_char_p, _u64, C.POINTER(_P)]),
    ("hd_replay_free", C.c_int, [_P]),
    ("hd_replay_info", C.c_int, [_P, C.POINTER(_u64), C.POINTER(_u64), C.POINTER(_u64)]),
    ("hd_replay_get_action", C.c_int, [_P, _u64, C.POINTER(ReplayAction)]),
    ("hd_replay_write", C.c_int, [_P, C.c_char_p]),
    ("hd_replay_reset", C.c_int, [_P]),
    ("hd_replay_frame", C.c_int, [_P, _P, C.POINTER(ReplayConfig), C.POINTER(Camera), C.POINTER(_u32)]),
    ("hd_load_snapshot", C.c_int, [_P, C.c_char_p, C.POINTER(DagInfo)]),
    ("hd_trace_primary", C.c_int, [_P, C.POINTER(Camera), _u32, _u32, _P, C.POINTER(_f32)]),
    ("hd_trace_shadow", C.c_int, [_P, C.POINTER(Camera), _u32, _u32, _P, C.POINTER(_f32), _f32, _P,
                                  C.POINTER(_f32)]),
    ("hd_trace_frame", C.c_int, [_P, C.POINTER(Camera), _u32, _u32, C.POINTER(_f32), _f32, _P, _P,
                                 C.POINTER(_f32), C.POINTER(_f32)]),
    ("hd_trace_views", C.c_int, [_P, C.POINTER(Camera), _u32, _u32, _u32, _P, C.POINTER(_f32), _f32, _P,
                                 C.POINTER(_f32)]),
    ("hd_trace_views_host", C.c_int, [_P, C.POINTER(Camera), _u32, _u32, _u32, _P, C.POINTER(_f32), _f32, _P, _u32,
                                      C.POINTER(_f32)]),
    ("hd_trace_counters", C.c_int, [_P, C.POINTER(Camera), _u32, _u32, C.POINTER(_f32), _f32, _P, _P,
                                    C.POINTER(_u64)]),
    ("hd_trace_counters_noalloc", C.c_int, [_P, C.POINTER(Camera), _u32, _u32, C.POINTER(_f32), _f32, _P, _P,
                                            C.POINTER(_u64)]),
    ("hd_set_fp_mode", C.c_int, [_P, _u32]),
    ("hd_set_page_reserve", C.c_int, [_P, _u32]),
    ("hd_set_test_barrier_skip", C.c_int, [_P, _u32, _u32]),
    ("hd_get_values", C.c_int, [_P, _P, _u64, _P]),
    ("hd_edit_apply", C.c_int, [_P, C.POINTER(Edit), C.POINTER(EditStats)]),
    ("hd_edit_batch", C.c_int, [_P, C.POINTER(Edit), _u32, C.POINTER(EditStats)]),
    ("hd_edit_batch_ex", C.c_int, [_P, C.POINTER(Edit), _u32, C.POINTER(EditStats), C.POINTER(EditStats)]),
    ("hd_set_batch_tuning", C.c_int, [_P, C.POINTER(BatchTuning)]),
    ("hd_get_batch_tuning", C.c_int, [_P, C.POINTER(BatchTuning)]),
    ("hd_autotune_batch", C.c_int, [_P, C.POINTER(Edit), _u32, C.POINTER(BatchTuning), C.POINTER(_f32)]),
    ("hd_batch_fallbacks", C.c_int, [_P, C.POINTER(_u64)]),
    ("hd_gc", C.c_int, [_P, _P, _u32]),
    ("hd_get_root", C.c_int, [_P, C.POINTER(_u32)]),
    ("hd_set_root", C.c_int, [_P, _u32]),
    ("hd_get_config", C.c_int, [_P, C.POINTER(Config)]),
    ("hd_get_level_stats", C.c_int, [_P, C.POINTER(LevelStats)]),
    ("hd_table_sizes", C.c_int, [_P, C.POINTER(_u64), C.POINTER(_u64), C.POINTER(_u64)]),
    ("hd_export_table", C.c_int, [_P, _P, _P, _P, _u64, _P]),
    ("hd_import_table", C.c_int, [_P, _P, _P, _P, _u64, _P, _u32]),
    ("hd_device_table", C.c_int, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
]

_lib = None


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m hashdag_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(ctx, status):
    if status != HD_OK:
        msg = lib().hd_last_error(ctx)
        raise HashDagError(status, msg.decode() if msg else "")
