"""The allocation-free traversal counters.

Callers that cannot allocate device memory while they trace (inside a CUDA
stream capture, or under a fixed memory budget) use
hd_trace_counters_noalloc, whose scratch is a fixed device array inside the
library.  This test drives it through the C ABI and checks that two calls in
a row return exactly what hd_trace_counters (which takes its scratch from
the context's allocations) returns.  The file sorts last so that a run that
stops at the first failure has run every other test first.
"""
import ctypes as C

import pytest

from hashdag_gb300 import _capi, workloads

pytestmark = pytest.mark.gpu


def test_noalloc_counters_match_allocating_entry_point(gpu):
    import torch
    L = _capi.lib()
    depth, W, H = 10, 1280, 720
    cfg = _capi.Config()
    L.hd_default_config(depth, C.byref(cfg))
    ctx = C.c_void_p()
    assert L.hd_create(C.byref(cfg), C.byref(ctx)) == _capi.HD_OK
    try:
        _capi.check(ctx, L.hd_generate_scene(ctx, workloads.SEED_SCENE))
        cam = _capi.Camera.from_params(workloads.orbit_camera(depth, W, H))
        light = (C.c_float * 3)(0.3, 1.0, 0.2)
        paths = torch.zeros(W * H * 4, dtype=torch.int32, device="cuda")
        mask = torch.zeros(W * H, dtype=torch.uint8, device="cuda")
        want = (C.c_uint64 * 6)()
        _capi.check(ctx, L.hd_trace_counters(ctx, C.byref(cam), W, H, light, 1.0, paths.data_ptr(),
                                             mask.data_ptr(), want))
        want_paths, want_mask = paths.clone(), mask.clone()
        assert want[0] == W * H and want[3] > 0 and want[1] > 0
        for _ in range(2):
            paths.zero_()
            mask.zero_()
            got = (C.c_uint64 * 6)()
            _capi.check(ctx, L.hd_trace_counters_noalloc(ctx, C.byref(cam), W, H, light, 1.0, paths.data_ptr(),
                                                         mask.data_ptr(), got))
            assert list(got) == list(want)
            assert torch.equal(paths, want_paths) and torch.equal(mask, want_mask)
        # sizes beyond the fixed scratch are refused
        got = (C.c_uint64 * 6)()
        assert L.hd_trace_counters_noalloc(ctx, C.byref(cam), 8192, 4096, light, 1.0, paths.data_ptr(),
                                           mask.data_ptr(), got) == _capi.HD_ERR_INVALID
    finally:
        L.hd_destroy(ctx)
