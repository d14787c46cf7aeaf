"""The allocation-free traversal counters.

Some callers cannot call cudaMalloc while they trace: an application that
reserves the device memory budget at start-up and forbids later
allocations, or a real-time loop that cannot take the device-wide
synchronisation an allocation may cause.  They use
hd_trace_counters_noalloc, whose scratch is a fixed device array inside the
library.  This test drives it through the C ABI and checks that calls in a
row return exactly what hd_trace_counters (which takes its scratch from the
context's allocations) returns: in both arithmetic modes, at the largest
accepted image, and on a small frame right after that large one (the shared
array keeps the large call's partial sums).  The file sorts last so that a
run that stops at the first failure has run every other test first.
"""
import ctypes as C

import pytest

from hashdag_gb300 import _capi, workloads

pytestmark = pytest.mark.gpu


def _trace(L, ctx, fn, cam, W, H, light, paths, mask):
    paths.zero_()
    mask.zero_()
    out = (C.c_uint64 * 6)()
    _capi.check(ctx, fn(ctx, C.byref(cam), W, H, light, 1.0, paths.data_ptr(), mask.data_ptr(), out))
    return list(out), paths[: W * H * 4].clone(), mask[: W * H].clone()


def test_noalloc_counters_match_allocating_entry_point(gpu):
    import torch
    L = _capi.lib()
    depth = 10
    cfg = _capi.Config()
    L.hd_default_config(depth, C.byref(cfg))
    ctx = C.c_void_p()
    assert L.hd_create(C.byref(cfg), C.byref(ctx)) == _capi.HD_OK
    try:
        _capi.check(ctx, L.hd_generate_scene(ctx, workloads.SEED_SCENE))
        light = (C.c_float * 3)(0.3, 1.0, 0.2)
        big = 4096 * 4096
        paths = torch.zeros(big * 4, dtype=torch.int32, device="cuda")
        mask = torch.zeros(big, dtype=torch.uint8, device="cuda")
        # small, largest accepted (262144 blocks), then small again: the
        # second small call follows a call that filled the whole array
        for fp_mode in (1, 0):
            _capi.check(ctx, L.hd_set_fp_mode(ctx, fp_mode))
            for W, H in ((1280, 720), (4096, 4096), (1280, 720), (33, 17)):
                cam = _capi.Camera.from_params(workloads.orbit_camera(depth, W, H))
                want = _trace(L, ctx, L.hd_trace_counters, cam, W, H, light, paths, mask)
                assert want[0][0] == W * H and want[0][1] > 0
                for _ in range(2):
                    got = _trace(L, ctx, L.hd_trace_counters_noalloc, cam, W, H, light, paths, mask)
                    assert got[0] == want[0], (fp_mode, W, H)
                    assert torch.equal(got[1], want[1]) and torch.equal(got[2], want[2]), (fp_mode, W, H)
        # sizes beyond the fixed scratch, or taller than a launch grid
        # allows, are refused before anything runs
        cam = _capi.Camera.from_params(workloads.orbit_camera(depth, 1280, 720))
        got = (C.c_uint64 * 6)()
        for W, H in ((8192, 4096), (4104, 4096), (8, 600000)):
            assert L.hd_trace_counters_noalloc(ctx, C.byref(cam), W, H, light, 1.0, paths.data_ptr(),
                                               mask.data_ptr(), got) == _capi.HD_ERR_INVALID, (W, H)
            assert b"exceeds" in L.hd_last_error(ctx)
        # the allocating entry point refuses the tall image too
        assert L.hd_trace_counters(ctx, C.byref(cam), 8, 600000, light, 1.0, paths.data_ptr(), mask.data_ptr(),
                                   got) == _capi.HD_ERR_INVALID
    finally:
        L.hd_destroy(ctx)
