"""Traversal against the reference's own CUDA tracer on the same GPU.

The reference's tracer.cu, compiled unmodified for sm_103a with its own
build's flags (nvcc defaults, --expt-relaxed-constexpr), is
loaded from oracle/_ref and launched as its headless DAGTracer launches it
(oracle/refgpu.py).  Whole 1920 x 1080 frames of the 2^10, 2^12 and 2^15
scenes: the library's paths and shadow masks at its default arithmetic
(fp_mode 0: every operation rounded on its own, which is what nvcc makes of
the reference's code on sm_103a) must equal the reference kernel's bit for
bit.
"""
import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import workloads
from oracle import refgpu

pytestmark = pytest.mark.gpu
LIGHT = (0.3, 1.0, 0.2)
W, H = 1920, 1080


def _poses(depth, n):
    return [workloads.orbit_camera(depth, W, H)] + workloads.catmull_rom_path(depth, 64, W, H)[::64 // n][:n]


@pytest.mark.parametrize("depth,n_path", [(10, 6), (12, 4), (15, 3)])
def test_frames_equal_reference_gpu_tracer(gpu, depth, n_path):
    ctl, bits = workloads.color_tree_levels(depth), workloads.top_bucket_bits(depth)
    if not refgpu.available(depth, ctl, bits):
        pytest.skip("the reference tracer's cubin is built only where the reference sources are")
    d = hd.HashDAG(depth)
    d.generate_scene(workloads.SEED_SCENE)
    ref = refgpu.RefGpuTracer(depth, ctl, bits)
    try:
        assert (ref.width, ref.height) == (W, H)
        ref.set_table(d.export_table())
        tr = hd.DAGTracer(W, H)
        d.set_fp_mode(0)
        for k, cam in enumerate(_poses(depth, n_path)):
            want_paths, want_mask, ms = ref.trace_view(cam, LIGHT, 1.0)
            tr.resolve_paths(cam, d)
            tr.resolve_shadows(cam, d, 1.0, LIGHT)
            paths = np.ascontiguousarray(tr.get_paths()).reshape(H, W, 4)
            mask = np.ascontiguousarray(tr.get_shadows()).reshape(H, W)
            hits = int((want_paths[..., :3] != 0).any(-1).sum())
            assert hits > W * H // 100, (depth, k)
            diff = int((paths != want_paths).any(-1).sum())
            assert diff == 0, f"depth {depth} pose {k}: {diff} pixels differ from the reference kernel"
            assert np.array_equal(mask, want_mask), (depth, k)
            assert ms[0] > 0 and ms[1] > 0
    finally:
        ref.close()
        d.free()


@pytest.mark.parametrize("depth,n_views", [(12, 6), (15, 8)])
def test_views_equal_reference_gpu_tracer(gpu, depth, n_views):
    """The many-view launch (hd_trace_views: camera tables, the shadow-ray
    origin without double divisions, the exact path where those cannot
    decide) against the reference kernel, view by view."""
    import ctypes as C

    import torch
    from hashdag_gb300 import _capi
    ctl, bits = workloads.color_tree_levels(depth), workloads.top_bucket_bits(depth)
    if not refgpu.available(depth, ctl, bits):
        pytest.skip("the reference tracer's cubin is built only where the reference sources are")
    d = hd.HashDAG(depth)
    d.generate_scene(workloads.SEED_SCENE)
    ref = refgpu.RefGpuTracer(depth, ctl, bits)
    try:
        ref.set_table(d.export_table())
        d.set_fp_mode(0)
        poses = workloads.catmull_rom_path(depth, 64, W, H)[::64 // n_views][:n_views]
        cams = (_capi.Camera * n_views)(*[_capi.Camera.from_params(p) for p in poses])
        paths = torch.zeros(n_views * W * H * 4, dtype=torch.int32, device="cuda")
        mask = torch.zeros(n_views * W * H, dtype=torch.uint8, device="cuda")
        light = (C.c_float * 3)(*LIGHT)
        d._check(_capi.lib().hd_trace_views(d.handle, cams, n_views, W, H, paths.data_ptr(), light, 1.0,
                                            mask.data_ptr(), None))
        paths = paths.cpu().numpy().view(np.uint32).reshape(n_views, H, W, 4)
        mask = mask.cpu().numpy().reshape(n_views, H, W)
        for v, cam in enumerate(poses):
            want_paths, want_mask, _ = ref.trace_view(cam, LIGHT, 1.0)
            diff = int((paths[v] != want_paths).any(-1).sum())
            assert diff == 0, f"depth {depth} view {v}: {diff} pixels differ from the reference kernel"
            assert np.array_equal(mask[v], want_mask), (depth, v, int((mask[v] != want_mask).sum()))
    finally:
        ref.close()
        d.free()
