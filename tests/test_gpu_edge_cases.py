"""Edge cases of the GPU path against the oracle: cameras inside the volume,
inside solid ground, looking away, rays and lights along the axes (zero
direction components, infinite reciprocals), tiny and odd image sizes;
edits that touch nothing, that fill the whole volume or would empty it;
empty batches; roots and imported tables that do not describe a table."""
import os

import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import workloads
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
DEPTH = 10
E = float(1 << DEPTH)
LIGHT = (0.3, 1.0, 0.2)


def _scene():
    d = hd.HashDAG(DEPTH)
    d.generate_scene(workloads.SEED_SCENE)
    return d


def _oracle():
    t = po.Table(po.default_config(DEPTH))
    t.load_basic_dag(po.generate_basic_dag(workloads.SEED_SCENE, DEPTH, workloads.color_tree_levels(DEPTH)))
    return t


def _axis_camera(position, forward, right, up, step):
    """Pixel (0, 0) looks exactly along `forward`; pixel (x, y) along
    forward + x step right + y step up (step a power of two, so every
    direction component is exact)."""
    p = np.asarray(position, np.float64)
    return dict(position=p.tolist(), ray_min=(p + np.asarray(forward, np.float64)).tolist(),
                ray_ddx=(step * np.asarray(right, np.float64)).tolist(),
                ray_ddy=(step * np.asarray(up, np.float64)).tolist())


CAMERAS = {
    "inside_air": lambda w, h: workloads.trace_params((0.5 * E, 0.97 * E, 0.41 * E), (0.8 * E, 0.6 * E, 0.7 * E), w, h),
    "inside_solid": lambda w, h: workloads.trace_params((0.5 * E, 3.0, 0.5 * E), (E, 3.0, 0.6 * E), w, h),
    "looking_away": lambda w, h: workloads.trace_params((-0.5 * E, 0.5 * E, 0.5 * E), (-2.0 * E, 0.5 * E, 0.5 * E),
                                                        w, h),
    "down_the_y_axis": lambda w, h: _axis_camera((0.5 * E + 0.5, 2.0 * E, 0.5 * E + 0.5), (0, -1, 0), (1, 0, 0),
                                                 (0, 0, 1), 2.0 ** -7),
    "along_x_on_a_node_plane": lambda w, h: _axis_camera((-3.0, 0.5 * E, 0.25 * E), (1, 0, 0), (0, 0, 1),
                                                         (0, 1, 0), 2.0 ** -8),
    "grazing_the_box_edge": lambda w, h: workloads.trace_params((-E, E, -E), (0.0, E, 0.0), w, h, fov_deg=30.0),
}


@pytest.mark.parametrize("name", sorted(CAMERAS))
@pytest.mark.parametrize("size", [(1, 1), (33, 17), (160, 96)])
@pytest.mark.parametrize("light", [LIGHT, (0.0, 1.0, 0.0), (1.0, 0.0, 0.0)])
def test_edge_cameras_match_oracle(gpu, name, size, light):
    w, h = size
    d = _edge_cache("dag", _scene)
    ot = _edge_cache("oracle", _oracle)
    cam = CAMERAS[name](w, h)
    tr = hd.DAGTracer(w, h)
    tr.resolve_paths(cam, d)
    tr.resolve_shadows(cam, d, 1.0, light)
    paths, mask = ot.trace_frame(cam, w, h, light, 1.0, threads=os.cpu_count() or 4)
    assert np.array_equal(tr.get_paths(), paths)
    assert np.array_equal(tr.get_shadows(), mask)
    if name == "looking_away":  # every ray misses: no path, the miss value 2 in the mask
        assert not paths.any() and (mask == 2).all()


_cache = {}


def _edge_cache(key, make):
    if key not in _cache:
        _cache[key] = make()
    return _cache[key]


@pytest.mark.parametrize("edit", [
    (0, (0.5 * E, 0.5 * E, 0.5 * E), 0.0),          # radius 0: touches nothing
    (1, (-400.0, -400.0, -400.0), 100.0),           # a fill wholly outside the volume
    (0, (E + 300.0, 0.5 * E, 0.5 * E), 299.5),      # a carve just short of the volume
    (3, (0.5 * E, 0.5 * E, 0.5 * E), E),            # a box fill over the whole volume
    (1, (0.5 * E, 0.5 * E, 0.5 * E), E),            # a sphere fill over the whole volume
    (2, (0.5, 0.5, 0.5), 0.5),                      # a box carve of one corner voxel
])
def test_degenerate_edits_match_oracle(gpu, edit):
    d = _scene()
    ot = _oracle()
    s = d.edit_threads(hd.editor_from_tuple(edit))
    os_ = ot.edit(*edit)
    assert d.firstNodeIndex == ot.root
    assert (s.num_voxels, s.num_nodes, s.find_or_add_calls, s.nodes_added) == \
        (os_.num_voxels, os_.num_nodes, os_.find_or_add_calls, os_.nodes_added)
    w, h = 96, 64
    cam = workloads.orbit_camera(DEPTH, w, h)
    tr = hd.DAGTracer(w, h)
    tr.resolve_paths(cam, d)
    tr.resolve_shadows(cam, d, 1.0, LIGHT)
    paths, mask = ot.trace_frame(cam, w, h, LIGHT, 1.0)
    assert np.array_equal(tr.get_paths(), paths)
    assert np.array_equal(tr.get_shadows(), mask)
    d.free()


CARVE_ALL = (0, (0.5 * E, 0.5 * E, 0.5 * E), E)


def test_edit_that_would_empty_the_scene_is_refused(gpu):
    """The reference would leave an invalid root; the library refuses the
    edit with HD_ERR_STATE and keeps the scene, on both edit paths."""
    d = _scene()
    root = d.firstNodeIndex
    with pytest.raises(hd.HashDagError) as err:
        d.edit_threads(hd.editor_from_tuple(CARVE_ALL))
    assert err.value.status == hd._capi.HD_ERR_STATE
    assert d.firstNodeIndex == root
    q = np.array([[int(0.5 * E), 2, int(0.5 * E)]], np.uint32)
    assert d.get_values(q)[0] == 1
    # batched: the edits before the refused one stay applied
    first = workloads.mixed_edits(DEPTH, 2, (4.0, 40.0), seed=9)
    a = _scene()
    a.edit_threads(hd.editor_from_tuple(first[0]))
    with pytest.raises(hd.HashDagError) as err:
        d.edit_batch([hd.editor_from_tuple(first[0]), hd.editor_from_tuple(CARVE_ALL),
                      hd.editor_from_tuple(first[1])])
    assert err.value.status == hd._capi.HD_ERR_STATE
    assert d.firstNodeIndex == a.firstNodeIndex
    d.free()
    a.free()


def test_empty_batch_changes_nothing(gpu):
    d = _scene()
    root = d.firstNodeIndex
    total, per = d.edit_batch([], per_edit=True)
    assert per == [] and total.num_voxels == 0 and total.find_or_add_calls == 0
    assert d.firstNodeIndex == root
    d.free()


def test_roots_off_the_table_are_refused(gpu):
    d = _scene()
    root = d.firstNodeIndex
    for bad in (hd._capi.INVALID_NODE, 0xFFFFFFFF, 5):   # 5: on the never-mapped page 0
        with pytest.raises(hd.HashDagError) as err:
            d.firstNodeIndex = bad
        assert err.value.status == hd._capi.HD_ERR_INVALID
        assert d.firstNodeIndex == root
    d.firstNodeIndex = root
    d.free()


def test_import_checks_the_table(gpu):
    d = _scene()
    t = d.export_table()
    top = int(t["pool"].size // 512)
    e = hd.HashDAG(DEPTH)
    bad_pt = t["page_table"].copy()
    bad_pt[np.nonzero(bad_pt)[0][0]] = top          # a page past the pool
    bad_bs = t["bucket_sizes"].copy()
    bad_bs[0] = 1 << 20                              # more than a bucket holds
    for kw in (dict(page_table=bad_pt), dict(bucket_sizes=bad_bs), dict(root=hd._capi.INVALID_NODE)):
        tt = dict(t, **kw)
        with pytest.raises(hd.HashDagError) as err:
            e.import_table(tt)
        assert err.value.status == hd._capi.HD_ERR_INVALID
    e.import_table(t)
    assert e.firstNodeIndex == d.firstNodeIndex
    w, h = 64, 48
    cam = workloads.orbit_camera(DEPTH, w, h)
    a, b = hd.DAGTracer(w, h), hd.DAGTracer(w, h)
    a.resolve_paths(cam, d)
    b.resolve_paths(cam, e)
    assert np.array_equal(a.get_paths(), b.get_paths())
    d.free()
    e.free()
