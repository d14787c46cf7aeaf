"""GPU parity of the file formats: the library reads the files the
reference's writers produce (rebuilt byte for byte by the oracle and checked
against the fixture's SHA-256) into the state the reference's loaders build,
writes the BasicDAG file the reference writes, reads a reference hash-DAG
file (traced as saved, edited after a GC as the reference edits it after
its GC), and a snapshot round-trips a coloured, edited scene."""
import numpy as np
import pytest

import hashdag_gb300 as hd
from hashdag_gb300 import workloads
from tests import file_fixture as ff

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    fx = ff.fixture()
    d = tmp_path_factory.mktemp("files")
    out = {}
    for name, data in ff.rebuild(fx).items():
        assert ff.sha(data) == fx["files"][name]["sha256"], name
        p = d / name
        p.write_bytes(data)
        out[name] = str(p)
    return fx, out


def _dag(fx):
    o, cfg = ff.config(fx), hd._capi.Config()
    for name, _ in hd._capi.Config._fields_:
        setattr(cfg, name, getattr(o, name))
    return hd.HashDAG(config=cfg)


def test_load_reference_basic_dag_and_colours(gpu, files):
    fx, paths = files
    dag = _dag(fx)
    info = dag.load_dag_from_file(paths[ff.NAMES[0]])
    assert info == ff.info(fx)
    assert dag.firstNodeIndex == fx["reference_load"]["root"]
    dag.load_compressed_colors_from_file(paths[ff.NAMES[1]])
    pts = ff.box_points(fx["boxes"], fx["half"])
    vals = dag.get_values(pts)
    n, digest = ff.colors_digest(pts, vals, dag.get_colors(pts))
    assert (n, digest) == (fx["reference_load"]["present"], fx["reference_load"]["digest"])
    # every slot views the one main leaf
    st = dag.color_stats()
    assert st["blocks"] > 0 and st["leaves"] > 0
    dag.free()


def test_save_basic_dag_file_is_the_reference_bytes(gpu, files, tmp_path):
    fx, paths = files
    dag = _dag(fx)
    dag.generate_scene(fx["seed"], shell=True)
    out = tmp_path / "saved.bin"
    dag.save_dag_to_file(str(out), ff.info(fx))
    assert ff.sha(out.read_bytes()) == fx["files"][ff.NAMES[0]]["sha256"]
    dag.free()


def test_edits_on_file_colours_equal_edits_on_scene_colours(gpu, files):
    """A paint and a carve on the shared main leaf give the colours they give
    on per-slot leaves of the same scene."""
    fx, paths = files
    a, b = _dag(fx), _dag(fx)
    a.load_dag_from_file(paths[ff.NAMES[0]])
    a.load_compressed_colors_from_file(paths[ff.NAMES[1]])
    b.generate_scene(fx["seed"], shell=True)
    b.colors_from_scene(fx["color_seed"])
    for e in fx["edits"]:
        for d in (a, b):
            ed = (hd.SpherePaintEditor(e["center"], e["radius"]) if e["tool"] == hd.TOOL_SPHERE_PAINT
                  else hd.editor_from_tuple((e["tool"], e["center"], e["radius"])))
            d.edit_threads(ed)
    assert a.firstNodeIndex == b.firstNodeIndex == fx["edited"]["root"]
    pts = ff.box_points(fx["boxes"], fx["half"])
    va, vb = a.get_values(pts), b.get_values(pts)
    assert np.array_equal(va, vb)
    assert ff.occupancy_digest(va) == (fx["edited"]["present"], fx["edited"]["digest"])
    assert np.array_equal(a.get_colors(pts)[va.astype(bool)], b.get_colors(pts)[vb.astype(bool)])
    a.free()
    b.free()


def test_reference_hash_dag_file(gpu, files, tmp_path):
    fx, paths = files
    dag = _dag(fx)
    info = dag.load_snapshot(paths[ff.NAMES[2]])
    assert info == ff.info(fx)
    assert dag.firstNodeIndex == fx["edited"]["root"]
    pts = ff.box_points(fx["boxes"], fx["half"])
    assert ff.occupancy_digest(dag.get_values(pts)) == (fx["edited"]["present"], fx["edited"]["digest"])
    # the snapshot writer starts with the reference's format
    out = tmp_path / "snap.bin"
    dag.save_snapshot(str(out), ff.info(fx))
    ref = open(paths[ff.NAMES[2]], "rb").read()
    assert out.read_bytes()[:len(ref)] == ref
    # no bucket sizes: edits wait for the GC
    e = fx["gc_then_edit"]["edit"]
    with pytest.raises(hd.HashDagError) as err:
        dag.edit_threads(hd.editor_from_tuple((e["tool"], e["center"], e["radius"])))
    assert err.value.status == hd._capi.HD_ERR_STATE
    dag.remove_stale_nodes()
    dag.edit_threads(hd.editor_from_tuple((e["tool"], e["center"], e["radius"])))
    got = ff.occupancy_digest(dag.get_values(pts))
    assert got == (fx["gc_then_edit"]["present"], fx["gc_then_edit"]["digest"])
    dag.free()


def test_snapshot_round_trip(gpu, tmp_path):
    depth = 10
    a = hd.HashDAG(depth)
    a.generate_scene(workloads.SEED_SCENE, shell=True)
    a.colors_from_scene(workloads.SEED_COLORS)
    rng = np.random.default_rng(5)
    edits = []
    for tool in (hd.TOOL_SPHERE_REMOVE, hd.TOOL_SPHERE_PAINT, hd.TOOL_BOX_ADD):
        c = [float(v) for v in rng.integers(200, 800, 3)]
        edits.append((tool, c, float(rng.uniform(8, 40))))
    for tool, c, r in edits:
        a.edit_threads(hd.SpherePaintEditor(c, r) if tool == hd.TOOL_SPHERE_PAINT
                       else hd.editor_from_tuple((tool, c, r)))
    path = tmp_path / "scene.snapshot"
    a.save_snapshot(str(path), ((0, 0, 0), (1024, 1024, 1024)))
    b = hd.HashDAG(depth)
    assert b.load_snapshot(str(path)) == ((0.0, 0.0, 0.0), (1024.0, 1024.0, 1024.0))
    assert b.firstNodeIndex == a.firstNodeIndex
    sa, sb = a.level_stats(), b.level_stats()
    assert list(sa.words) == list(sb.words) and list(sa.nodes) == list(sb.nodes)
    assert a.color_stats() == b.color_stats()
    pts = rng.integers(0, 1024, (20000, 3)).astype(np.uint32)
    assert np.array_equal(a.get_values(pts), b.get_values(pts))
    assert np.array_equal(a.get_colors(pts), b.get_colors(pts))
    cam = workloads.orbit_camera(depth, 320, 180)
    ta, tb = hd.DAGTracer(320, 180), hd.DAGTracer(320, 180)
    ta.resolve_paths(cam, a)
    tb.resolve_paths(cam, b)
    assert np.array_equal(ta.get_paths(), tb.get_paths())
    # both stay editable the same way
    for d in (a, b):
        d.edit_threads(hd.editor_from_tuple((hd.TOOL_SPHERE_ADD, [512.0, 600.0, 512.0], 30.0)))
    assert a.firstNodeIndex == b.firstNodeIndex
    a.free()
    b.free()
