"""The oracle's restatement of the reference's file formats (BasicDAG,
compressed colours, hash-DAG file) rebuilds, byte for byte, the files the
reference's own writers produced (fixture made by
tests/golden/make_golden_files.py), and the colours the reference's loaders
read from them are the oracle's colours of the same scene."""
import numpy as np

from oracle import pyoracle as po
from tests import file_fixture as ff


def test_rebuilt_files_equal_the_reference_writers():
    fx = ff.fixture()
    files = ff.rebuild(fx)
    for name in ff.NAMES:
        assert len(files[name]) == fx["files"][name]["bytes"], name
        assert ff.sha(files[name]) == fx["files"][name]["sha256"], name


def test_reference_loaders_read_the_oracle_colours():
    fx = ff.fixture()
    D, T = fx["depth"], fx["color_tree_levels"]
    t = po.Table(ff.config(fx))
    t.load_basic_dag(po.generate_basic_dag(fx["seed"], D, T, flags=po.SCENE_SHELL))
    assert t.root == fx["reference_load"]["root"] == fx["base"]["root"]
    col = po.Colors(t)
    col.from_scene(fx["color_seed"])
    pts = ff.box_points(fx["boxes"], fx["half"])
    vals = [t.get_value(*p) for p in pts]
    cols = [col.get_color(*p) for p in pts]
    n, digest = ff.colors_digest(pts, vals, cols)
    assert (n, digest) == (fx["reference_load"]["present"], fx["reference_load"]["digest"])
    assert ff.occupancy_digest(vals) == (fx["base"]["present"], fx["base"]["digest"])
