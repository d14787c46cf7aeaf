"""The replay reader and writer (hd_replay_load / hd_replay_write) against
the reference's own ReplayManager (fixture made by
tests/golden/make_golden_replay.py): every action's cells as load_csv
parses them, the frame count, and write_csv's text byte for byte.  Host
code only: runs without a GPU."""
import json
import os

import numpy as np
import pytest

import hashdag_gb300 as hd

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture():
    with open(os.path.join(GOLDEN, "replay_d10.json")) as f:
        return json.load(f)


def _fields(t, floats, ints, flag):
    """The reference's field order (ref_replay_action) from the parsed cells."""
    if t == "SetToolParameters":
        return [float(v) for v in ints[:9]] + [floats[0], float(ints[9])]
    if t in ("EditSphere", "EditCube"):
        return floats + [float(flag)]
    if t == "EditCopy":
        if len(floats) == 10:  # the reference fills in the identity transform and swirl period 1
            return floats + [1, 0, 0, 0, 1, 0, 0, 0, 1, float(flag), 1.0]
        return floats[:19] + [float(flag), floats[19]]
    return floats


def test_parse_matches_reference_load_csv():
    fx = _fixture()
    r = hd.ReplayManager(os.path.join(GOLDEN, "replay_d10.csv"))
    assert len(r) == len(fx["actions"]) and r.num_frames() == fx["frames"]
    for i, want in enumerate(fx["actions"]):
        t, floats, ints, flag = r.action(i)
        assert t == want["type"], i
        got = np.array(_fields(t, floats, ints, flag), np.float64)
        assert np.array_equal(got.astype(np.float32), np.array(want["fields"], np.float64).astype(np.float32)), i


def test_write_is_reference_write_csv(tmp_path):
    src = os.path.join(GOLDEN, "replay_d10.csv")
    r = hd.ReplayManager(src)
    out = tmp_path / "out.csv"
    r.write_csv(str(out))
    assert out.read_bytes() == open(src, "rb").read()


def test_malformed_lines_are_refused():
    for text in ("EditSphere,1,2,3\n", "Teleport,1\n", "EditCube,1,2,3,4,maybe\n", "SetLocation,a,b,c\n",
                 "SetToolParameters,4294967291,0,0,0,0,0,0,0,0,1.0,1\n"):
        with pytest.raises(hd.HashDagError) as e:
            hd.ReplayManager(text=text)
        assert e.value.status == hd._capi.HD_ERR_INVALID
    # a last line without its newline is not read (load_csv)
    r = hd.ReplayManager(text="EndFrame\nUndo")
    assert len(r) == 1 and r.num_frames() == 1
