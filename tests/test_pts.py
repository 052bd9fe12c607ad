"""The .pts point files (SavePoints / RunPlayback layout) on the CPU: the
writer's bytes against the reference layout parsed independently, a file in
the reference's three-field layout read back, and malformed files."""
from __future__ import annotations

import struct

import numpy as np
import pytest

import fluids3_gb300 as F
from fluids3_gb300 import scenes
from fluids3_gb300.pts import read_pts, write_pts

from helpers import assert_bit_equal


def _reference_layout(n, pos, vel, clr, veval=None):
    """SavePoints' bytes (fluid_system.cpp:1511-1545), built field by field."""
    out = struct.pack("<ii", n, 4 if veval is not None else 3)
    out += struct.pack("<ii", 2, 3) + pos.astype("<f4").tobytes()
    out += struct.pack("<ii", 2, 3) + vel.astype("<f4").tobytes()
    out += struct.pack("<ii", 0, 4) + clr.astype("<u4").tobytes()
    if veval is not None:
        out += struct.pack("<ii", 2, 3) + veval.astype("<f4").tobytes()
    return out


def test_pts_write_matches_the_reference_layout(tmp_path):
    sc = scenes.dam_break(n=777)
    ve = np.random.default_rng(1).standard_normal((777, 3)).astype(np.float32)
    for veval in (None, ve):
        p = tmp_path / "a.pts"
        write_pts(p, sc.pos, sc.vel, sc.clr, veval)
        assert p.read_bytes() == _reference_layout(777, sc.pos, sc.vel, sc.clr, veval)
        got = read_pts(p)
        assert got["nfields"] == (3 if veval is None else 4)
        assert_bit_equal(got["pos"], sc.pos, "pos")
        assert_bit_equal(got["vel"], sc.vel, "vel")
        assert_bit_equal(got["clr"], sc.clr, "clr")
        if veval is None:
            assert got["veval"] is None
        else:
            assert_bit_equal(got["veval"], veval, "veval")


def test_pts_reads_a_three_field_file_and_rejects_broken_ones(tmp_path):
    rng = np.random.default_rng(2)
    pos = rng.standard_normal((50, 3)).astype(np.float32)
    vel = rng.standard_normal((50, 3)).astype(np.float32)
    clr = rng.integers(0, 2**32, 50, dtype=np.uint32)
    p = tmp_path / "ref.pts"
    p.write_bytes(_reference_layout(50, pos, vel, clr))
    got = read_pts(p)
    assert_bit_equal(got["pos"], pos, "pos")
    assert_bit_equal(got["clr"], clr, "clr")
    bad = tmp_path / "bad.pts"
    bad.write_bytes(_reference_layout(50, pos, vel, clr)[:-7])            # truncated colour field
    with pytest.raises(F.FluidsError) as e:
        read_pts(bad)
    assert e.value.code == -8
    bad.write_bytes(struct.pack("<ii", 5, 3) + struct.pack("<ii", 3, 3))  # double positions: not this layout
    with pytest.raises(F.FluidsError) as e:
        read_pts(bad)
    assert e.value.code == -8 and "type 3 x 3" in str(e.value)
    with pytest.raises(F.FluidsError):
        read_pts(tmp_path / "missing.pts")
    empty = tmp_path / "empty.pts"
    write_pts(empty, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros(0, np.uint32))
    assert read_pts(empty)["pos"].shape == (0, 3)
