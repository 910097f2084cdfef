"""Autotuned launch configurations (smd_autotune / smd_set_tuning): every
list-build kernel and lane count gives bitwise the same mixed-form
trajectory: pair forces are summed in int64 and the list content beyond rc
never reaches the forces."""
import numpy as np
import pytest

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu

# (pair-pass lanes, list kernel)
CONFIGS = [(8, 0), (4, 1), (16, 2), (8, 2), (16, 0)]


def _bilayer(tmp_path):
    p = str(tmp_path / "t.mpd")
    smd.synth_bilayer(p, 31, 1500, 3.45, 16.0, 0.01, 0.2)
    return smd.read_mpd(p)


def test_every_configuration_gives_the_same_trajectory(built, tmp_path):
    m = _bilayer(tmp_path)
    out = []
    for lanes, kern in CONFIGS:
        s = smd.System(m, precision=smd.MIXED)
        s.set_tuning(lanes, kern)
        s.prepare()
        s.advance(160)
        out.append((s.state(), s.box(), s.mc_stats(), s.rebuilds()))
        s.close()
    for (st, box, mc, nb) in out[1:]:
        assert np.array_equal(st[0], out[0][0][0]) and np.array_equal(st[1], out[0][0][1])
        assert np.array_equal(box, out[0][1]) and mc == out[0][2] and nb == out[0][3]


def test_autotune_reports_a_valid_choice(built, tmp_path):
    m = _bilayer(tmp_path)
    s = smd.System(m, precision=smd.MIXED)
    s.prepare()
    r0 = s.rebuilds()
    lanes, kern, ms = s.autotune(force=True)
    assert lanes in (4, 8, 16) and kern in (0, 1, 2)
    assert all(t > 0 for t in ms)
    assert s.rebuilds() == r0  # tuning rebuilds are not run rebuilds
    print(f"lanes {lanes}, list kernel {kern}, list ms {ms[:3]}, pair-pass ms {ms[3:]}")
    s.advance(40)
    t = smd.System(m, precision=smd.MIXED)
    t.set_tuning(8, 0)
    t.prepare()
    t.advance(40)
    assert np.array_equal(s.state()[0], t.state()[0])
