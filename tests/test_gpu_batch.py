"""Batched replicas (independent systems of uneven size, seeds and tensions
advancing in the same launches with per-replica offsets).

A replica's forces and trajectory must not depend on the batch it runs in:
in the mixed form (order-independent fixed-point force sums, noise keyed by
the replica's own seed, barostat energy differences summed in fixed point)
they are bitwise identical to the system run alone.
"""
import numpy as np
import pytest
from conftest import load_golden, mpd_from_golden

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu


def _systems(tmp_path):
    ms = [mpd_from_golden(load_golden("bil400")), mpd_from_golden(load_golden("ves300"))]
    p = str(tmp_path / "t.mpd")
    smd.synth_bilayer(p, 31, 500, 3.45, 18.0, 0.01, 0.5)  # tension 0.5, own seed and box
    ms.append(smd.read_mpd(p))
    return ms


@pytest.mark.parametrize("precision", [smd.MIXED, smd.PLAIN_FP64])
def test_batch_forces_equal_single_system(built, tmp_path, precision):
    ms = _systems(tmp_path)
    b = smd.System(ms, precision=precision)
    fb = b.forces()
    off = 0
    for m in ms:
        n = len(m.type)
        f = smd.System(m, precision=precision).forces()
        if precision == smd.MIXED:
            assert np.array_equal(fb[off:off + n], f)
        else:
            assert np.abs(fb[off:off + n] - f).max() <= 1e-12 * np.abs(f).max()
        off += n
    assert off == len(fb)


def test_batch_trajectories_equal_single_runs(built, tmp_path):
    ms = _systems(tmp_path)
    b = smd.System(ms, precision=smd.MIXED)
    b.prepare()
    b.advance(120)  # includes barostat trials for the two bilayers
    pb, vb = b.state()
    off = 0
    for k, m in enumerate(ms):
        n = len(m.type)
        s = smd.System(m, precision=smd.MIXED)
        s.prepare()
        s.advance(120)
        p, v = s.state()
        assert np.array_equal(pb[off:off + n], p), k
        assert np.array_equal(vb[off:off + n], v), k
        assert np.array_equal(b.box(k), s.box()), k
        assert b.mc_stats(k) == s.mc_stats(), k
        off += n
    assert b.mc_stats(0)["trials"] >= 14 and b.mc_stats(2)["trials"] >= 14
    assert b.mc_stats(1)["trials"] == 0  # the vesicle runs without the barostat
