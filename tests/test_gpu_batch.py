"""Batched replicas (independent systems of uneven size, seeds and tensions
advancing in the same launches with per-replica offsets).

A replica's forces and trajectory must not depend on the batch it runs in:
in the mixed form (order-independent fixed-point force sums, noise keyed by
the replica's own seed, barostat energy differences summed in fixed point)
they are bitwise identical to the system run alone.
"""
import numpy as np
import pytest

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu


def _systems(tmp_path):
    """Three bilayers sharing the pair tables: own sizes, seeds and boxes;
    tension 0 and 0.5 with the barostat, and one without it."""
    ms = []
    for k, (seed, lipids, dlxy, tension) in enumerate(((31, 400, 0.01, 0.0), (32, 260, 0.0, 0.0),
                                                       (33, 500, 0.01, 0.5))):
        p = str(tmp_path / f"t{k}.mpd")
        smd.synth_bilayer(p, seed, lipids, 3.45, 18.0, dlxy, tension)
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
    assert b.mc_stats(1)["trials"] == 0  # replica 1 runs without the barostat
