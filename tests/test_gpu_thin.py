"""Boxes with fewer than three Verlet-list cells on an axis.

The reference's CellOpt grid needs L >= 3 rc per axis; the Verlet-list grid
of the device (cells of at least rc + skin) has only two cells on an axis
with 3 rc <= L < 3 (rc + skin).  The list build then applies a minimum image
per candidate and guards its padding sentinels.  Here the 400-lipid bilayer
fixture is folded into a box 6.5 sigma high (3 reference cells, 2 list cells
in z): forces, cell keys and the set of pairs within rc against the oracle,
then a run through list rebuilds.
"""
import numpy as np
import pytest
from conftest import load_golden, mpd_from_golden

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu

FORCE_TOL = {smd.PLAIN_FP64: 1e-12, smd.MIXED: 1e-5}


def _thin():
    g = dict(load_golden("bil400"))
    box = np.array(g["box"], np.float64).copy()
    box[2] = 6.5
    g["box"] = box
    g["pos"] = np.mod(np.asarray(g["pos"], np.float64), box)
    return g


@pytest.mark.parametrize("precision", [smd.PLAIN_FP64, smd.MIXED])
def test_thin_box_matches_oracle(built, oracle, precision):
    g = _thin()
    rc = float(g["cutoff"])
    assert int(g["box"][2] // rc) == 3 and int(g["box"][2] // (rc + 0.5)) == 2
    ref = oracle.forces(g)
    s = smd.System(mpd_from_golden(g), precision=precision)
    err = np.abs(s.forces() - ref).max() / np.abs(ref).max()
    assert err <= FORCE_TOL[precision], err
    assert np.array_equal(s.cell_keys(), oracle.cell_keys(g["pos"], g["box"], rc))
    want = np.sort(oracle.pair_list(g["pos"], g["box"], rc), axis=1)
    got = np.sort(s.pair_list(), axis=1)
    want = want[np.lexsort((want[:, 1], want[:, 0]))]
    got = got[np.lexsort((got[:, 1], got[:, 0]))]
    assert got.shape == want.shape and np.array_equal(got, want)
    s.close()


@pytest.mark.parametrize("precision", [smd.PLAIN_FP64, smd.MIXED])
def test_thin_box_runs_through_rebuilds(built, oracle, precision):
    g = _thin()
    s = smd.System(mpd_from_golden(g), precision=precision)
    s.prepare()
    s.advance(64)
    pos, vel = s.state()
    assert np.isfinite(pos).all() and np.isfinite(vel).all()
    assert s.rebuilds() >= 8
    # the list built on the moved state still gives the oracle's forces (in
    # the box the barostat left)
    moved = dict(g)
    moved["pos"] = pos
    moved["box"] = s.box()
    ref = oracle.forces(moved)
    err = np.abs(s.forces() - ref).max() / np.abs(ref).max()
    assert err <= FORCE_TOL[precision], err
    s.close()
