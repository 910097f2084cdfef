"""Capacity limits of the Verlet list.

The list is sized from the start configuration (twice the largest neighbour
count plus a margin).  A denser state set later must grow it, not overflow
it; a list cell holding more beads than the list kernels stage (a collapsed
system) is refused with an error by the kernels' own bounds checks.
"""
import numpy as np
import pytest
from conftest import load_golden, mpd_from_golden

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [(smd.PLAIN_FP64, 1e-12), (smd.MIXED, 1e-5)])
def test_denser_state_grows_the_list(built, oracle, precision, tol):
    """The bilayer squeezed to 0.35 of its thickness (about three times the
    neighbours per bead) through smd_set_state: forces against the oracle."""
    g = dict(load_golden("bil400"))
    s = smd.System(mpd_from_golden(g), precision=precision)
    pos = np.array(g["pos"], np.float64)
    zc = np.median(pos[:, 2])
    pos[:, 2] = zc + 0.35 * (pos[:, 2] - zc)
    s.set_state(pos, np.array(g["vel"], np.float64))
    squeezed = dict(g)
    squeezed["pos"] = pos
    ref = oracle.forces(squeezed)
    err = np.abs(s.forces() - ref).max() / np.abs(ref).max()
    assert err <= tol, err
    # and the squeezed state runs on
    s.prepare()
    s.advance(16)
    p, v = s.state()
    assert np.isfinite(p).all() and np.isfinite(v).all()
    s.close()


def test_collapsed_cell_is_refused(built):
    """1,100 beads in one list cell (the kernels stage at most 1,024)."""
    g = dict(load_golden("bil400"))
    rng = np.random.default_rng(3)
    n = 1100
    box = np.array([7.5, 7.5, 7.5])
    m = mpd_from_golden(g)
    import dataclasses
    m = dataclasses.replace(m, pos=rng.uniform(0.05, 2.4, (n, 3)), vel=np.zeros((n, 3)),
                            type=rng.choice([2, 3], n).astype(np.int32), box=box,
                            chain_blocks=np.zeros((0, 3), np.int32), chain_consts=np.zeros((0, 4)),
                            delta_lxy=0.0)
    with pytest.raises(smd.SmdError, match="more than 1024 beads"):
        smd.System(m, precision=smd.MIXED)
