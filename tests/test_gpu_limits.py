"""Capacity limits of the Verlet list.

The list is sized from the start configuration (twice the largest neighbour
count plus a margin).  A denser state set later must grow it, not overflow
it; a list cell holding more beads than the list kernels stage (a collapsed
system) is refused with an error by the kernels' own bounds checks; a state
that is out of its box or not finite is refused before it is loaded.
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


@pytest.mark.parametrize("bad", ["outside", "nan position", "inf velocity"])
def test_refused_state_leaves_the_handle_unchanged(built, bad):
    """smd_set_state checks the staged state on the device before loading it
    (a position outside its replica's box or not finite, a velocity that is
    not finite): the call is refused, the handle keeps its state and runs on."""
    g = load_golden("bil400")
    s = smd.System(mpd_from_golden(g), precision=smd.MIXED)
    p0, v0 = s.state()
    pos, vel = p0.copy(), v0.copy()
    if bad == "outside":
        pos[10, 0] = s.box()[0] + 0.1
    elif bad == "nan position":
        pos[20, 2] = np.nan
    else:
        vel[30, 1] = np.inf
    with pytest.raises(smd.SmdError, match="state is unchanged"):
        s.set_state(pos, vel)
    p1, v1 = s.state()
    assert np.array_equal(p1, p0) and np.array_equal(v1, v0)
    s.set_state(p0, v0)  # a valid state is still taken
    s.prepare()
    s.advance(8)
    p, v = s.state()
    assert np.isfinite(p).all() and np.isfinite(v).all()
    s.close()


def test_failed_allocation_is_not_the_next_launchs_error(built):
    """An adjoint whose checkpoints cannot be allocated (2^30 steps with a
    checkpoint each: tens of terabytes) fails with its own error, and the
    handle's next steps run: the failed cudaMalloc's error is not left as the
    runtime's last error for the next launch check to report."""
    m = mpd_from_golden(load_golden("bil400"))
    m.delta_lxy = 0.0
    s = smd.System(m)
    s.prepare()
    with pytest.raises(smd.SmdError, match="adjoint checkpoints"):
        s.adjoint(1 << 30, checkpoint_every=1)
    s.advance(8)
    pos, vel = s.state()
    assert np.isfinite(pos).all() and np.isfinite(vel).all()
