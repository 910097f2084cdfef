"""The loop as CUDA graphs (one MC period per graph, the list build of each
step a conditional node) against the same loop launched kernel by kernel
(profiling mode records events around every step, so it never uses graphs).
In the mixed form the two trajectories are bitwise identical."""
import numpy as np
import pytest

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu


def _bilayer(tmp_path, tension=0.0):
    p = str(tmp_path / "g.mpd")
    smd.synth_bilayer(p, 77, 600, 3.45, 18.0, 0.01, tension)
    return smd.read_mpd(p)


def _run(m, graphs, steps, precision=smd.MIXED, stop=False):
    s = smd.System(m, precision=precision)
    s.profile(not graphs)
    s.prepare()
    l0 = s.launches()
    s.advance(steps, stop_at_measure=stop)
    pos, vel = s.state()
    return dict(pos=pos, vel=vel, box=s.box(), mc=s.mc_stats(), rebuilds=s.rebuilds(), launches=s.launches() - l0)


@pytest.mark.parametrize("tension", [0.0, 0.5])
def test_graph_loop_matches_kernel_by_kernel(built, tmp_path, tension):
    m = _bilayer(tmp_path, tension)
    a = _run(m, graphs=True, steps=203)
    b = _run(m, graphs=False, steps=203)
    assert np.array_equal(a["pos"], b["pos"])
    assert np.array_equal(a["vel"], b["vel"])
    assert np.array_equal(a["box"], b["box"])
    assert a["mc"] == b["mc"] and a["mc"]["trials"] == 25
    assert a["rebuilds"] == b["rebuilds"] > 0
    # idle list-build kernels are skipped inside graphs
    assert a["launches"] < b["launches"]


def test_graph_loop_with_measure_stops(built, tmp_path):
    """Stops at measure steps (as the MD driver makes them) between graph runs."""
    m = _bilayer(tmp_path)
    sa = smd.System(m, precision=smd.MIXED)
    sb = smd.System(m, precision=smd.MIXED)
    sb.profile(True)
    for s in (sa, sb):
        s.prepare()
        for _ in range(4):
            s.advance(50, stop_at_measure=True)
            s.energy()
    pa, va = sa.state()
    pb, vb = sb.state()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    assert sa.mc_stats() == sb.mc_stats()


def test_graph_loop_plain_form(built, tmp_path):
    m = _bilayer(tmp_path)
    a = _run(m, graphs=True, steps=40, precision=smd.PLAIN_FP64)
    b = _run(m, graphs=False, steps=40, precision=smd.PLAIN_FP64)
    assert np.abs(a["pos"] - b["pos"]).max() < 1e-9
    assert a["mc"]["trials"] == b["mc"]["trials"] == 4
