"""BOND and BEND residues (explicit pair / triplet lists) on the GPU:
Blob::doBondForce / doBendForce and their potentials and size-change
differences (include/system.h:1880-2040, 2718-2821, 3399-3524).

net400 is a relaxed 400-lipid bilayer whose heads carry two BOND residues
(l0 0.8 k 50, l0 1.1 k 20) and one BEND residue (a 1 k 10) beside the CHAIN
lipids; its forces, energies and differences were dumped from the
reference's own code.  Tolerances relative to max |F| as in the other parity
tests: 1e-12 plain, 1e-5 mixed.
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest
from conftest import GOLDEN, load_golden, mpd_from_golden

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu

PREC = [smd.PLAIN_FP64, smd.MIXED]
FORCE_TOL = {smd.PLAIN_FP64: 1e-12, smd.MIXED: 1e-5}
NET = os.path.join(GOLDEN, "net200")


@pytest.mark.parametrize("precision", PREC)
def test_term_forces_against_reference(built, precision):
    g = load_golden("net400")
    assert len(g["bonds"]) > 100 and len(g["bends"]) > 50
    s = smd.System(mpd_from_golden(g), precision=precision)
    scale = np.abs(g["force"]).max()
    f = s.forces()
    err = np.abs(f - g["force"]).max() / scale
    # the terms matter: the CHAIN-only forces differ from the reference's
    m = mpd_from_golden(g)
    m.bonds = m.bond_consts = m.bends = m.bend_consts = None
    f0 = smd.System(m, precision=precision).forces()
    print(f"precision {precision}: max rel err {err:.3e}; terms change forces by {np.abs(f0 - f).max():.3g}")
    assert err <= FORCE_TOL[precision]
    assert np.abs(f0 - f).max() > 1.0


@pytest.mark.parametrize("precision", PREC)
def test_term_energies_against_reference(built, precision):
    g = load_golden("net400")
    s = smd.System(mpd_from_golden(g), precision=precision)
    e = s.energy()[0]
    tol = 1e-12 if precision == smd.PLAIN_FP64 else 2e-6
    assert abs(e["bonded"] - g["energy"][1]) <= tol * abs(g["energy"][1])
    for k, sc in enumerate(g["scales"]):
        want = g["energy"][3 + 3 * k] + g["energy"][4 + 3 * k]
        got = s.dU(sc)[0]
        ref_scale = (abs(g["energy"][0]) + abs(g["energy"][1])) * np.abs(sc - 1).max()
        assert abs(got - want) <= (1e-10 if precision == smd.PLAIN_FP64 else 2e-4) * ref_scale, (k, got, want)


def test_plain_term_trajectory_with_reference_noise(built, oracle, tmp_path):
    """24 steps (3 barostat trials) with the reference's MT19937 noise against
    the oracle's MD run of the same input."""
    from oracle_binding import MD
    txt = open(os.path.join(NET, "net.mpd")).read().replace("finalTime 0.96", "finalTime 0.48")
    (tmp_path / "net.mpd").write_text(txt)
    m = smd.read_mpd(str(tmp_path / "net.mpd"))
    r = subprocess.run([MD, "net", "1"], cwd=tmp_path, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert r.returncode == 0, r.stdout
    want = smd.read_mpd(str(tmp_path / "net.mpd"))
    n = len(m.type)
    s = smd.System(m, precision=smd.PLAIN_FP64)
    noise = 2.0 * oracle.rand53(m.seed, 3 * n * 25) - 1.0
    s.set_noise_once(noise[:3 * n])
    s.prepare(do_second=False)
    for k in range(1, 25):
        s.set_noise_once(noise[3 * n * k:3 * n * (k + 1)])
        s.advance(1)
    pos, vel = s.state()
    assert np.allclose(s.box(), want.box, rtol=0, atol=1e-12)
    assert np.abs(pos - want.pos).max() < 1e-9
    assert np.abs(vel - want.vel).max() < 1e-8


@pytest.mark.parametrize("precision", PREC)
def test_md_executable_with_terms(built, tmp_path, precision):
    shutil.copy(os.path.join(NET, "net.mpd"), tmp_path)
    env = dict(os.environ, SMD_PRECISION="plain" if precision == smd.PLAIN_FP64 else "mixed")
    r = subprocess.run([smd.MD_EXE, "net"], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert set(os.listdir(tmp_path)) == set(json.load(open(os.path.join(NET, "digests.json"))))


def test_term_graph_loop_matches_kernel_by_kernel(built):
    m = smd.read_mpd(os.path.join(NET, "net.mpd"))
    out = []
    for graphs in (True, False):
        s = smd.System(m, precision=smd.MIXED)
        s.profile(not graphs)
        s.prepare()
        s.advance(120)
        out.append(s.state())
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_terms_batched_as_alone(built):
    """Term indices are per replica: a replica runs the same alone and in a batch."""
    m = smd.read_mpd(os.path.join(NET, "net.mpd"))
    b = smd.read_mpd(os.path.join(GOLDEN, "traj_bil", "bil.mpd"))
    alone = smd.System(m, precision=smd.MIXED)
    both = smd.System([b, m], precision=smd.MIXED)
    for s in (alone, both):
        s.prepare()
        s.advance(40)
    pa = alone.state()[0]
    pb = both.state()[0][len(b.type):]
    assert np.array_equal(pa, pb)


def test_adjoint_rejects_terms(built):
    m = mpd_from_golden(load_golden("net400"))
    m.delta_lxy = 0.0
    s = smd.System(m, precision=smd.MIXED)
    with pytest.raises(smd.SmdError, match="BOND"):
        s.adjoint(10, 5)
