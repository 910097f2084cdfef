"""External-field residues on the GPU: BOUNDARY, FLOATING_BASE, ZTORQUE,
ZPOWERPOTENTIAL and BALL (Blob::doBoundaryForce, doFloatingBaseForce,
doZTorqueForce, doZPowerForce, doBallForce and their potentials,
include/system.h:1937-1971, 2335-2447, 2583-2779, 3138-3151; the formulas in
include/MD.h:458-617, 1116-1222).

field400 is a relaxed 400-lipid bilayer carrying one residue of each kind:
a wall above the top heads, a z well on the bottom heads, a torque on every
chain's first bond below the midplane, a z power law on 300 beads and a
soft ball around one head.  Its
forces and energies were dumped from the reference's own code; field200 is
a 48-step reference MD run with the same residues.  The reference's
barostat adds no size-change term for these residues, so dU is that of the
pair and CHAIN terms alone.
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
FIELD = os.path.join(GOLDEN, "field200")


@pytest.mark.parametrize("precision", PREC)
def test_field_forces_against_reference(built, precision):
    g = load_golden("field400")
    kinds, counts = np.unique(g["fields"][:, 0], return_counts=True)
    assert list(kinds) == [11, 15, 16, 17, 19] and counts[:4].min() > 100 and counts[4] > 20
    s = smd.System(mpd_from_golden(g), precision=precision)
    scale = np.abs(g["force"]).max()
    f = s.forces()
    err = np.abs(f - g["force"]).max() / scale
    # the fields matter: the forces without them differ from the reference's
    m = mpd_from_golden(g)
    m.fields = m.field_consts = None
    f0 = smd.System(m, precision=precision).forces()
    print(f"precision {precision}: max rel err {err:.3e}; fields change forces by {np.abs(f0 - f).max():.3g}")
    assert err <= FORCE_TOL[precision]
    assert np.abs(f0 - f).max() > 1.0


@pytest.mark.parametrize("precision", PREC)
def test_field_energies_against_reference(built, precision):
    g = load_golden("field400")
    s = smd.System(mpd_from_golden(g), precision=precision)
    e = s.energy()[0]
    tol = 1e-12 if precision == smd.PLAIN_FP64 else 2e-6
    assert abs(e["bonded"] - g["energy"][1]) <= tol * abs(g["energy"][1])
    for k, sc in enumerate(g["scales"]):
        want = g["energy"][3 + 3 * k] + g["energy"][4 + 3 * k]
        got = s.dU(sc)[0]
        ref_scale = (abs(g["energy"][0]) + abs(g["energy"][1])) * np.abs(sc - 1).max()
        assert abs(got - want) <= (1e-10 if precision == smd.PLAIN_FP64 else 2e-4) * ref_scale, (k, got, want)


def test_plain_field_trajectory_with_reference_noise(built, oracle, tmp_path):
    """24 steps (3 barostat trials) with the reference's MT19937 noise against
    the oracle's MD run of the same input."""
    from oracle_binding import MD
    txt = open(os.path.join(FIELD, "fld.mpd")).read().replace("finalTime 0.96", "finalTime 0.48")
    (tmp_path / "fld.mpd").write_text(txt)
    m = smd.read_mpd(str(tmp_path / "fld.mpd"))
    r = subprocess.run([MD, "fld", "1"], cwd=tmp_path, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert r.returncode == 0, r.stdout
    want = smd.read_mpd(str(tmp_path / "fld.mpd"))
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
def test_md_executable_with_fields(built, tmp_path, precision):
    """The MD driver runs the residues and writes the reference's file set;
    its potential at t = 0 (before any step) equals the reference's."""
    shutil.copy(os.path.join(FIELD, "fld.mpd"), tmp_path)
    env = dict(os.environ, SMD_PRECISION="plain" if precision == smd.PLAIN_FP64 else "mixed")
    r = subprocess.run([smd.MD_EXE, "fld"], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert set(os.listdir(tmp_path)) == set(json.load(open(os.path.join(FIELD, "digests.json"))))
    first = open(tmp_path / "potential_fld.dat").readline().split()
    assert first[0] == "0" and abs(float(first[1]) - (-13109.1)) < 0.1


def test_fields_batched_as_alone(built):
    """Field-term indices are per replica: a replica runs the same alone and in a batch."""
    m = smd.read_mpd(os.path.join(FIELD, "fld.mpd"))
    b = smd.read_mpd(os.path.join(GOLDEN, "traj_bil", "bil.mpd"))
    alone = smd.System(m, precision=smd.MIXED)
    both = smd.System([b, m], precision=smd.MIXED)
    for s in (alone, both):
        s.prepare()
        s.advance(40)
    pa = alone.state()[0]
    pb = both.state()[0][len(b.type):]
    assert np.array_equal(pa, pb)
