"""Two-lipid membranes on the GPU: 8 bead types, HEAD2/TAIL2 lipids
(generate/include.h:34-35, models/lipidModels.h:2070-2125) over the 8-type
tables of generate/continuumSphereAndBilayer.cpp:95-131, and the thermostat
given per type.

mix400 is a relaxed 400-lipid bilayer with 40 % of its lipids retyped
HEAD2/TAIL2; its forces and energies were dumped from the reference's own
code.  mix200 is a 48-step reference MD run of a 200-lipid one under a
temperature ramp.  Tolerances relative to max |F| as in the other parity tests.
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
MIX = os.path.join(GOLDEN, "mix200")


@pytest.mark.parametrize("precision", PREC)
def test_two_lipid_forces_against_reference(built, precision):
    g = load_golden("mix400")
    assert int(g["n_types"]) == 8 and set(np.unique(g["type"])) == {2, 3, 6, 7}
    s = smd.System(mpd_from_golden(g), precision=precision)
    scale = np.abs(g["force"]).max()
    err = np.abs(s.forces() - g["force"]).max() / scale
    perr = np.abs(s.forces(pair_only=True) - g["pair_force"]).max() / scale
    print(f"precision {precision}: max rel err {err:.3e}, pair {perr:.3e}")
    assert err <= FORCE_TOL[precision] and perr <= FORCE_TOL[precision]


@pytest.mark.parametrize("precision", PREC)
def test_two_lipid_energies_against_reference(built, precision):
    g = load_golden("mix400")
    s = smd.System(mpd_from_golden(g), precision=precision)
    e = s.energy()[0]
    tol = 1e-12 if precision == smd.PLAIN_FP64 else 2e-6
    assert abs(e["pair"] - g["energy"][0]) <= tol * abs(g["energy"][0])
    assert abs(e["bonded"] - g["energy"][1]) <= tol * abs(g["energy"][1])
    for k, sc in enumerate(g["scales"]):
        want = g["energy"][3 + 3 * k] + g["energy"][4 + 3 * k]
        got = s.dU(sc)[0]
        ref_scale = (abs(g["energy"][0]) + abs(g["energy"][1])) * np.abs(sc - 1).max()
        assert abs(got - want) <= (1e-10 if precision == smd.PLAIN_FP64 else 2e-4) * ref_scale, (k, got, want)


def test_plain_two_lipid_trajectory_with_reference_noise(built, oracle, tmp_path):
    """24 steps (3 barostat trials) with the reference's MT19937 noise against
    the oracle's MD run of the same input (the ramp taken out: the device
    call runs at one temperature)."""
    from oracle_binding import MD
    txt = open(os.path.join(MIX, "mix.mpd")).read()
    txt = txt.replace("finalTime 0.96", "finalTime 0.48").replace("finalTemp 3.3", "finalTemp 3")
    txt = txt.replace("tempStepInterval 0.16", "")
    (tmp_path / "mix.mpd").write_text(txt)
    m = smd.read_mpd(str(tmp_path / "mix.mpd"))
    r = subprocess.run([MD, "mix", "1"], cwd=tmp_path, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert r.returncode == 0, r.stdout
    want = smd.read_mpd(str(tmp_path / "mix.mpd"))
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
def test_md_executable_two_lipids_with_ramp(built, tmp_path, precision):
    """The reference's file set; the potential at t = 0 (before any step)
    and the ramp's temperatures in temp_ equal the reference's."""
    shutil.copy(os.path.join(MIX, "mix.mpd"), tmp_path)
    env = dict(os.environ, SMD_PRECISION="plain" if precision == smd.PLAIN_FP64 else "mixed")
    r = subprocess.run([smd.MD_EXE, "mix"], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert set(os.listdir(tmp_path)) == set(json.load(open(os.path.join(MIX, "digests.json"))))
    first = open(tmp_path / "potential_mix.dat").readline().split()
    assert first[0] == "0" and abs(float(first[1]) - (-16348.5)) < 0.1
    temps = [ln.split() for ln in open(tmp_path / "temp_mix.dat")]
    assert temps[:3] == [["0", "3"], ["0.16", "3.1"], ["0.32", "3.15"]]


def test_per_type_gamma_applies_entry_zero(built, tmp_path):
    """A `gammaType` line stands in for `gamma` with its first entry for every
    bead (include/algorithms/langevin.h:257 reads type 0): the same seed gives
    the same run as `gamma` = that entry.  (The reference's own reader cannot
    take the line: include/system.h:1266-1269 stores into an unsized vector.)"""
    base = open(os.path.join(MIX, "mix.mpd")).read()
    base = base.replace("finalTemp 3.3", "finalTemp 3").replace("tempStepInterval 0.16", "")
    runs = {}
    for tag, txt in (("g", base.replace("gamma 1 ", "gamma 0.8 ")),
                     ("t", base.replace("gamma 1 \n", "") + "gammaType 0.8 1 1 1 1 1 2 2 \n")):
        d = tmp_path / tag
        d.mkdir()
        (d / "mix.mpd").write_text(txt)
        r = subprocess.run([smd.MD_EXE, "mix"], cwd=d, env=dict(os.environ, SMD_PRECISION="plain"),
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        runs[tag] = d
    assert "gammaType 0.8 1 1 1 1 1 2 2" in " ".join(open(runs["t"] / "mix.mpd").read().split())
    for f in ("potential_mix.dat", "kinetic_mix.dat", "frames_mix.xyz", "size_mix.dat"):
        assert (runs["g"] / f).read_bytes() == (runs["t"] / f).read_bytes(), f
