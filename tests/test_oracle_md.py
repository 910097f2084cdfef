"""The oracle's MD driver reproduces the reference `MD` run byte for byte.

tests/golden/traj_bil holds a 48-step reference run of a 200-lipid bilayer
with the barostat on, stores every 24 steps and measurements every 8 steps:
the input and the sha256 of every file the run wrote.  The digests were made
on x86-64 (glibc prints the 0/0 bond-length average as "-nan" there).
"""
import hashlib
import json
import os
import platform
import shutil
import subprocess

import pytest
from conftest import GOLDEN

TRAJ = os.path.join(GOLDEN, "traj_bil")
NET = os.path.join(GOLDEN, "net200")
FIELD = os.path.join(GOLDEN, "field200")
CORE = os.path.join(GOLDEN, "core200")
MIX = os.path.join(GOLDEN, "mix200")
RESTART_BIL = os.path.join(GOLDEN, "restart_bil")
RESTART_CORE = os.path.join(GOLDEN, "restart_core")
MSD = os.path.join(GOLDEN, "msd_bil")


@pytest.mark.skipif(platform.machine() != "x86_64", reason="digests are of x86-64 glibc number formatting")
@pytest.mark.parametrize("where,name", [(TRAJ, "bil"), (NET, "net"), (FIELD, "fld"), (CORE, "core"),
                                        (MIX, "mix"), (RESTART_BIL, "bil"), (RESTART_CORE, "core"),
                                        (MSD, "bil")])
def test_md_oracle_matches_reference_outputs(oracle, tmp_path, where, name):
    """traj_bil: CHAIN lipids, barostat on; net200: the same with BOND and
    BEND residues over the heads; field200: with one residue of each
    external-field kind (BOUNDARY, FLOATING_BASE, ZTORQUE, ZPOWERPOTENTIAL,
    BALL); core200: a vesicle with a two-core NANOCORE residue; mix200: a
    two-lipid bilayer (HEAD2/TAIL2, 8-type tables) under a temperature ramp;
    restart_bil / restart_core: continuations from the checkpoints the
    reference stores at t = 0.48 (initialTime != 0, MD.cpp:274-308);
    msd_bil: a run from t = 99.84 across 100 tau, where the reference starts
    tracking diffusion and writes meanSquareDisplacement_bil.dat."""
    from oracle_binding import MD
    shutil.copy(os.path.join(where, name + ".mpd"), tmp_path)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([MD, name, "1"], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    want = json.load(open(os.path.join(where, "digests.json")))
    got = {f: hashlib.sha256(open(os.path.join(tmp_path, f), "rb").read()).hexdigest()
           for f in os.listdir(tmp_path)}
    assert sorted(got) == sorted(want)
    for f in want:
        assert got[f] == want[f], f
    assert "Resize acceptance ratio" in r.stderr


def test_md_oracle_refuses_a_kinetic_energy_beyond_the_histogram(oracle, tmp_path):
    """A bead whose kinetic energy lies beyond the measurement histogram's
    2^26 bins of 1e-4 (a blown-up state) ends the run with a message at the
    t = 0 measurement, as the device measurement does, before a bin index
    is formed from it."""
    from oracle_binding import MD
    txt = open(os.path.join(TRAJ, "bil.mpd")).read()
    head, tail = txt.split("velocities", 1)
    vals = tail.split()
    vals[0] = "200.0"  # 0.5 v^2 = 2e4 per bead: 2e8 bins
    (tmp_path / "bil.mpd").write_text(head + "velocities\n" + " ".join(vals) + "\n")
    r = subprocess.run([MD, "bil", "1"], cwd=tmp_path, env=dict(os.environ, OMP_NUM_THREADS="1"),
                       capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "exceeds the measurement histogram" in r.stdout
