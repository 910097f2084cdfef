"""Continuation from a checkpoint on the GPU (MD.cpp:274-308).

restart_bil and restart_core hold the .mpd the reference stores at t = 0.48
(x(t+dt), v(t+dt/2), initialTime 0.48) for a 200-lipid bilayer with the
barostat on and for a vesicle with a two-core NANOCORE residue.  A restart
recomputes the forces, runs one second() half-kick (a core's acceleration
divided by its mass once) and enters the loop at step 24; the barostat's
trial steps and random stream continue from there.
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest
from conftest import GOLDEN

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu

CASES = [("restart_bil", "bil"), ("restart_core", "core")]


@pytest.mark.parametrize("where,name", CASES)
def test_plain_continuation_with_reference_noise(built, oracle, tmp_path, where, name):
    """The 24 steps from the checkpoint with the reference's MT19937 noise
    (fresh streams, as a restarted run seeds them) against the oracle's
    continuation: state and box at t = 0.96."""
    from oracle_binding import MD
    shutil.copy(os.path.join(GOLDEN, where, name + ".mpd"), tmp_path)
    m = smd.read_mpd(str(tmp_path / (name + ".mpd")))
    assert m.initial_time == 0.48
    r = subprocess.run([MD, name, "1"], cwd=tmp_path, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert r.returncode == 0, r.stdout
    want = smd.read_mpd(str(tmp_path / (name + ".mpd")))
    assert want.initial_time == 0.96
    n = len(m.type)
    s = smd.System(m, precision=smd.PLAIN_FP64)
    noise = 2.0 * oracle.rand53(m.seed, 3 * n * 25) - 1.0
    s.set_noise_once(noise[:3 * n])
    s.prepare(do_second=True)
    for k in range(1, 25):
        s.set_noise_once(noise[3 * n * k:3 * n * (k + 1)])
        s.advance(1)
    pos, vel = s.state()
    assert np.allclose(s.box(), want.box, rtol=0, atol=1e-12)
    assert np.abs(pos - want.pos).max() < 1e-9
    assert np.abs(vel - want.vel).max() < 1e-8
    assert np.abs(pos - m.pos).max() > 1e-3  # it moved


@pytest.mark.parametrize("where,name", CASES)
@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_md_executable_continues_a_checkpoint(built, tmp_path, where, name, precision):
    """`MD <name>` on the checkpoint writes the reference continuation's file
    set, stores the state at t = 0.96 and measures from t = 0.64 on."""
    shutil.copy(os.path.join(GOLDEN, where, name + ".mpd"), tmp_path)
    r = subprocess.run([smd.MD_EXE, name], cwd=tmp_path, env=dict(os.environ, SMD_PRECISION=precision),
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert set(os.listdir(tmp_path)) == set(json.load(open(os.path.join(GOLDEN, where, "digests.json"))))
    assert smd.read_mpd(str(tmp_path / (name + ".mpd"))).initial_time == 0.96
    times = [float(ln.split()[0]) for ln in open(tmp_path / f"potential_{name}.dat")]
    assert np.allclose(times, [0.64, 0.8, 0.96])
