"""NANOCORE residues on the GPU (Blob::doNanoCoreForce / doNanoCorePotential,
include/system.h:2216-2263, 3029-3073, and the per-core masses of
MD.cpp:280-303, 485-510).

core300 is a 300-lipid vesicle with two cores of the BEAD table's
sphere-head row, 0.8 sigma outside its heads and 3.9 sigma apart: each core
acts on every other bead, the other core included, with its own row, and the
reference's barostat drops the NANOCORE size-change difference.  core200 is
a 48-step reference MD run of a 200-lipid one.  Tolerances relative to max |F|
as in the other parity tests.
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
CORE = os.path.join(GOLDEN, "core200")


@pytest.mark.parametrize("precision", PREC)
def test_core_forces_against_reference(built, precision):
    g = load_golden("core300")
    assert len(g["core_index"]) == 2
    s = smd.System(mpd_from_golden(g), precision=precision)
    scale = np.abs(g["force"]).max()
    f = s.forces()
    err = np.abs(f - g["force"]).max() / scale
    ci = g["core_index"]
    err_core = np.abs(f[ci] - g["force"][ci]).max() / np.abs(g["force"][ci]).max()
    print(f"precision {precision}: max rel err {err:.3e}, cores {err_core:.3e}")
    assert err <= FORCE_TOL[precision]
    assert err_core <= 10 * FORCE_TOL[precision]
    # the cores act on each other (their forces are not the pair forces alone)
    pf = s.forces(pair_only=True)
    assert np.abs(f[ci] - pf[ci]).max() > 1.0


@pytest.mark.parametrize("precision", PREC)
def test_core_energy_and_no_size_change_term(built, precision):
    g = load_golden("core300")
    s = smd.System(mpd_from_golden(g), precision=precision)
    e = s.energy()[0]
    tol = 1e-12 if precision == smd.PLAIN_FP64 else 2e-6
    assert e["sphere"] != 0.0
    assert abs(e["sphere"] - g["energy"][2]) <= tol * abs(g["energy"][2])
    for k, sc in enumerate(g["scales"]):
        # the dump's bead difference is that of the reference's barostat: none
        want = g["energy"][3 + 3 * k] + g["energy"][4 + 3 * k]
        got = s.dU(sc)[0]
        ref_scale = (abs(g["energy"][0]) + abs(g["energy"][1])) * np.abs(sc - 1).max()
        assert abs(got - want) <= (1e-10 if precision == smd.PLAIN_FP64 else 2e-4) * ref_scale, (k, got, want)


def test_plain_core_trajectory_with_reference_noise(built, oracle, tmp_path):
    """24 steps with the reference's MT19937 noise: per-core masses (divided
    once a step, after the forces, unlike a BEAD sphere's, which the reference
    divides again before first()) and the cores' terms on each other reproduce
    the oracle's MD run."""
    from oracle_binding import MD
    txt = open(os.path.join(CORE, "core.mpd")).read().replace("finalTime 0.96", "finalTime 0.48")
    (tmp_path / "core.mpd").write_text(txt)
    m = smd.read_mpd(str(tmp_path / "core.mpd"))
    r = subprocess.run([MD, "core", "1"], cwd=tmp_path, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert r.returncode == 0, r.stdout
    want = smd.read_mpd(str(tmp_path / "core.mpd"))
    n = len(m.type)
    s = smd.System(m, precision=smd.PLAIN_FP64)
    noise = 2.0 * oracle.rand53(m.seed, 3 * n * 25) - 1.0
    s.set_noise_once(noise[:3 * n])
    s.prepare(do_second=False)
    for k in range(1, 25):
        s.set_noise_once(noise[3 * n * k:3 * n * (k + 1)])
        s.advance(1)
    pos, vel = s.state()
    ci = m.core_index
    assert np.abs(pos - want.pos).max() < 1e-9
    assert np.abs(vel - want.vel).max() < 1e-8
    assert np.abs(pos[ci] - m.pos[ci]).max() > 1e-6  # the cores moved


@pytest.mark.parametrize("precision", PREC)
def test_md_executable_with_cores(built, tmp_path, precision):
    """The reference's file set, beadPotential_ included."""
    shutil.copy(os.path.join(CORE, "core.mpd"), tmp_path)
    env = dict(os.environ, SMD_PRECISION="plain" if precision == smd.PLAIN_FP64 else "mixed")
    r = subprocess.run([smd.MD_EXE, "core"], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert set(os.listdir(tmp_path)) == set(json.load(open(os.path.join(CORE, "digests.json"))))


def test_bead_and_core_residues_together_are_refused(built):
    g = load_golden("core300")
    m = mpd_from_golden(g)
    s = load_golden("sphere300")
    m.sphere_index, m.sphere_consts = s["sphere_index"].astype(np.int32), s["sphere_consts"]
    with pytest.raises(smd.SmdError, match="BEAD and a NANOCORE"):
        smd.System(m)


def _many_cores(g, count, range_=None, seed=3):
    """core300 with `count` cores: the two of the fixture and more of the same
    row in the solvent, at least 2 radius + 1 from the others and one range
    from every lipid bead; `range_` replaces every core's constant 0."""
    rng = np.random.default_rng(seed)
    pos, typ, vel = g["pos"].copy(), g["type"].copy(), g["vel"].copy()
    box = g["box"]
    ci = list(g["core_index"])
    rows = np.asarray(g["core_consts"]).reshape(-1, 22).copy()
    rad, c0 = rows[0][4], rows[0][0]
    lip = np.delete(pos, ci, axis=0)

    def mind(p, q):
        d = q - p
        d -= box * np.round(d / box)
        return np.sqrt((d * d).sum(-1))

    cores = [pos[k] for k in ci]
    while len(cores) < count:
        p = rng.uniform(0, box)
        if mind(p, lip).min() > c0 + 0.5 and mind(p, np.array(cores)).min() > 2 * rad + 1:
            cores.append(p)
    extra = np.array(cores[len(ci):])
    n = len(typ)
    pos = np.concatenate([pos, extra])
    typ = np.concatenate([typ, np.full(len(extra), typ[ci[0]], typ.dtype)])
    vel = np.concatenate([vel, np.zeros_like(extra)])
    rows = np.concatenate([rows, np.repeat(rows[:1], len(extra), 0)])
    if range_ is not None:
        rows[:, 0] = range_
    h = dict(g)
    h.update(pos=pos, type=typ, vel=vel, core_index=np.array(ci + list(range(n, n + len(extra))), np.int32),
             core_consts=rows)
    return h


@pytest.mark.parametrize("range_", [None, 7.5])
@pytest.mark.parametrize("precision", PREC)
def test_many_cores_against_oracle(built, oracle, precision, range_):
    """50 cores take the reference's hash-cell branch (include/system.h:
    2264-2318): with the fixture's range 4 the cells are 8 wide (5 per axis)
    and every partner counts once; with range 7.5 the int-truncated range 7
    gives cells 14 wide, 2 per axis, and partners in the other cell along an
    axis count twice (four or eight times across two or three axes)."""
    h = _many_cores(load_golden("core300"), 50, range_)
    want = oracle.forces(h)
    s = smd.System(mpd_from_golden(h), precision=precision)
    f = s.forces()
    err = np.abs(f - want).max() / np.abs(want).max()
    print(f"range {range_} precision {precision}: max rel err {err:.3e}")
    assert err <= FORCE_TOL[precision]
    if range_ is not None:
        # the repeated cells matter: 49 cores (brute force) give other forces
        h49 = dict(h)
        h49["core_index"] = h["core_index"][:49]
        h49["core_consts"] = h["core_consts"][:49]
        assert np.abs(oracle.forces(h49)[h["core_index"][:49]] - want[h["core_index"][:49]]).max() > 1e-6
