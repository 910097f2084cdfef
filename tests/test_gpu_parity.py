"""CUDA step against the oracle / the reference's golden vectors.

Tolerances (relative to max |F| of the reference forces):
  plain FP64 form: 1e-12, mixed form: 1e-5 (the target of the mixed form).
Cell keys and the set of pairs within rc must match exactly.
"""
import os
import shutil

import numpy as np
import pytest
from conftest import GOLDEN, load_golden, mpd_from_golden

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu

CASES = ["ves300", "bil400"]
PREC = [smd.PLAIN_FP64, smd.MIXED]
FORCE_TOL = {smd.PLAIN_FP64: 1e-12, smd.MIXED: 1e-5}


def system(case, precision, skin=0.5):
    return smd.System(mpd_from_golden(load_golden(case)), precision=precision, skin=skin)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision", PREC)
def test_cell_keys_bit_exact(built, case, precision):
    s = system(case, precision)
    assert np.array_equal(s.cell_keys(), load_golden(case)["keys"])


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision", PREC)
def test_pair_set_matches_reference_traversal(built, case, precision):
    g = load_golden(case)
    got = s_pairs = system(case, precision).pair_list()
    ref = np.sort(g["pairs"], axis=1)
    ref = ref[np.lexsort((ref[:, 1], ref[:, 0]))]
    got = s_pairs[np.lexsort((s_pairs[:, 1], s_pairs[:, 0]))]
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision", PREC)
def test_forces_against_reference(built, case, precision):
    g = load_golden(case)
    s = system(case, precision)
    scale = np.abs(g["force"]).max()
    pf = s.forces(pair_only=True)
    f = s.forces()
    err_pair = np.abs(pf - g["pair_force"]).max() / scale
    err = np.abs(f - g["force"]).max() / scale
    rms = np.sqrt(np.mean((f - g["force"]) ** 2)) / scale
    print(f"{case} prec={precision}: max rel err {err:.3e} (pair {err_pair:.3e}), rms {rms:.3e}")
    assert err_pair <= FORCE_TOL[precision]
    assert err <= FORCE_TOL[precision]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision", PREC)
def test_energies_against_reference(built, case, precision):
    g = load_golden(case)
    e = system(case, precision).energy()[0]
    tol = 1e-12 if precision == smd.PLAIN_FP64 else 2e-6
    assert abs(e["pair"] - g["energy"][0]) <= tol * abs(g["energy"][0])
    assert abs(e["bonded"] - g["energy"][1]) <= tol * abs(g["energy"][1])
    ke = 0.5 * np.sum(g["vel"] ** 2)
    assert abs(e["kinetic"] - ke) <= 1e-12 * ke


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision", PREC)
def test_size_change_difference(built, case, precision):
    """U(x) - U(s x) of the barostat trial (computeDPotential + doChainDPotential)."""
    g = load_golden(case)
    s = system(case, precision)
    for k, sc in enumerate(g["scales"]):
        want = g["energy"][3 + 3 * k] + g["energy"][4 + 3 * k]
        got = s.dU(sc)[0]
        # absolute scale of the terms that cancel: |U| * |s - 1|
        ref_scale = (abs(g["energy"][0]) + abs(g["energy"][1])) * np.abs(sc - 1).max()
        tol = 1e-10 if precision == smd.PLAIN_FP64 else 2e-4
        assert abs(got - want) <= tol * ref_scale, (k, got, want)


def test_plain_trajectory_with_reference_noise(built, oracle, tmp_path):
    """24 steps with the reference's own noise stream (MTRand(seed), one
    thread) against the oracle's run of the same input: positions and
    half-step velocities at the store agree to the .mpd's 15 digits."""
    import subprocess
    from oracle_binding import MD
    src = os.path.join(GOLDEN, "traj_bil", "bil.mpd")
    txt = open(src).read().replace("finalTime 0.96", "finalTime 0.48")
    (tmp_path / "bil.mpd").write_text(txt)
    r = subprocess.run([MD, "bil", "1"], cwd=tmp_path, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert r.returncode == 0, r.stdout
    want = smd.read_mpd(str(tmp_path / "bil.mpd"))
    m = smd.read_mpd(src)
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
    # the store of step 24 precedes that step's box move: trials at 8 and 16
    assert s.mc_stats()["trials"] == 2


@pytest.mark.parametrize("precision", PREC)
def test_runs_are_reproducible(built, precision):
    m = mpd_from_golden(load_golden("bil400"))
    out = []
    for _ in range(2):
        s = smd.System(m, precision=precision)
        s.prepare()
        s.advance(100)
        out.append(s.state())
        s.close()
    if precision == smd.MIXED:  # fixed-point sums: bitwise independent of order
        assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    else:  # FP64 sums follow the list order, which atomics make run-dependent
        assert np.abs(out[0][0] - out[1][0]).max() < 1e-6


@pytest.mark.parametrize("precision", PREC)
def test_md_executable_outputs(built, tmp_path, precision):
    """`MD <name>` on the GPU writes the reference's file set, and the t=0
    measurement line equals the reference's."""
    import json
    import subprocess
    traj = os.path.join(GOLDEN, "traj_bil")
    shutil.copy(os.path.join(traj, "bil.mpd"), tmp_path)
    env = dict(os.environ, SMD_PRECISION="plain" if precision == smd.PLAIN_FP64 else "mixed")
    r = subprocess.run([smd.MD_EXE, "bil"], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    want = set(json.load(open(os.path.join(traj, "digests.json"))))
    assert set(os.listdir(tmp_path)) == want
    for f in ("potential_bil.dat", "kinetic_bil.dat", "size_bil.dat", "temp_bil.dat"):
        first_ref = open(os.path.join(traj, "out", f)).readline()
        first_got = open(tmp_path / f).readline()
        if f == "potential_bil.dat" and precision == smd.MIXED:
            t, v = first_got.split()
            assert abs(float(v) / float(first_ref.split()[1]) - 1) < 1e-5
        else:
            assert first_got == first_ref, f
    assert len(open(tmp_path / "potential_bil.dat").readlines()) == 7
    m = smd.read_mpd(str(tmp_path / "bil.mpd"))
    assert (m.pos >= 0).all() and (m.pos <= m.box + 1e-9).all()
    assert "Resize acceptance ratio" in r.stderr
