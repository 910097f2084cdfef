"""The BEAD continuum sphere on the GPU (Blob::doBeadForce / doBeadPotential /
doBeadDPotential, include/system.h:2043-2212, 2936-3074, 3584-3700, and the
sphere mass of MD.cpp:340-355, 480-509).

The fixture sphere300 holds what the reference's own code computes for a
300-lipid vesicle with one sphere of radius 5 whose surface sits 0.8 sigma
outside the heads.  Tolerances relative to max |F| (or |U|): plain FP64 form
1e-12, mixed form 1e-5 for forces.
"""
import os
import re
import subprocess

import numpy as np
import pytest
from conftest import load_golden, mpd_from_golden

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu

PREC = [smd.PLAIN_FP64, smd.MIXED]
FORCE_TOL = {smd.PLAIN_FP64: 1e-12, smd.MIXED: 1e-5}


def _system(precision):
    return smd.System(mpd_from_golden(load_golden("sphere300")), precision=precision)


@pytest.mark.parametrize("precision", PREC)
def test_sphere_forces_against_reference(built, precision):
    g = load_golden("sphere300")
    s = _system(precision)
    scale = np.abs(g["force"]).max()
    f = s.forces()
    pf = s.forces(pair_only=True)
    err = np.abs(f - g["force"]).max() / scale
    err_pair = np.abs(pf - g["pair_force"]).max() / scale
    k = int(g["sphere_index"][0])
    err_sphere = np.abs(f[k] - g["force"][k]).max() / np.abs(g["force"][k]).max()
    print(f"precision {precision}: max rel err {err:.3e}, pair {err_pair:.3e}, sphere bead {err_sphere:.3e}")
    assert err <= FORCE_TOL[precision] and err_pair <= FORCE_TOL[precision]
    assert err_sphere <= 10 * FORCE_TOL[precision]
    # the sphere term is present: total and non-bonded forces differ on the heads near it
    assert np.abs(f - pf).max() > 1.0


@pytest.mark.parametrize("precision", PREC)
def test_sphere_energy_and_size_change(built, precision):
    g = load_golden("sphere300")
    s = _system(precision)
    e = s.energy()[0]
    # FP64 arithmetic in both forms; the mixed form reads positions from the
    # 32-bit fractional mirror (exact to box * 2^-32), as its pair energy does
    tol = 1e-12 if precision == smd.PLAIN_FP64 else 2e-6
    assert abs(e["sphere"] - g["energy"][2]) <= tol * abs(g["energy"][2])
    for k, sc in enumerate(g["scales"]):
        want = g["energy"][3 + 3 * k] + g["energy"][4 + 3 * k] + g["energy"][5 + 3 * k]
        got = s.dU(sc)[0]
        ref_scale = (abs(g["energy"][0]) + abs(g["energy"][1]) + abs(g["energy"][2])) * np.abs(sc - 1).max()
        tol = 1e-10 if precision == smd.PLAIN_FP64 else 2e-4
        assert abs(got - want) <= tol * ref_scale, (k, got, want)


def _sphere_mpd(tmp_path, final):
    p = str(tmp_path / "sph.mpd")
    # head well Umin -10 with Umax 300 and tails Umax 100: the table's inner
    # polynomial is then a barrier that keeps beads out of the singular core
    smd.synth_vesicle_sphere(p, 99, 300, 3.45, 40.0, 5.0, -10.0, 300.0, 0.8, 100.0)
    t = open(p).read()
    for key in ("finalTime", "storeInterval", "measureInterval"):
        t = re.sub(key + r" \S+", f"{key} {final}", t)
    open(p, "w").write(t)
    return p


def test_plain_sphere_trajectory_with_reference_noise(built, oracle, tmp_path):
    """24 steps with the reference's MT19937 noise: the sphere's double mass
    division and its reactions reproduce the oracle's MD run."""
    from oracle_binding import MD
    p = _sphere_mpd(tmp_path, 0.48)
    m = smd.read_mpd(p)
    r = subprocess.run([MD, "sph", "1"], cwd=tmp_path, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert r.returncode == 0, r.stdout
    want = smd.read_mpd(p)
    n = len(m.type)
    s = smd.System(m, precision=smd.PLAIN_FP64)
    noise = 2.0 * oracle.rand53(m.seed, 3 * n * 25) - 1.0
    s.set_noise_once(noise[:3 * n])
    s.prepare(do_second=False)
    for k in range(1, 25):
        s.set_noise_once(noise[3 * n * k:3 * n * (k + 1)])
        s.advance(1)
    pos, vel = s.state()
    k = int(m.sphere_index[0])
    assert np.abs(pos - want.pos).max() < 1e-9
    assert np.abs(vel - want.vel).max() < 1e-8
    assert np.abs(pos[k] - m.pos[k]).max() > 1e-6  # the sphere moved


def test_sphere_graph_loop_matches_kernel_by_kernel(built, tmp_path):
    m = smd.read_mpd(_sphere_mpd(tmp_path, 4.0))
    out = []
    for graphs in (True, False):
        s = smd.System(m, precision=smd.MIXED)
        s.profile(not graphs)
        s.prepare()
        s.advance(101)
        out.append(s.state())
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert np.isfinite(out[0][0]).all()


def test_sphere_mixed_run_stays_close_to_plain(built, tmp_path):
    """20 steps of both forms from the same state and noise key: the mixed
    form's FP32 forces keep the trajectory within a small distance."""
    m = smd.read_mpd(_sphere_mpd(tmp_path, 4.0))
    res = []
    for prec in PREC:
        s = smd.System(m, precision=prec)
        s.prepare()
        s.advance(20)
        res.append(s.state()[0])
    assert np.abs(res[0] - res[1]).max() < 1e-3


def test_batch_rejects_spheres(built):
    m = mpd_from_golden(load_golden("sphere300"))
    with pytest.raises(smd.SmdError, match="single-system"):
        smd.System([m, m], precision=smd.MIXED)


# ---------------------------------------------------------------- BEAD residues of several beads
# spheres6: the brute-force branch (a sphere's force leaves out the residue's
# other spheres); spheres24: the hash-cell branch (it takes them, and the
# sphere-sphere rows attract); spheres21n2: hash cells 2 x 3 x 3, where the
# reference counts partners in the other cell along x twice.  Energies and
# size-change differences take every other bead in all three.
MANY = ["spheres6", "spheres24", "spheres21n2"]


@pytest.mark.parametrize("case", MANY)
@pytest.mark.parametrize("precision", PREC)
def test_many_sphere_forces_against_reference(built, case, precision):
    g = load_golden(case)
    s = smd.System(mpd_from_golden(g), precision=precision)
    f = s.forces()
    scale = np.abs(g["force"]).max()
    err = np.abs(f - g["force"]).max() / scale
    idx = g["sphere_index"]
    err_sph = np.abs(f[idx] - g["force"][idx]).max() / np.abs(g["force"][idx]).max()
    print(f"{case} precision {precision}: max rel err {err:.3e}, spheres {err_sph:.3e}")
    assert err <= FORCE_TOL[precision]
    assert err_sph <= 10 * FORCE_TOL[precision]


@pytest.mark.parametrize("case", MANY)
@pytest.mark.parametrize("precision", PREC)
def test_many_sphere_energy_and_size_change(built, case, precision):
    g = load_golden(case)
    s = smd.System(mpd_from_golden(g), precision=precision)
    e = s.energy()[0]
    tol = 1e-12 if precision == smd.PLAIN_FP64 else 2e-6
    assert abs(e["sphere"] - g["energy"][2]) <= tol * abs(g["energy"][2])
    for k, sc in enumerate(g["scales"]):
        want = g["energy"][3 + 3 * k] + g["energy"][4 + 3 * k] + g["energy"][5 + 3 * k]
        got = s.dU(sc)[0]
        ref_scale = (abs(g["energy"][0]) + abs(g["energy"][1]) + abs(g["energy"][2])) * np.abs(sc - 1).max()
        tol = 1e-10 if precision == smd.PLAIN_FP64 else 2e-4
        assert abs(got - want) <= tol * ref_scale, (k, got, want)


def _many_sphere_mpd(tmp_path, count, final):
    """The spheres24 construction on the stable vesicle of _sphere_mpd (head
    Umax 300, tails 100), radius 1.5, as a run of `final` tau."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import to_many_spheres
    p = str(tmp_path / "sph.mpd")
    smd.synth_vesicle_sphere(p, 99, 300, 3.45, 40.0, 2.5, -10.0, 300.0, 0.8, 100.0)
    to_many_spheres(p, count, 5, None, 3.25)
    t = open(p).read()
    for key in ("finalTime", "storeInterval", "measureInterval"):
        t = re.sub(key + r" \S+", f"{key} {final}", t)
    open(p, "w").write(t)
    return p


@pytest.mark.parametrize("count", [6, 24])
def test_plain_many_sphere_trajectory_with_reference_noise(built, oracle, tmp_path, count):
    """24 steps with the reference's MT19937 noise: the spheres' forces on
    each other as bead partners (or not, below 21 beads) and their
    sphere-sphere terms reproduce the oracle's MD run."""
    from oracle_binding import MD
    p = _many_sphere_mpd(tmp_path, count, 0.48)
    m = smd.read_mpd(p)
    assert len(m.sphere_index) == count
    r = subprocess.run([MD, "sph", "1"], cwd=tmp_path, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert r.returncode == 0, r.stdout
    want = smd.read_mpd(p)
    n = len(m.type)
    s = smd.System(m, precision=smd.PLAIN_FP64)
    noise = 2.0 * oracle.rand53(m.seed, 3 * n * 25) - 1.0
    s.set_noise_once(noise[:3 * n])
    s.prepare(do_second=False)
    for k in range(1, 25):
        s.set_noise_once(noise[3 * n * k:3 * n * (k + 1)])
        s.advance(1)
    pos, vel = s.state()
    assert np.abs(pos - want.pos).max() < 1e-9
    assert np.abs(vel - want.vel).max() < 1e-8


def test_many_sphere_graph_loop_matches_kernel_by_kernel(built, tmp_path):
    m = smd.read_mpd(_many_sphere_mpd(tmp_path, 24, 4.0))
    out = []
    for graphs in (True, False):
        s = smd.System(m, precision=smd.MIXED)
        s.profile(not graphs)
        s.prepare()
        s.advance(101)
        out.append(s.state())
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert np.isfinite(out[0][0]).all()


def test_sphere_limit_and_small_box(built):
    """More than 256 spheres, or a box below one hash cell of the many-sphere
    branch (where the reference divides by zero), are refused."""
    g = load_golden("spheres24")
    m = mpd_from_golden(g)
    m.sphere_index = np.arange(257, dtype=np.int32)
    with pytest.raises(smd.SmdError, match="at most 256"):
        smd.System(m, precision=smd.MIXED)
    m = mpd_from_golden(g)
    m.sphere_consts = m.sphere_consts.copy()
    m.sphere_consts[0] = 25.0  # range 25: one cell needs a box of 50
    with pytest.raises(smd.SmdError, match="hash cell"):
        smd.System(m, precision=smd.MIXED)
