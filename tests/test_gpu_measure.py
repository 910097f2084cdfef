"""Measurement on the device: the .dat series of the `MD` executable and the
reductions behind them (dataExtraction::compute, dataExtraction.h:827-1050,
1456-1650; Kinetic::compute, include/algorithms/dataCollection.h:666-674).

The GPU `MD` reads back only the device's reductions at a measure step
(smd_measure), and from the first measurement after 100 tau it tracks each
bead's displacement on the device for meanSquareDisplacement_ (MD.cpp:64,
538-539).  With the Langevin noise of a one-thread reference run
(SMD_REFERENCE_NOISE=1) the plain form follows the reference's trajectory
to ~1e-9, so every series it writes is compared line by line with the
oracle's run of the same input (the oracle's `MD` reproduces the reference's
runs byte for byte, test_oracle_md.py):
  traj_bil  a 200-lipid bilayer with the barostat, 48 steps;
  net200    the same with BOND and BEND residues (lBond_, bend_);
  msd_bil   a checkpoint at t = 99.84 run across 100 tau
            (meanSquareDisplacement_).
Series are compared to 1e-5 relative (six printed digits, a last-digit flip
allowed); the kinetic-energy histogram bin by bin.
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

RUNS = [("traj_bil", "bil"), ("net200", "net"), ("msd_bil", "bil")]


def _rows(path):
    out = []
    for ln in open(path):
        out.append([float(x) for x in ln.split()])
    return out


def _run_both(tmp_path, where, name, precision="plain", ref_noise=True):
    from oracle_binding import MD
    ref, gpu = tmp_path / "ref", tmp_path / "gpu"
    for d in (ref, gpu):
        d.mkdir()
        shutil.copy(os.path.join(GOLDEN, where, name + ".mpd"), d)
    r = subprocess.run([MD, name, "1"], cwd=ref, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert r.returncode == 0, r.stdout + r.stderr
    env = dict(os.environ, SMD_PRECISION=precision)
    if ref_noise:
        env["SMD_REFERENCE_NOISE"] = "1"
    g = subprocess.run([smd.MD_EXE, name], cwd=gpu, env=env, capture_output=True, text=True)
    assert g.returncode == 0, g.stdout + g.stderr
    return ref, gpu


@pytest.mark.parametrize("where,name", RUNS)
def test_every_series_follows_the_reference(built, tmp_path, where, name):
    ref, gpu = _run_both(tmp_path, where, name)
    want = set(json.load(open(os.path.join(GOLDEN, where, "digests.json"))))
    assert set(os.listdir(gpu)) == want == set(os.listdir(ref))
    series = sorted(f for f in want if f.endswith(".dat") and not f.startswith("kEnergyDensity_"))
    assert {"potential_", "kinetic_", "size_", "lBond_", "bend_", "temp_", "flicker_"} <= \
        {f[:f.index("_") + 1] for f in series}
    for f in series:
        a, b = _rows(ref / f), _rows(gpu / f)
        assert len(a) == len(b), f
        for ra, rb in zip(a, b):
            ra, rb = np.array(ra), np.array(rb)
            assert ra.shape == rb.shape, f
            assert np.array_equal(np.isnan(ra), np.isnan(rb)), f
            ok = ~np.isnan(ra)
            assert np.allclose(rb[ok], ra[ok], rtol=1e-5, atol=1e-9), (f, ra, rb)
    # the run's kinetic-energy histogram, bin by bin (fractions of all beads measured)
    k = next(f for f in want if f.startswith("kEnergyDensity_"))
    ha, hb = np.array(_rows(ref / k)), np.array(_rows(gpu / k))
    n = min(len(ha), len(hb))
    assert abs(len(ha) - len(hb)) <= 1
    one = ha[ha[:, 1] > 0, 1].min()  # at least one bead's share of the total
    assert np.abs(ha[:n, 1] - hb[:n, 1]).sum() <= 6 * one  # at most three beads in a neighbouring bin
    if where == "msd_bil":
        msd = _rows(gpu / "meanSquareDisplacement_bil.dat")
        assert [r[0] for r in msd] == pytest.approx([100.16, 100.32, 100.48, 100.64, 100.8])
        assert msd[0][1] == 0.0 and msd[-1][1] > 0.05


def test_mixed_form_tracks_diffusion(built, tmp_path):
    """The mixed form with its own noise: the reference's file set, MSD from
    the first measurement after 100 tau, growing from zero."""
    _, gpu = _run_both(tmp_path, "msd_bil", "bil", precision="mixed", ref_noise=False)
    assert set(os.listdir(gpu)) == set(json.load(open(os.path.join(GOLDEN, "msd_bil", "digests.json"))))
    msd = _rows(gpu / "meanSquareDisplacement_bil.dat")
    assert len(msd) == 5 and msd[0][1] == 0.0
    assert all(0.0 < r[1] < 5.0 for r in msd[1:])


@pytest.mark.parametrize("precision", [smd.PLAIN_FP64, smd.MIXED])
def test_device_reductions_equal_the_host_formulas(built, precision):
    """smd_measure on a stopped state against the reference's expressions
    evaluated in numpy on the same state (net400: BOND and BEND residues),
    and the histogram of three measurements bin by bin."""
    g = load_golden("net400")
    m = mpd_from_golden(g)
    s = smd.System(m, precision=precision)
    s.prepare()
    bins = {}
    for _ in range(3):
        s.advance(8, stop_at_measure=True)
        pos, vel = s.state()
        box = s.box()
        d = s.measure()
        v2 = vel[:, 0] * vel[:, 0] + vel[:, 1] * vel[:, 1] + vel[:, 2] * vel[:, 2]
        assert d["kinetic"] == pytest.approx(np.sum(v2 / 2.0), rel=1e-13)
        assert np.array_equal(d["lo"], pos.min(axis=0)) and np.array_equal(d["hi"], pos.max(axis=0))

        def wrap(x):
            x = np.where(x >= box / 2.0, x - box, x)
            return np.where(x <= -box / 2.0, x + box, x)
        b = np.asarray(m.bonds)
        da = wrap(pos[b[:, 0]] - pos[b[:, 1]])
        assert d["n_bond"] == len(b)
        assert d["bond_length_sum"] == pytest.approx(np.sqrt((da * da).sum(1)).sum(), rel=1e-13)
        e = np.asarray(m.bends)
        xa, xb = wrap(pos[e[:, 0]] - pos[e[:, 1]]), wrap(pos[e[:, 1]] - pos[e[:, 2]])
        ra, rb = np.sqrt((xa * xa).sum(1)), np.sqrt((xb * xb).sum(1))
        assert d["n_bend"] == len(e)
        assert d["bend_cos_sum"] == pytest.approx(((xa * xb).sum(1) / (ra * rb)).sum(), rel=1e-12, abs=1e-12)
        assert d["bend_len0_sum"] == pytest.approx(ra.sum(), rel=1e-13)
        assert d["bend_len1_sum"] == pytest.approx(rb.sum(), rel=1e-13)
        for q in (0.5 * v2 / 0.0001).astype(np.int64):
            bins[q] = bins.get(q, 0) + 1
    hist = s.ke_histogram()
    assert len(hist) == max(bins) + 1
    want = np.zeros(len(hist), np.int64)
    for q, c in bins.items():
        want[q] = c
    assert np.array_equal(hist, want)
    s.close()


@pytest.mark.parametrize("precision", [smd.PLAIN_FP64, smd.MIXED])
def test_displacement_since_the_start(built, precision):
    """Without box moves the tracked displacement is the unwrapped change of
    position since smd_start_diffusion; each group averages its entries."""
    g = load_golden("bil400")
    m = mpd_from_golden(g)
    m.delta_lxy = 0.0
    s = smd.System(m, precision=precision)
    s.prepare()
    s.advance(8, stop_at_measure=True)
    p0, _ = s.state()
    s.start_diffusion()
    n = len(m.type)
    heads = np.arange(0, n, 3)
    groups = [np.arange(n), heads, np.array([5, 5, 7])]  # a bead listed twice counts twice
    off = np.cumsum([0] + [len(x) for x in groups])
    s.set_msd_groups(off, np.concatenate(groups))
    s.advance(24, stop_at_measure=True)
    p1, _ = s.state()
    box = s.box()
    dx = p1 - p0
    dx -= box * np.rint(dx / box)
    r2 = (dx * dx).sum(1)
    d = s.measure(len(groups))
    assert d["msd"]
    for k, grp in enumerate(groups):
        assert d["msd_sum"][k] == pytest.approx(r2[grp].sum(), rel=1e-9)
    assert r2.mean() > 1e-3
    s.close()
