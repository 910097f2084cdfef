"""Statistical parity of trajectories.

The device step draws its Langevin noise from a counter-based generator, the
reference from per-thread MT19937 streams, so trajectories differ sample by
sample.  The GPU `MD` executable (mixed precision) and the oracle's
restatement of the reference `MD` loop run the same 400-lipid bilayer with the
constant-tension barostat on; after equilibration their time averages of
temperature, area per lipid, potential energy per bead, bilayer thickness and
the heads' width of the reference's avgThicknessFrames tool must agree within 4 combined standard errors (block averages) plus a 0.5 %
allowance for the finite run.  A 2,048-lipid bilayer compares the
height-fluctuation spectrum of the reference's structureFactorFrames tool.
"""
import os
import re
import subprocess

import numpy as np
import pytest
from analysis_obs import width_frames

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu

N_LIPIDS = 400
DT = 0.02
EQUIL_TAU = 20.0
TOTAL_TAU = 160.0
MEASURE_TAU = 0.4
STORE_TAU = 2.0


def _prepare(dirpath):
    p = os.path.join(dirpath, "bil.mpd")
    smd.synth_bilayer(p, 2024, N_LIPIDS, 3.45, 20.0, 0.01, 0.0)
    t = open(p).read()
    t = re.sub(r"finalTime \S+", f"finalTime {TOTAL_TAU}", t)
    t = re.sub(r"storeInterval \S+", f"storeInterval {STORE_TAU}", t)
    t = re.sub(r"measureInterval \S+", f"measureInterval {MEASURE_TAU}", t)
    open(p, "w").write(t)


def _series(dirpath, name):
    a = np.loadtxt(os.path.join(dirpath, f"{name}_bil.dat"), ndmin=2)
    keep = a[:, 0] >= EQUIL_TAU
    return a[keep]


def _thickness(dirpath):
    """Mean head-head distance across the bilayer from the stored frames."""
    lines = open(os.path.join(dirpath, "frames_bil.xyz")).read().split("\n")
    n = int(lines[0])
    out = []
    k = 0
    frame = 0
    while k + n + 2 <= len(lines) and lines[k].strip():
        rows = [l.split() for l in lines[k + 2:k + 2 + n]]
        t = frame * STORE_TAU
        if t >= EQUIL_TAU:
            a = np.array(rows, dtype=float)
            heads = a[a[:, 0] == 2]
            mid = a[:, 3].mean()
            up = heads[heads[:, 3] > mid, 3]
            lo = heads[heads[:, 3] <= mid, 3]
            out.append(up.mean() - lo.mean())
        k += n + 2
        frame += 1
    return np.array(out)


def _block_mean(x, blocks=8):
    x = np.asarray(x, float)
    m = len(x) // blocks
    b = x[:m * blocks].reshape(blocks, m).mean(axis=1)
    return b.mean(), b.std(ddof=1) / np.sqrt(blocks)


def test_observables_match_reference_statistics(built, tmp_path):
    from oracle_binding import MD as ORACLE_MD
    gpu, cpu = tmp_path / "gpu", tmp_path / "cpu"
    gpu.mkdir()
    cpu.mkdir()
    _prepare(str(gpu))
    _prepare(str(cpu))
    r1 = subprocess.run([smd.MD_EXE, "bil"], cwd=gpu, capture_output=True, text=True,
                        env=dict(os.environ, SMD_PRECISION="mixed"))
    assert r1.returncode == 0, r1.stdout + r1.stderr
    threads = str(min(16, os.cpu_count() or 1))
    r2 = subprocess.run([ORACLE_MD, "bil", threads], cwd=cpu, capture_output=True, text=True,
                        env=dict(os.environ, OMP_NUM_THREADS=threads))
    assert r2.returncode == 0, r2.stdout + r2.stderr
    n_beads = 3 * N_LIPIDS
    results = {}
    for d, tag in ((gpu, "gpu"), (cpu, "cpu")):
        ke = _series(d, "kinetic")[:, 1]
        size = _series(d, "size")
        pot = _series(d, "potential")[:, 1]
        results[tag] = {
            "temperature": _block_mean(ke / (1.5 * n_beads)),
            "area_per_lipid": _block_mean(size[:, 1] * size[:, 2] / (N_LIPIDS / 2)),
            "potential_per_bead": _block_mean(pot / n_beads),
            "thickness": _block_mean(_thickness(d), blocks=5),
            # avgThicknessFrames bil 20 z 2 2: the heads' width along z in 2-sigma columns
            "head_width": _block_mean(width_frames(os.path.join(d, "frames_bil.xyz"), os.path.join(d, "size_bil.dat"),
                                                   STORE_TAU, EQUIL_TAU, 2, 2.0, [2]), blocks=5),
        }
    for key in results["gpu"]:
        (mg, sg), (mc, sc) = results["gpu"][key], results["cpu"][key]
        allowed = 4.0 * np.hypot(sg, sc) + 0.005 * abs(mc)
        print(f"{key}: gpu {mg:.5f} +- {sg:.5f}  reference {mc:.5f} +- {sc:.5f}")
        assert abs(mg - mc) <= allowed, (key, mg, sg, mc, sc)


SF_LIPIDS = 2048
SF_TOTAL_TAU = 200.0
SF_STORE_TAU = 1.0
SF_GRID = 16


def _prepare_sf(dirpath):
    p = os.path.join(dirpath, "bil.mpd")
    smd.synth_bilayer(p, 2025, SF_LIPIDS, 3.45, 20.0, 0.01, 0.0)
    t = open(p).read()
    t = re.sub(r"finalTime \S+", f"finalTime {SF_TOTAL_TAU}", t)
    t = re.sub(r"storeInterval \S+", f"storeInterval {SF_STORE_TAU}", t)
    t = re.sub(r"measureInterval \S+", f"measureInterval {MEASURE_TAU}", t)
    open(p, "w").write(t)


def test_undulation_spectrum_matches_reference_statistics(built, tmp_path):
    """The height-fluctuation spectrum of analysis/structureFactorFrames.cpp
    (head beads, a 16 x 16 grid, frames from 20 tau) of a 2,048-lipid
    bilayer run for 200 tau with the barostat on: the GPU `MD` executable
    against the oracle's restatement of the reference loop, ring by ring,
    within 4 combined standard errors (5 blocks) plus 5 % for the finite run.
    Two oracle runs with different seeds differ by at most 1.3 combined
    errors on this protocol."""
    from analysis_obs import structure_factor_frames
    from oracle_binding import MD as ORACLE_MD
    gpu, cpu = tmp_path / "gpu", tmp_path / "cpu"
    gpu.mkdir()
    cpu.mkdir()
    _prepare_sf(str(gpu))
    _prepare_sf(str(cpu))
    r1 = subprocess.run([smd.MD_EXE, "bil"], cwd=gpu, capture_output=True, text=True,
                        env=dict(os.environ, SMD_PRECISION="mixed"))
    assert r1.returncode == 0, r1.stdout + r1.stderr
    threads = str(min(16, os.cpu_count() or 1))
    r2 = subprocess.run([ORACLE_MD, "bil", threads], cwd=cpu, capture_output=True, text=True,
                        env=dict(os.environ, OMP_NUM_THREADS=threads))
    assert r2.returncode == 0, r2.stdout + r2.stderr
    spectra = {}
    for d, tag in ((gpu, "gpu"), (cpu, "cpu")):
        q, S = structure_factor_frames(str(d / "frames_bil.xyz"), str(d / "size_bil.dat"), SF_STORE_TAU,
                                       EQUIL_TAU, SF_GRID, SF_GRID, [2])
        assert len(S) >= 150
        spectra[tag] = (q, [_block_mean(S[:, k], blocks=5) for k in range(S.shape[1])])
    qg, sg = spectra["gpu"]
    qc, sc = spectra["cpu"]
    assert np.allclose(qg, qc, rtol=0.02)  # the barostat left boxes of the same size
    for k, ((mg, eg), (mc, ec)) in enumerate(zip(sg, sc)):
        allowed = 4.0 * np.hypot(eg, ec) + 0.05 * abs(mc)
        print(f"q {qc[k]:.3f}: gpu {mg:.5f} +- {eg:.5f}  reference {mc:.5f} +- {ec:.5f}")
        assert abs(mg - mc) <= allowed, (k, mg, eg, mc, ec)
