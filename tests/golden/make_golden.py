"""Generates the golden fixtures in this directory from the reference's own code.

Run where the reference sources are present (it needs oracle/_ref, built by
oracle/build_ref.sh):  python tests/golden/make_golden.py

Fixtures
  <case>.npz       state of a system relaxed by the reference MD (ves300,
                   bil400, net400 = bil400 plus BOND and BEND residues over the
                   heads, sphere300 at its start), plus what the
                   reference's CellOpt / Blob code computes on it (ref_dump):
                   cell keys, visited pair list, pair and total forces, pair /
                   bonded / BEAD energies and their size-change differences for
                   the scales in `scales`, and 4096 MTRand(seed).rand53() draws.
  traj_bil/        a 48-step reference MD run on a 200-lipid bilayer with the
                   barostat on: input .mpd, sha256 of every file the run writes
                   (digests.json) and the small ones verbatim (out/).
  net200/          a 200-lipid bilayer with BOND and BEND residues (input of
                   the network trajectory and MD tests) and the sha256 of
                   every file a 48-step reference MD run of it writes.
  field400.npz     a relaxed 400-lipid bilayer with one residue of each
                   external-field kind (BOUNDARY, FLOATING_BASE, ZTORQUE,
                   ZPOWERPOTENTIAL), dumped as the cases above.
  field200/        a 200-lipid bilayer with the same residues and the sha256
                   of every file a 48-step reference MD run of it writes.
                   (`--only-fields` regenerates these two alone.)
  core300.npz      a 300-lipid vesicle with a NANOCORE residue of two cores;
  core200/         its 48-step reference MD run (`--only-nanocore`).
  mix400.npz       a relaxed 400-lipid bilayer with 40 % of its lipids
                   retyped HEAD2/TAIL2 over 8-type tables;
  mix200/          a 200-lipid two-lipid bilayer's 48-step reference MD run
                   with a temperature ramp (`--only-mixed`).
  restart_bil/,    the checkpoint a reference run of traj_bil / core200
  restart_core/    stores at t = 0.48, extended to 0.96, and the sha256 of
                   every file the reference's continuation writes
                   (`--only-restart`; made after traj_bil and core200).
  msd_bil/         the traj_bil bilayer entered as a checkpoint at t = 99.84
                   and run to 100.8 (stores every 0.48, measurements every
                   0.16): the reference starts diffusion tracking at its first
                   measurement after 100 tau (MD.cpp:64, 538-539) and writes
                   meanSquareDisplacement_bil.dat; sha256 of every file and the
                   small ones verbatim (`--only-msd`).
  spheres6.npz,    300-lipid vesicles with BEAD residues of 6, 24 and 21
  spheres24.npz,   spheres (both force branches of Blob::doBeadForce, and
  spheres21n2.npz  hash cells of two along x), dumped as the cases above
                   (`--only-spheres`).
  generators.json  sha256 of the reference generators' .mpd for a few seeds.
Inputs are seeded synthetic membranes built in the reference generators' terms
(softmold_gb300 synth_*, byte-identical to generate/liposome and bilayer).
"""
from __future__ import annotations

import glob
import hashlib
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import softmold_gb300 as smd  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
SCALES = np.array([[1.0001, 1.0001, 0.9998000099990001], [0.9995, 0.9995, 1.0010007505629221],
                   [1.01, 0.99, 1.0]])


def set_run(path, final, store, measure):
    t = open(path).read()
    t = re.sub(r"finalTime \S+", f"finalTime {final}", t)
    t = re.sub(r"storeInterval \S+", f"storeInterval {store}", t)
    t = re.sub(r"measureInterval \S+", f"measureInterval {measure}", t)
    open(path, "w").write(t)


def add_network(path, seed):
    """Adds BOND and BEND residues over the head beads of a bilayer .mpd: two
    BOND residues (nearest-neighbour heads, l0 0.8 k 50; next-nearest, l0 1.1
    k 20) and one BEND residue (collinear head triplets, a 1 k 10), as the
    molecule blocks `6 nBond / l0 k / i j ...` and `7 nBond / a k / i j l ...`."""
    m = smd.read_mpd(path)
    rng = np.random.default_rng(seed)
    heads = np.flatnonzero(m.type == 2)
    P = m.pos[heads]
    d = P[:, None, :] - P[None, :, :]
    d -= m.box * np.round(d / m.box)
    r = np.sqrt((d ** 2).sum(-1))
    near, nnear = [], []
    for a in range(len(heads)):
        for b in range(a + 1, len(heads)):
            if abs(d[a, b, 2]) > 1.0:  # other leaflet
                continue
            if r[a, b] < 0.9:
                near.append((heads[a], heads[b]))
            elif r[a, b] < 1.2:
                nnear.append((heads[a], heads[b]))
    near = [near[k] for k in rng.permutation(len(near))[:max(1, len(near) // 3)]]
    nnear = [nnear[k] for k in rng.permutation(len(nnear))[:max(1, len(nnear) // 4)]]
    trip = []
    for a in range(len(heads)):
        for b in range(len(heads)):
            if b == a or not (0.5 < r[a, b] < 0.9) or abs(d[a, b, 2]) > 1.0:
                continue
            for c in range(len(heads)):
                if c in (a, b) or not (0.5 < r[b, c] < 0.9):
                    continue
                if np.dot(d[a, b], d[b, c]) / (r[a, b] * r[b, c]) > 0.95 and a < c:
                    trip.append((heads[a], heads[b], heads[c]))
    trip = [trip[k] for k in rng.permutation(len(trip))[:max(1, len(trip) // 6)]]
    blocks = ["6\t%d\n0.8 50\n" % len(near) + "".join(f"{a} {b}\n" for a, b in near),
              "6\t%d\n1.1 20\n" % len(nnear) + "".join(f"{a} {b}\n" for a, b in nnear),
              "7\t%d\n1 10\n" % len(trip) + "".join(f"{a} {b} {c}\n" for a, b, c in trip)]
    lines = open(path).read().split("\n")
    k = next(i for i, ln in enumerate(lines) if ln.strip() == "molecule")
    lines = lines[:k + 4] + "".join(blocks).rstrip("\n").split("\n") + lines[k + 4:]
    text = "\n".join(lines)
    text = re.sub(r"nMolecules (\d+)", lambda mm: f"nMolecules {int(mm.group(1)) + 3}", text)
    open(path, "w").write(text)
    return len(near), len(nnear), len(trip)


def add_fields(path, seed):
    """Adds one residue of each external-field kind after the CHAIN block of a
    bilayer .mpd (molecule blocks `type nBond / constants / indices`):
      BOUNDARY 11         a wall normal to z 0.6 sigma above the top heads, k 0.5,
                          on every top-leaflet head;
      FLOATING_BASE 15    a z well on the bottom-leaflet heads (6 constants per
                          type; type 0 carries a nonzero first constant, which
                          the reference's potential subtracts from z);
      ZTORQUE 16          over every lipid chain, cut off at the midplane;
      ZPOWERPOTENTIAL 17  on the first 300 beads;
      BALL 19             a soft ball of radius 1.5 around one top head, bonded
                          to the beads within 2 sigma of it.
    """
    m = smd.read_mpd(path)
    z = m.pos[:, 2]
    zc = float(np.median(z))
    heads = np.flatnonzero(m.type == 2)
    top = heads[z[heads] > zc]
    bottom = heads[z[heads] <= zc]
    wall = float(z[top].max()) + 0.6
    fb = np.zeros((m.n_types, 6))
    fb[0] = [1.0, 2.0, 0.1, 0.01, 0.0, 0.01]
    fb[2] = [zc - 2.0, zc + 1.0, 0.5, 0.05, 0.0, 0.02]
    n = len(m.type)
    # BALL: a soft exclusion ball of radius 1.5 around one top head, tethered
    # to the beads within 2 sigma of it
    centre = int(top[0])
    dc = m.pos - m.pos[centre]
    dc -= m.box * np.round(dc / m.box)
    rc_ = np.sqrt((dc ** 2).sum(1))
    ball = [int(k) for k in np.flatnonzero((rc_ < 2.0) & (np.arange(n) != centre))]
    blocks = ["11\t%d\n2 %.17g 0 0.5\n" % (len(top), wall) + "".join(f"{b}\n" for b in top),
              "15\t%d\n" % len(bottom) + " ".join(f"{x:.17g}" for x in fb.ravel()) + "\n" +
              "".join(f"{b}\n" for b in bottom),
              "16\t1\n2 1 1 %.17g\n0 %d 3\n" % (zc, n // 3),
              "17\t1\n-0.01 2.1\n0 300\n",
              "19\t%d\n1.5 20\n" % len(ball) + "".join(f"{centre} {b}\n" for b in ball)]
    lines = open(path).read().split("\n")
    k = next(i for i, ln in enumerate(lines) if ln.strip() == "molecule")
    lines = lines[:k + 4] + "".join(blocks).rstrip("\n").split("\n") + lines[k + 4:]
    text = "\n".join(lines)
    text = re.sub(r"nMolecules (\d+)", lambda mm: f"nMolecules {int(mm.group(1)) + 5}", text)
    open(path, "w").write(text)
    return len(top), len(bottom)


def mixed_tables(rc=2.0, rm=1.0):
    """The 8-type two-body tables of a two-lipid membrane in the terms of
    generate/continuumSphereAndBilayer.cpp:95-131 (HEAD 2, TAIL 3, HEAD2 6,
    TAIL2 7): every pair Umin 0 / Umax 100 except the tail pairs and the
    HEAD-HEAD2 pair (Umax 200).  TAIL-TAIL2 takes -5.5, the value
    generate/bilayer.cpp:76-80 carries, so the cross pair differs from the
    like pairs.  Formulas of mpd::laradjiRevaleeFC / PC."""
    nT = 8
    umax = np.full(nT * nT, 100.0)
    umin = np.zeros(nT * nT)
    for a, b, lo in ((3, 3, -6.0), (7, 7, -6.0), (7, 3, -5.5), (3, 7, -5.5), (6, 2, -6.0), (2, 6, -6.0)):
        umin[a + b * nT], umax[a + b * nT] = lo, 200.0
    fc, pc = [], []
    for i in range(nT):
        for j in range(nT):
            g = i + j * nT
            fc += [rm, 2.0 * (umax[g] - umin[g]) / (rm * rm), 0.0, rc,
                   6.0 * umin[g] / ((rc - rm) ** 2), 6.0 * umin[g] / ((rc - rm) ** 3)]
            pc += [rm, (umax[g] - umin[g]) / (rm * rm), umin[g], rc,
                   3.0 * umin[g] / ((rc - rm) ** 2), 2.0 * umin[g] / ((rc - rm) ** 3)]
    return np.array(fc), np.array(pc)


def to_mixed(path, seed, frac=0.4, ramp=None):
    """Turns a 6-type bilayer .mpd into a two-lipid one: nTypes 8 with
    mixed_tables(), a seeded `frac` of the lipids (three-bead CHAIN members)
    retyped HEAD2/TAIL2.  `ramp` (final temperature, step interval) adds a
    temperature ramp.  The thermostat stays `gamma`: the reference's reader
    stores a `gammaType` line into a vector it has not sized
    (include/system.h:1266-1269, sized only by setGammaType, :4519-4525) and
    crashes on it."""
    m = smd.read_mpd(path)
    rng = np.random.default_rng(seed)
    n_lip = len(m.type) // 3
    pick = np.zeros(len(m.type), bool)
    for lip in rng.permutation(n_lip)[:int(frac * n_lip)]:
        pick[3 * lip:3 * lip + 3] = True
    fc, pc = mixed_tables()
    row = lambda v: "".join(" " + " ".join("%.15g" % x for x in v[k:k + 6]) + "\n"  # noqa: E731
                            for k in range(0, len(v), 6))
    lines = open(path).read().split("\n")
    out, i = [], 0
    while i < len(lines):
        ln = lines[i]
        key = ln.split()[0] if ln.split() else ""
        if key == "nTypes":
            out.append("nTypes 8 ")
        elif key == "finalTemp" and ramp is not None:
            out.append("finalTemp %.15g " % ramp[0])
        elif key in ("twoBodyFconst", "twoBodyUconst"):
            out.append(ln)
            out.extend(row(fc if key == "twoBodyFconst" else pc).rstrip("\n").split("\n"))
            i += 1
            while lines[i].strip():
                i += 1
            continue
        elif key == "positions":
            out.append(ln)
            for b in range(len(m.type)):
                i += 1
                tok = lines[i].split()
                t = int(tok[0])
                if pick[b]:
                    t = {2: 6, 3: 7}[t]
                out.append(" %d %s" % (t, " ".join(tok[1:])))
        else:
            out.append(ln)
        i += 1
    text = "\n".join(out).rstrip("\n") + "\n"
    if ramp is not None:
        text += "tempStepInterval %.15g \n" % ramp[1]
    open(path, "w").write(text)
    return int(pick.sum()) // 3


def make_mixed(tmp):
    """mix400 (a relaxed 400-lipid bilayer, 40 % of its lipids retyped
    HEAD2/TAIL2 over 8-type tables) and mix200/ (a 48-step
    reference MD run of a 200-lipid one with a temperature ramp)."""
    smd.synth_bilayer(os.path.join(tmp, "mix.mpd"), 95, 400, 3.45, 20.0, 0.01, 0.0)
    set_run(os.path.join(tmp, "mix.mpd"), 4, 4, 4)
    run_ref_md(tmp, "mix")
    to_mixed(os.path.join(tmp, "mix.mpd"), 95)
    dump_case(tmp, "mix", "mix400")
    mdir = os.path.join(HERE, "mix200")
    os.makedirs(mdir, exist_ok=True)
    smd.synth_bilayer(os.path.join(mdir, "mix.mpd"), 10, 200, 3.45, 16.0, 0.01, 0.0)
    set_run(os.path.join(mdir, "mix.mpd"), 0.96, 0.48, 0.16)
    to_mixed(os.path.join(mdir, "mix.mpd"), 10, ramp=(3.3, 0.16))
    run_dir = os.path.join(tmp, "mixrun")
    os.makedirs(run_dir)
    shutil.copy(os.path.join(mdir, "mix.mpd"), run_dir)
    run_ref_md(run_dir, "mix")
    json.dump({os.path.basename(f): hashlib.sha256(open(f, "rb").read()).hexdigest()
               for f in sorted(glob.glob(os.path.join(run_dir, "*")))},
              open(os.path.join(mdir, "digests.json"), "w"), indent=1)


def make_restart(tmp):
    """restart_bil/ and restart_core/: the checkpoint a reference MD run of
    traj_bil / core200 stores at t = 0.48 (x(t+dt), v(t+dt/2), initialTime
    0.48), extended to finalTime 0.96, and the sha256 of every file the
    reference's continuation from it writes (MD.cpp:274-308 restart)."""
    for src, name in ((os.path.join(HERE, "traj_bil", "bil.mpd"), "bil"),
                      (os.path.join(HERE, "core200", "core.mpd"), "core")):
        first = os.path.join(tmp, "first_" + name)
        os.makedirs(first)
        shutil.copy(src, first)
        set_run(os.path.join(first, name + ".mpd"), 0.48, 0.48, 0.16)
        run_ref_md(first, name)
        rdir = os.path.join(HERE, "restart_" + name)
        os.makedirs(rdir, exist_ok=True)
        shutil.copy(os.path.join(first, name + ".mpd"), rdir)
        set_run(os.path.join(rdir, name + ".mpd"), 0.96, 0.48, 0.16)
        run_dir = os.path.join(tmp, "cont_" + name)
        os.makedirs(run_dir)
        shutil.copy(os.path.join(rdir, name + ".mpd"), run_dir)
        run_ref_md(run_dir, name)
        json.dump({os.path.basename(f): hashlib.sha256(open(f, "rb").read()).hexdigest()
                   for f in sorted(glob.glob(os.path.join(run_dir, "*")))},
                  open(os.path.join(rdir, "digests.json"), "w"), indent=1)


def to_nanocore(path, sep):
    """Turns the BEAD residue of a vesicle-and-sphere .mpd into a NANOCORE
    residue of two cores (molecule block `18 nBond / 22 constants per core /
    indices`): the sphere bead and a new bead of its type `sep` sigma from it,
    tangent to the vesicle, both with the sphere-head row of the BEAD table
    (the row applies to every partner type)."""
    m = smd.read_mpd(path)
    s0 = int(m.sphere_index[0])
    ts, nT = int(m.type[s0]), m.n_types
    row = m.sphere_consts[22 * (ts * nT + 2):22 * (ts * nT + 2) + 22]
    centre = m.pos[np.arange(len(m.type)) != s0].mean(0)
    r = m.pos[s0] - centre
    t = np.cross(r, [0.0, 0.0, 1.0]) if abs(r[2]) < 0.9 * np.linalg.norm(r) else np.cross(r, [1.0, 0.0, 0.0])
    p2 = m.pos[s0] + sep * t / np.linalg.norm(t)
    n = len(m.type)
    tok = open(path).read().split("\n")
    out, i = [], 0
    while i < len(tok):
        ln = tok[i]
        key = ln.strip()
        if key.startswith("nParticles"):
            out.append(f"nParticles {n + 1} ")
        elif key == "positions":
            out.extend(tok[i:i + 1 + n])
            out.append(" %d %.15g %.15g %.15g" % (ts, *p2))
            i += n + 1
            continue
        elif key == "velocities":
            out.extend(tok[i:i + 1 + n])
            out.append(" 0 0 0")
            i += n + 1
            continue
        elif key.split() == ["9", "1"] or key.startswith("9\t"):
            # the BEAD block: header, its 22 nT^2 constants and one index
            out.append("18\t2")
            out.append(" " + " ".join("%.17g" % x for x in np.concatenate([row, row])))
            out.append(f" {s0}")
            out.append(f" {n}")
            vals = 0
            i += 1
            while vals < 22 * nT * nT + 1:
                vals += len(tok[i].split())
                i += 1
            continue
        else:
            out.append(ln)
        i += 1
    open(path, "w").write("\n".join(out))


def to_many_spheres(path, count, seed, size=None, pair_gap=None):
    """Adds spheres to the BEAD residue of a vesicle-and-sphere .mpd until it
    holds `count` beads of the sphere's type: the generator's sphere, then
    spheres at its distance from the vesicle's centre in other directions
    (tangent to the vesicle like it), then (with `pair_gap`) two pairs in the
    solvent `pair_gap` apart, then solvent spheres at least one range from
    every lipid bead.  Spheres keep 2 radius + 1 between centres, except the
    pairs.  `size` replaces the box first (beads stay put)."""
    m = smd.read_mpd(path)
    s0 = int(m.sphere_index[0])
    ts, nT = int(m.type[s0]), m.n_types
    rad, rng_c0 = float(m.sphere_consts[4]), float(m.sphere_consts[0])
    box = np.array(size if size is not None else m.box, dtype=float)
    lip = m.pos[np.arange(len(m.type)) != s0]
    centre = lip.mean(0)
    d0 = np.linalg.norm(m.pos[s0] - centre)
    rng = np.random.default_rng(seed)

    def mind(p, q):
        d = q - p
        d -= box * np.round(d / box)
        return np.sqrt((d * d).sum(-1))

    spheres = [m.pos[s0].copy()]
    # tangent to the vesicle: Fibonacci directions, kept where far enough apart
    k = 0
    while len(spheres) < count and k < 400:
        z = 1.0 - 2.0 * (k + 0.5) / 400
        phi = k * np.pi * (3.0 - np.sqrt(5.0))
        k += 7
        p = centre + d0 * np.array([np.sqrt(1 - z * z) * np.cos(phi), np.sqrt(1 - z * z) * np.sin(phi), z])
        p = np.mod(p, box)
        if mind(p, np.array(spheres)).min() > 2 * rad + 1 and len(spheres) < max(2, count // 2):
            spheres.append(p)
    tries = 0

    def free(p, sep):
        return mind(p, lip).min() > rng_c0 + 0.5 and mind(p, np.array(spheres)).min() > sep

    if pair_gap is not None:
        for _ in range(2):
            if len(spheres) + 2 > count:
                break
            while True:
                tries += 1
                p = rng.uniform(0, box)
                u = rng.normal(size=3)
                q = np.mod(p + pair_gap * u / np.linalg.norm(u), box)
                if free(p, 2 * rad + 1) and free(q, 2 * rad + 1) and mind(p, q[None])[0] > 2 * rad + 1e-9:
                    spheres += [p, q]
                    break
    while len(spheres) < count:
        tries += 1
        assert tries < 200000, "no room for the spheres"
        p = rng.uniform(0, box)
        if free(p, 2 * rad + 1):
            spheres.append(p)
    extra = spheres[1:]
    n = len(m.type)
    tok = open(path).read().split("\n")
    out, i = [], 0
    while i < len(tok):
        ln = tok[i]
        key = ln.strip()
        if key.startswith("nParticles"):
            out.append(f"nParticles {n + len(extra)} ")
        elif key.startswith("size") and size is not None:
            out.append("size %.17g %.17g %.17g " % tuple(box))
        elif key == "positions":
            out.extend(tok[i:i + 1 + n])
            out.extend(" %d %.15g %.15g %.15g" % (ts, *p) for p in extra)
            i += n + 1
            continue
        elif key == "velocities":
            out.extend(tok[i:i + 1 + n])
            out.extend(" 0 0 0" for _ in extra)
            i += n + 1
            continue
        elif key.split() == ["9", "1"]:
            # the BEAD block: header, its 22 nT^2 constants, then one index per
            # bead; the sphere-sphere row becomes the head-sphere row, so that
            # spheres in each other's range attract as bead partners too
            out.append("9\t %d" % len(spheres))
            i += 1
            vals = []
            while len(vals) < 22 * nT * nT:
                vals += tok[i].split()
                i += 1
            C = np.array(vals, dtype=float).reshape(nT * nT, 22)
            C[ts * nT + ts] = C[ts * nT + 2]
            out.extend(" " + "  ".join("%.17g" % x for x in row) for row in C)
            while not tok[i].split():
                out.append(tok[i])
                i += 1
            out.append(tok[i])  # the generator's sphere
            out.extend(f" {n + q}" for q in range(len(extra)))
            i += 1
            continue
        else:
            out.append(ln)
        i += 1
    open(path, "w").write("\n".join(out))


def make_spheres(tmp):
    """spheres24 / spheres6 / spheres21n2: BEAD residues of several beads on a
    300-lipid vesicle, dumped by the reference (forces at the start
    configuration, as sphere300).  spheres24 (radius 1.5, range 3.5) takes the
    hash-cell branch with 5 cells per axis and holds two sphere pairs 3.25
    apart, inside each other's range; spheres6 keeps six of its beads (the
    generator's, three tangent ones and the first close pair), the
    brute-force branch; spheres21n2 (radius 6, range 8) takes the hash-cell
    branch in a 40 x 52 x 52 box, 2 x 3 x 3 cells, where the reference visits
    the other cell along x twice.  The beads outside a residue keep the
    sphere's type and interact through the pair table only."""
    for name, count, R, size, gap in (("spheres24", 24, 2.5, None, 3.25), ("spheres6", 6, 2.5, None, 3.25),
                                      ("spheres21n2", 21, 7.0, (40.0, 52.0, 52.0), None)):
        f = os.path.join(tmp, name + ".mpd")
        smd.synth_vesicle_sphere(f, 99, 300, 3.45, 40.0, R, -10.0, 10.0, 0.8)
        if name == "spheres6":
            shutil.copy(os.path.join(tmp, "spheres24.mpd"), f)
            to_some_spheres(f, [0, 1, 2, 3, 12, 13])
        else:
            to_many_spheres(f, count, 5, size, gap)
        dump_case(tmp, name, name)


def to_some_spheres(path, keep):
    """Keeps the beads of the BEAD residue at the list positions `keep` (the
    others stay as ordinary beads of the sphere's type)."""
    tok = open(path).read().split("\n")
    mol = tok.index("molecule ")
    out, i = tok[:mol], mol
    while i < len(tok):
        f = tok[i].split()
        if len(f) == 2 and f[0] == "9":  # a molecule header: BEAD and its bead count
            out.append("9\t %d" % len(keep))
            i += 1
            while len(tok[i].split()) != 1:  # constant rows and blank lines
                out.append(tok[i])
                i += 1
            idx = tok[i:i + int(f[1])]
            out.extend(idx[q] for q in keep)
            i += int(f[1])
            continue
        out.append(tok[i])
        i += 1
    open(path, "w").write("\n".join(out))


def make_msd(tmp):
    """msd_bil/: a reference run that crosses 100 tau, so that it tracks
    diffusion: the 200-lipid bilayer of traj_bil as a checkpoint at
    initialTime 99.84, to finalTime 100.8."""
    mdir = os.path.join(HERE, "msd_bil")
    shutil.rmtree(mdir, ignore_errors=True)
    os.makedirs(os.path.join(mdir, "out"))
    path = os.path.join(mdir, "bil.mpd")
    smd.synth_bilayer(path, 5, 200, 3.45, 16.0, 0.01, 0.0)
    set_run(path, 100.8, 0.48, 0.16)
    t = open(path).read()
    t = re.sub(r"initialTime \S+", "initialTime 99.84", t)
    open(path, "w").write(t)
    run_dir = os.path.join(tmp, "msd")
    os.makedirs(run_dir)
    shutil.copy(path, run_dir)
    run_ref_md(run_dir, "bil")
    digests = {}
    for f in sorted(glob.glob(os.path.join(run_dir, "*"))):
        data = open(f, "rb").read()
        digests[os.path.basename(f)] = hashlib.sha256(data).hexdigest()
        if len(data) < 100_000:  # large histograms are kept as digests only
            shutil.copy(f, os.path.join(mdir, "out"))
    json.dump(digests, open(os.path.join(mdir, "digests.json"), "w"), indent=1)


def run_ref_md(workdir, name):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.run([os.path.join(REF, "MD"), name], cwd=workdir, env=env, check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


def dump_case(workdir, name, out_name):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    dump = os.path.join(workdir, "dump")
    os.makedirs(dump, exist_ok=True)
    args = [os.path.join(REF, "ref_dump"), name, dump] + [f"{x:.17g}" for x in SCALES.ravel()]
    subprocess.run(args, cwd=workdir, env=env, check=True, stdout=subprocess.DEVNULL)
    m = smd.read_mpd(os.path.join(workdir, name + ".mpd"))
    n = len(m.type)
    rd = lambda f, dt: np.fromfile(os.path.join(dump, f), dtype=dt)  # noqa: E731
    np.savez_compressed(
        os.path.join(HERE, out_name + ".npz"),
        pos=m.pos, vel=m.vel, type=m.type, box=m.box, cutoff=m.cutoff, n_types=m.n_types,
        fconst=m.fconst, uconst=m.uconst, chain_blocks=m.chain_blocks, chain_consts=m.chain_consts,
        dt=m.dt, gamma=m.gamma, temperature=m.temperature, seed=m.seed, tension=m.tension,
        delta_lxy=m.delta_lxy,
        sphere_index=m.sphere_index if m.sphere_index is not None else np.zeros(0, np.int32),
        sphere_consts=m.sphere_consts if m.sphere_consts is not None else np.zeros(0),
        bonds=m.bonds if m.bonds is not None else np.zeros((0, 2), np.int32),
        bond_consts=m.bond_consts if m.bond_consts is not None else np.zeros((0, 2)),
        bends=m.bends if m.bends is not None else np.zeros((0, 3), np.int32),
        bend_consts=m.bend_consts if m.bend_consts is not None else np.zeros((0, 2)),
        fields=m.fields if m.fields is not None else np.zeros((0, 3), np.int32),
        field_consts=m.field_consts if m.field_consts is not None else np.zeros((0, 8)),
        core_index=m.core_index if m.core_index is not None else np.zeros(0, np.int32),
        core_consts=m.core_consts if m.core_consts is not None else np.zeros((0, 22)),
        keys=rd("keys.i32", np.int32), pairs=rd("pairs.i32", np.int32).reshape(-1, 2),
        pair_force=rd("pair_force.f64", np.float64).reshape(n, 3),
        force=rd("force.f64", np.float64).reshape(n, 3),
        energy=rd("energy.f64", np.float64), scales=SCALES,
        rand53=rd("rand53.f64", np.float64))


def make_fields(tmp):
    """field400 (relaxed bilayer with the four external-field residues) and
    field200/ (their 48-step reference MD run)."""
    smd.synth_bilayer(os.path.join(tmp, "fld.mpd"), 93, 400, 3.45, 20.0, 0.01, 0.0)
    set_run(os.path.join(tmp, "fld.mpd"), 4, 4, 4)
    run_ref_md(tmp, "fld")
    add_fields(os.path.join(tmp, "fld.mpd"), 93)
    dump_case(tmp, "fld", "field400")
    fdir = os.path.join(HERE, "field200")
    os.makedirs(fdir, exist_ok=True)
    smd.synth_bilayer(os.path.join(fdir, "fld.mpd"), 6, 200, 3.45, 16.0, 0.01, 0.0)
    add_fields(os.path.join(fdir, "fld.mpd"), 6)
    set_run(os.path.join(fdir, "fld.mpd"), 0.96, 0.48, 0.16)
    run_dir = os.path.join(tmp, "fldrun")
    os.makedirs(run_dir)
    shutil.copy(os.path.join(fdir, "fld.mpd"), run_dir)
    run_ref_md(run_dir, "fld")
    json.dump({os.path.basename(f): hashlib.sha256(open(f, "rb").read()).hexdigest()
               for f in sorted(glob.glob(os.path.join(run_dir, "*")))},
              open(os.path.join(fdir, "digests.json"), "w"), indent=1)


def make_nanocore(tmp):
    """core300 (a 300-lipid vesicle with a NANOCORE residue of two cores,
    0.8 sigma outside its heads and 3.9 sigma apart, at the edge of each other's
    well) and core200/ (a 48-step reference MD run of a 200-lipid one)."""
    smd.synth_vesicle_sphere(os.path.join(tmp, "core.mpd"), 99, 300, 3.45, 40.0, 3.0, -10.0, 300.0, 0.8, 100.0)
    to_nanocore(os.path.join(tmp, "core.mpd"), 3.9)
    dump_case(tmp, "core", "core300")
    cdir = os.path.join(HERE, "core200")
    os.makedirs(cdir, exist_ok=True)
    smd.synth_vesicle_sphere(os.path.join(cdir, "core.mpd"), 8, 200, 3.45, 36.0, 3.0, -10.0, 300.0, 0.8, 100.0)
    to_nanocore(os.path.join(cdir, "core.mpd"), 3.9)
    set_run(os.path.join(cdir, "core.mpd"), 0.96, 0.48, 0.16)
    run_dir = os.path.join(tmp, "corerun")
    os.makedirs(run_dir)
    shutil.copy(os.path.join(cdir, "core.mpd"), run_dir)
    run_ref_md(run_dir, "core")
    json.dump({os.path.basename(f): hashlib.sha256(open(f, "rb").read()).hexdigest()
               for f in sorted(glob.glob(os.path.join(run_dir, "*")))},
              open(os.path.join(cdir, "digests.json"), "w"), indent=1)


def main():
    if not os.path.exists(os.path.join(REF, "ref_dump")):
        sys.exit("oracle/_ref is missing: run oracle/build_ref.sh first")
    tmp = tempfile.mkdtemp(prefix="smd_golden_")
    if "--only-msd" in sys.argv:  # the diffusion-tracking fixture alone
        try:
            make_msd(tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        print("msd fixture written to", HERE)
        return
    if "--only-restart" in sys.argv:  # the checkpoint-continuation fixtures alone
        try:
            make_restart(tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        print("restart fixtures written to", HERE)
        return
    if "--only-mixed" in sys.argv:  # the two-lipid fixtures alone
        try:
            make_mixed(tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        print("mixed fixtures written to", HERE)
        return
    if "--only-nanocore" in sys.argv:  # the NANOCORE fixtures alone
        try:
            make_nanocore(tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        print("nanocore fixtures written to", HERE)
        return
    if "--only-spheres" in sys.argv:  # the many-sphere BEAD fixtures alone
        try:
            make_spheres(tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        print("sphere fixtures written to", HERE)
        return
    if "--only-fields" in sys.argv:  # the external-field fixtures alone
        try:
            make_fields(tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        print("field fixtures written to", HERE)
        return
    try:
        # relaxed vesicle, 300 lipids in a 30^3 box
        smd.synth_vesicle(os.path.join(tmp, "ves.mpd"), 1234, 300, 3.45, 30.0)
        set_run(os.path.join(tmp, "ves.mpd"), 4, 4, 4)
        run_ref_md(tmp, "ves")
        dump_case(tmp, "ves", "ves300")
        # relaxed bilayer, 400 lipids, barostat on
        smd.synth_bilayer(os.path.join(tmp, "bil.mpd"), 77, 400, 3.45, 20.0, 0.01, 0.0)
        set_run(os.path.join(tmp, "bil.mpd"), 4, 4, 4)
        run_ref_md(tmp, "bil")
        dump_case(tmp, "bil", "bil400")
        # relaxed bilayer with a head network: BOND and BEND residues beside CHAIN
        smd.synth_bilayer(os.path.join(tmp, "net.mpd"), 91, 400, 3.45, 20.0, 0.01, 0.0)
        add_network(os.path.join(tmp, "net.mpd"), 91)
        set_run(os.path.join(tmp, "net.mpd"), 4, 4, 4)
        run_ref_md(tmp, "net")
        dump_case(tmp, "net", "net400")
        # unrelaxed 200-lipid network system: input of trajectory and MD tests
        ndir = os.path.join(HERE, "net200")
        os.makedirs(ndir, exist_ok=True)
        smd.synth_bilayer(os.path.join(ndir, "net.mpd"), 5, 200, 3.45, 16.0, 0.01, 0.0)
        add_network(os.path.join(ndir, "net.mpd"), 5)
        set_run(os.path.join(ndir, "net.mpd"), 0.96, 0.48, 0.16)
        run_dir = os.path.join(tmp, "netrun")
        os.makedirs(run_dir)
        shutil.copy(os.path.join(ndir, "net.mpd"), run_dir)
        run_ref_md(run_dir, "net")
        json.dump({os.path.basename(f): hashlib.sha256(open(f, "rb").read()).hexdigest()
                   for f in sorted(glob.glob(os.path.join(run_dir, "*")))},
                  open(os.path.join(ndir, "digests.json"), "w"), indent=1)
        # vesicle with a continuum sphere (BEAD residue, radius 5) whose surface
        # is 0.8 sigma outside the outer heads, inside its attractive well; the
        # reference's Umax=10 core is not repulsive enough for a stable run, so
        # the forces are dumped on the start configuration
        smd.synth_vesicle_sphere(os.path.join(tmp, "sph.mpd"), 99, 300, 3.45, 40.0, 5.0, -10.0, 10.0, 0.8)
        dump_case(tmp, "sph", "sphere300")
        # trajectory: every output file of a short reference run
        tdir = os.path.join(HERE, "traj_bil")
        shutil.rmtree(tdir, ignore_errors=True)
        os.makedirs(os.path.join(tdir, "out"))
        smd.synth_bilayer(os.path.join(tdir, "bil.mpd"), 5, 200, 3.45, 16.0, 0.01, 0.0)
        set_run(os.path.join(tdir, "bil.mpd"), 0.96, 0.48, 0.16)
        run_dir = os.path.join(tmp, "traj")
        os.makedirs(run_dir)
        shutil.copy(os.path.join(tdir, "bil.mpd"), run_dir)
        run_ref_md(run_dir, "bil")
        digests = {}
        for f in sorted(glob.glob(os.path.join(run_dir, "*"))):
            data = open(f, "rb").read()
            digests[os.path.basename(f)] = hashlib.sha256(data).hexdigest()
            if len(data) < 100_000:  # large histograms are kept as digests only
                shutil.copy(f, os.path.join(tdir, "out"))
        json.dump(digests, open(os.path.join(tdir, "digests.json"), "w"), indent=1)
        # generator digests
        gens = []
        for seed, n in [(1234, 300), (7, 1000)]:
            d = os.path.join(tmp, f"g{seed}")
            os.makedirs(d)
            subprocess.run([os.path.join(REF, "liposome"), "g", str(seed), str(n), "3.45"], cwd=d, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            gens.append(dict(kind="liposome", seed=seed, n=n, density=3.45,
                             sha256=hashlib.sha256(open(os.path.join(d, "g.mpd"), "rb").read()).hexdigest()))
        for seed, n in [(77, 400), (3, 2000)]:
            d = os.path.join(tmp, f"b{seed}")
            os.makedirs(d)
            subprocess.run([os.path.join(REF, "bilayer"), "g", str(seed), str(n), "3.45", "0", "0", "0", "0"],
                           cwd=d, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            gens.append(dict(kind="bilayer", seed=seed, n=n, density=3.45,
                             sha256=hashlib.sha256(open(os.path.join(d, "g.mpd"), "rb").read()).hexdigest()))
        json.dump(gens, open(os.path.join(HERE, "generators.json"), "w"), indent=1)
        make_fields(tmp)
        make_nanocore(tmp)
        make_mixed(tmp)
        make_restart(tmp)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
