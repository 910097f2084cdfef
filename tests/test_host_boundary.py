"""Host side of the boundary: the C-ABI library, the synthetic generators and
the .mpd reader.  No GPU is touched here."""
import ctypes
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest
from conftest import GOLDEN

import softmold_gb300 as smd


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(smd.LIB_PATH)
    declared = smd.declared_symbols()
    assert len(declared) >= 25
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    # the Python mirror binds every declared function
    assert sorted(set(declared) - set(smd._SIGS)) == []


def test_oracle_is_a_separate_library(built):
    """The product library carries no oracle code."""
    out = subprocess.run(["nm", "-D", "--defined-only", smd.LIB_PATH], capture_output=True, text=True).stdout
    assert "orc_" not in out


@pytest.mark.parametrize("entry", json.load(open(os.path.join(GOLDEN, "generators.json"))))
def test_generators_byte_identical_to_reference(built, tmp_path, entry):
    p = str(tmp_path / "g.mpd")
    if entry["kind"] == "liposome":
        smd.synth_vesicle(p, entry["seed"], entry["n"], entry["density"], 400.0)
    else:
        smd.synth_bilayer(p, entry["seed"], entry["n"], entry["density"], 40.0, 0.01, 0.0)
    assert hashlib.sha256(open(p, "rb").read()).hexdigest() == entry["sha256"]


def test_mpd_reader_roundtrip(built, tmp_path):
    p = str(tmp_path / "b.mpd")
    smd.synth_bilayer(p, 3, 200, 3.45, 16.0, 0.01, 0.25)
    m = smd.read_mpd(p)
    assert len(m.type) == 600 and m.pos.shape == (600, 3)
    assert m.chain_blocks.tolist() == [[0, 200, 3]]
    assert np.allclose(m.chain_consts, [[0.7, 100, 1, 100]])
    assert m.delta_lxy == 0.01 and m.tension == 0.25
    assert (m.pos >= 0).all() and (m.pos <= m.box).all()


def test_create_without_device_fails_loudly(built):
    """No CPU fallback: without a GPU the library refuses to build a system."""
    if smd.lib().smd_device_count() > 0:
        pytest.skip("a GPU is present")
    g = np.load(os.path.join(GOLDEN, "bil400.npz"))
    from conftest import mpd_from_golden
    with pytest.raises(smd.SmdError, match="no CUDA device"):
        smd.System(mpd_from_golden({k: g[k] for k in g.files}))


def test_md_executable_usage(built):
    r = subprocess.run([smd.MD_EXE], capture_output=True, text=True)
    assert r.returncode == 0 and "usage" in r.stderr


def _bad(**kw):
    import dataclasses
    from conftest import load_golden, mpd_from_golden
    m = mpd_from_golden(load_golden("bil400"))
    return dataclasses.replace(m, **kw)


@pytest.mark.parametrize("change,message", [
    ("empty", "n must be positive"),
    ("short box", "shorter than 3 cutoffs"),
    ("type", "bead type out of range"),
    ("outside", "position out of the box"),
    ("chain", "CHAIN block out of range"),
    ("bond", "BOND bead index out of range"),
    ("dt", "dt must be positive"),
    ("nan position", "position out of the box"),
    ("inf velocity", "velocity not finite"),
    ("nan table", "pair table value not finite"),
    ("nan chain", "CHAIN constant not finite"),
    ("inf gamma", "gamma, temperature"),
    ("negative temperature", "gamma, temperature"),
    ("nan bond", "BOND constant not finite"),
    ("inf box", "box must be positive and finite"),
    ("long box", "box edge above"),
    ("sparse grid", "cell grid of the handle exceeds"),
    ("inf skin", "skin not finite"),
])
def test_invalid_descriptors_are_refused_before_any_device_work(built, change, message):
    """The descriptor checks run on the host before the device is touched,
    so they hold with or without a GPU: an error code and a message, as the
    reference's `throw 0` with a message on stdout."""
    from conftest import load_golden
    g = load_golden("bil400")
    pos, typ = np.array(g["pos"]), np.array(g["type"], np.int32)
    if change == "empty":
        m = _bad(pos=np.zeros((0, 3)), vel=np.zeros((0, 3)), type=np.zeros(0, np.int32),
                 chain_blocks=np.zeros((0, 3), np.int32), chain_consts=np.zeros((0, 4)))
    elif change == "short box":
        box = np.array(g["box"], np.float64)
        box[2] = 5.9
        m = _bad(box=box, pos=np.mod(pos, box))
    elif change == "type":
        typ[0] = int(g["n_types"])
        m = _bad(type=typ)
    elif change == "outside":
        pos[0, 0] = -0.5
        m = _bad(pos=pos)
    elif change == "chain":
        m = _bad(chain_blocks=np.array([[len(pos) - 2, 1, 3]], np.int32), chain_consts=np.array([[0.7, 100, 1, 100]]))
    elif change == "bond":
        m = _bad(bonds=np.array([[0, len(pos)]], np.int32), bond_consts=np.array([[0.7, 100.0]]))
    elif change == "nan position":
        pos[3, 1] = np.nan
        m = _bad(pos=pos)
    elif change == "inf velocity":
        vel = np.array(g["vel"], np.float64)
        vel[5, 2] = np.inf
        m = _bad(vel=vel)
    elif change == "nan table":
        fc = np.array(g["fconst"], np.float64).copy()
        fc[7] = np.nan
        m = _bad(fconst=fc)
    elif change == "nan chain":
        cc = np.array(g["chain_consts"], np.float64).reshape(-1, 4).copy()
        cc[0, 1] = np.nan
        m = _bad(chain_consts=cc)
    elif change == "inf gamma":
        m = _bad(gamma=np.inf)
    elif change == "negative temperature":
        m = _bad(temperature=-1.0)
    elif change == "nan bond":
        m = _bad(bonds=np.array([[0, 1]], np.int32), bond_consts=np.array([[0.7, np.nan]]))
    elif change in ("inf box", "long box"):
        box = np.array(g["box"], np.float64)
        box[2] = np.inf if change == "inf box" else 1e12
        m = _bad(box=box)
    elif change == "sparse grid":
        # the beads stay where they are in a 10,000^3 box: 4,000 list cells
        # of cutoff 2 + skin 0.5 per axis, 6.4e10 in all, a count that
        # overflows an int
        m = _bad(box=np.full(3, 10000.0))
    elif change == "inf skin":
        with pytest.raises(smd.SmdError, match=message):
            smd.System(_bad(), skin=np.inf)
        return
    else:
        m = _bad(dt=0.0)
    with pytest.raises(smd.SmdError, match=message):
        smd.System(m)


def test_batch_cell_grid_is_bounded_over_all_replicas(built):
    """Each of 60 replicas in a 427^3 box has 171^3 ≈ 5.0 M list cells (170
    cells of cutoff 2 + skin 0.5 per axis, one extra), within the bound alone;
    the 54th brings the handle past 2^28 cells and the batch is refused before
    any device work."""
    box = np.full(3, 427.0)
    with pytest.raises(smd.SmdError, match="replica 53: the cell grid of the handle exceeds"):
        smd.System([_bad(box=box)] * 60)


def test_batch_replicas_must_share_the_pair_tables(built):
    a = _bad()
    f = np.array(a.fconst, np.float64).copy()
    f[0] += 1.0
    with pytest.raises(smd.SmdError, match="share the pair tables"):
        smd.System([a, _bad(fconst=f)])


@pytest.mark.parametrize("case,message", [
    ("missing", "Could not open"),
    ("truncated", "is missing (end of file)"),
    ("corrupt", "is not a numerical type"),
])
def test_md_executable_refuses_bad_input_files(built, tmp_path, case, message):
    """A missing, truncated or corrupt .mpd is reported with a message (the
    reference's Script reader throws with one) before any device work, and
    no output file is written."""
    src = open(os.path.join(GOLDEN, "traj_bil", "bil.mpd")).read()
    if case == "truncated":
        (tmp_path / "bil.mpd").write_text(src[:3000])
    elif case == "corrupt":
        (tmp_path / "bil.mpd").write_text(src.replace("cutoff 2", "cutoff two", 1))
    r = subprocess.run([smd.MD_EXE, "bil"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0
    assert message in r.stdout + r.stderr
    assert sorted(os.listdir(tmp_path)) == ([] if case == "missing" else ["bil.mpd"])


def test_reader_is_the_md_executables():
    """read_mpd goes through the library's reader and residue expansion
    (smd_mpd_load), the code path of the `MD` executable: residues expand
    into the device step's terms, run settings come with them, and files the
    device step cannot run are refused with the executable's message."""
    import softmold_gb300 as smd
    from conftest import GOLDEN
    net = smd.read_mpd(os.path.join(GOLDEN, "net200", "net.mpd"))
    assert len(net.type) == 600 and net.chain_blocks.shape == (1, 3) and net.bonds.shape[1] == 2
    assert net.bends is not None and net.fields is None and net.sphere_index is None
    fld = smd.read_mpd(os.path.join(GOLDEN, "field200", "fld.mpd"))
    assert set(np.unique(fld.fields[:, 0])) <= {11, 15, 16, 17, 19} and fld.field_consts.shape[1] == 8
    core = smd.read_mpd(os.path.join(GOLDEN, "core200", "core.mpd"))
    assert list(core.core_index) == [600, 601] and core.core_consts.shape == (2, 22) and core.sphere_index is None
    msd = smd.read_mpd(os.path.join(GOLDEN, "msd_bil", "bil.mpd"))
    assert msd.initial_time == 99.84 and msd.final_time == 100.8


def test_reader_refusals(tmp_path):
    import softmold_gb300 as smd
    from conftest import GOLDEN
    with pytest.raises(smd.SmdError):
        smd.read_mpd(str(tmp_path / "missing.mpd"))
    txt = open(os.path.join(GOLDEN, "traj_bil", "bil.mpd")).read()
    (tmp_path / "cut.mpd").write_text(txt[:len(txt) // 2])
    with pytest.raises(smd.SmdError):
        smd.read_mpd(str(tmp_path / "cut.mpd"))


@pytest.mark.parametrize("old,new,message", [
    ("nParticles 600", "nParticles -600", "Count for positions is negative"),
    ("nParticles 600", "nParticles 2000000000", "Value after positions is missing"),
    ("nTypes 6", "nTypes 100000", "nTypes must be in 0..4096"),
    ("8\t 1", "8\t -1", "bond count out of range"),
    ("8\t 1", "8\t 900000000", "bond count out of range"),
])
def test_reader_refuses_counts_before_allocating(tmp_path, old, new, message):
    """Counts in a damaged file (negative, or more entries than the file
    holds) are refused with a message before the reader sizes an array from
    them, so that no allocation error escapes the C ABI."""
    import softmold_gb300 as smd
    from conftest import GOLDEN
    txt = open(os.path.join(GOLDEN, "traj_bil", "bil.mpd")).read()
    assert txt.count(old) == 1
    (tmp_path / "bad.mpd").write_text(txt.replace(old, new))
    with pytest.raises(smd.SmdError, match=message):
        smd.read_mpd(str(tmp_path / "bad.mpd"))


def test_state_rewrite_checks_array_sizes(built, tmp_path):
    """mpd_update_state hands the library pointers it reads nParticles x 3
    values from: arrays of another size are refused before the call."""
    import softmold_gb300 as smd
    from conftest import GOLDEN
    src = os.path.join(GOLDEN, "traj_bil", "bil.mpd")
    m = smd.read_mpd(src)
    n = len(m.type)
    out = str(tmp_path / "out.mpd")
    with pytest.raises(ValueError, match="nParticles"):
        smd.mpd_update_state(src, out, np.zeros((n - 1, 3)), np.zeros((n, 3)), m.box, 1.0)
    with pytest.raises(ValueError, match="box 3"):
        smd.mpd_update_state(src, out, m.pos, m.vel, np.zeros(2), 1.0)
    smd.mpd_update_state(src, out, m.pos, m.vel, m.box, 1.0)
    back = smd.read_mpd(out)
    assert np.array_equal(back.pos, m.pos) and back.initial_time == 1.0
