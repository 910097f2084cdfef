"""The oracle against vectors dumped from the reference's own code.

The restatement keeps the reference's traversal and summation order and is
built with the same flags, so on one thread everything matches bit for bit.
"""
import numpy as np
import pytest
from conftest import load_golden

CASES = ["ves300", "bil400", "sphere300", "net400", "field400", "core300", "mix400", "spheres6", "spheres24",
         "spheres21n2"]


@pytest.mark.parametrize("case", CASES)
def test_mt19937_rand53(oracle, case):
    g = load_golden(case)
    assert np.array_equal(oracle.rand53(int(g["seed"]), len(g["rand53"])), g["rand53"])


@pytest.mark.parametrize("case", CASES)
def test_cell_keys_bit_exact(oracle, case):
    g = load_golden(case)
    keys = oracle.cell_keys(g["pos"], g["box"], float(g["cutoff"]))
    assert np.array_equal(keys, g["keys"])


@pytest.mark.parametrize("case", CASES)
def test_pair_list_visiting_order(oracle, case):
    g = load_golden(case)
    pairs = oracle.pair_list(g["pos"], g["box"], float(g["cutoff"]))
    assert pairs.shape == g["pairs"].shape
    assert np.array_equal(pairs, g["pairs"])


@pytest.mark.parametrize("case", CASES)
def test_forces_bit_exact(oracle, case):
    g = load_golden(case)
    assert np.array_equal(oracle.forces(g, pair_only=True), g["pair_force"])
    assert np.array_equal(oracle.forces(g), g["force"])


@pytest.mark.parametrize("case", CASES)
def test_energies_and_size_change(oracle, case):
    g = load_golden(case)
    e = g["energy"]
    pair, bonded, bead = oracle.energies(g)
    assert (pair, bonded, bead) == (e[0], e[1], e[2])
    for k, s in enumerate(g["scales"]):
        dp, db, dbead = oracle.energies(g, scale=s)
        assert (dp, db, dbead) == (e[3 + 3 * k], e[4 + 3 * k], e[5 + 3 * k])


def test_sphere_case_interacts():
    """The BEAD fixture exercises the continuum-sphere terms."""
    g = load_golden("sphere300")
    assert len(g["sphere_index"]) == 1
    assert g["energy"][2] != 0.0


def _sphere_geometry(g):
    idx = g["sphere_index"]
    p = g["pos"][idx]
    d = p[:, None, :] - p[None, :, :]
    d -= g["box"] * np.round(d / g["box"])
    r = np.sqrt((d * d).sum(-1))
    np.fill_diagonal(r, np.inf)
    return r, float(g["sphere_consts"][0])


def test_many_sphere_cases_exercise_both_branches(oracle):
    """spheres6 takes the brute-force branch (<= 20 beads) and spheres24 the
    hash-cell branch; both hold sphere pairs within each other's bead range,
    whose force the two branches treat differently.  spheres21n2 has two hash
    cells along x, where the reference visits the other cell twice."""
    for case, n in (("spheres6", 6), ("spheres24", 24), ("spheres21n2", 21)):
        g = load_golden(case)
        assert len(g["sphere_index"]) == n
        assert g["energy"][2] != 0.0
    for case in ("spheres6", "spheres24"):
        r, rng = _sphere_geometry(load_golden(case))
        assert (r < rng).sum() >= 2  # an ordered pair at least
    g = load_golden("spheres21n2")
    rng = float(g["sphere_consts"][0])
    cells = (g["box"] / (2 * rng)).astype(int)
    assert list(cells) == [2, 3, 3]
    # head beads in a sphere's range but in the other cell along x: their
    # terms count twice
    cx = np.floor(g["pos"][:, 0] / (g["box"][0] / 2)).astype(int)
    crossing = 0
    for s in g["sphere_index"]:
        d = g["pos"] - g["pos"][s]
        d -= g["box"] * np.round(d / g["box"])
        r = np.sqrt((d * d).sum(1))
        crossing += int(((r > 0) & (r < rng) & (cx != cx[s])).sum())
    assert crossing >= 1
    # the same beads through the brute-force rule would give other forces
    g6 = dict(load_golden("spheres24"))
    f_hash = oracle.forces(g6)
    g6["sphere_index"] = g6["sphere_index"][:20]
    f_brute = oracle.forces(g6)
    assert np.abs(f_hash - f_brute).max() > 0
