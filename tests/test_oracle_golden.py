"""The oracle against vectors dumped from the reference's own code.

The restatement keeps the reference's traversal and summation order and is
built with the same flags, so on one thread everything matches bit for bit.
"""
import numpy as np
import pytest
from conftest import load_golden

CASES = ["ves300", "bil400", "sphere300", "net400", "field400", "core300", "mix400"]


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
