"""smd_pair_forces_static: the non-bonded forces for callers that cannot
allocate device memory (another framework owns the device memory, or the
calling loop must not take cudaMalloc's implicit device synchronisation).

The entry point keeps its cell-list scratch in a fixed array inside the
library, so every call reuses the previous call's contents.  Two calls in a
row on different systems must each agree with smd_compute_pair_forces, the
allocating entry point, and with the pair forces dumped from the reference
(CellOpt::computeForce, include/algorithms/cellOpt.h:712-926), to the
plain-FP64 tolerance used for forces (1e-12 of max |F|).  Only in-range
inputs are sent to the GPU; the clamping of out-of-range coordinates and
types is checked on the CPU (test_static_cell_cpu.py).  This file is
collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
from conftest import load_golden, mpd_from_golden

import softmold_gb300 as smd

pytestmark = pytest.mark.gpu


def _static_forces(torch, g):
    dev = torch.device("cuda")
    pos = torch.tensor(np.ascontiguousarray(g["pos"]), dtype=torch.float64, device=dev)
    typ = torch.tensor(np.ascontiguousarray(g["type"]), dtype=torch.int32, device=dev)
    fc = torch.tensor(np.ascontiguousarray(g["fconst"]), dtype=torch.float64, device=dev)
    out = torch.full((len(g["type"]), 3), float("nan"), dtype=torch.float64, device=dev)
    box = np.ascontiguousarray(g["box"], np.float64)
    rc = smd.lib().smd_pair_forces_static(pos.data_ptr(), typ.data_ptr(), len(g["type"]), box.ctypes.data,
                                          float(g["cutoff"]), int(g["n_types"]), fc.data_ptr(), out.data_ptr(),
                                          None)
    assert rc == 0, smd.last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _allocating(g):
    s = smd.System(mpd_from_golden(g), precision=smd.PLAIN_FP64)
    try:
        return s.forces(pair_only=True)
    finally:
        s.close()


def test_static_forces_match_allocating_entry_point():
    torch = pytest.importorskip("torch")
    for case in ("bil400", "ves300"):  # different sizes and grids, one after the other
        g = load_golden(case)
        want = _allocating(g)
        got = _static_forces(torch, g)
        scale = np.abs(want).max()
        assert np.abs(got - want).max() / scale <= 1e-12, case
        # the reference's own pair forces, dumped from CellOpt::computeForce
        assert np.abs(got - g["pair_force"]).max() / np.abs(g["pair_force"]).max() <= 1e-12, case


def test_static_forces_on_the_box_faces(oracle):
    """Beads exactly on the faces x = 0 and x = L (both inside [0, L]):
    the reference's x >= n -> n-1 cell, against the allocating entry point
    and the oracle."""
    torch = pytest.importorskip("torch")
    g = dict(load_golden("bil400"))
    pos = np.array(g["pos"], np.float64)
    box = np.asarray(g["box"], np.float64)
    for k, i in enumerate(range(0, 48, 4)):
        d = k % 3
        pos[i, d] = 0.0 if k % 2 == 0 else box[d]
    g["pos"] = pos
    got = _static_forces(torch, g)
    want = _allocating(g)
    ref = oracle.forces(g, pair_only=True)
    assert np.isfinite(got).all()
    scale = np.abs(ref).max()
    assert np.abs(got - want).max() / scale <= 1e-12
    assert np.abs(got - ref).max() / scale <= 1e-12


def test_static_rejects_sizes_beyond_its_maximum():
    n = smd.lib().smd_pair_forces_static  # validation happens before any device work
    box = np.array([100.0, 100.0, 100.0])
    dummy = ctypes.c_void_p(16)
    rc = n(dummy, dummy, 40000, box.ctypes.data, 2.0, 6, dummy, dummy, None)
    assert rc != 0 and "static maximum" in smd.last_error()
    big = np.array([500.0, 500.0, 500.0])
    rc = n(dummy, dummy, 1000, big.ctypes.data, 2.0, 6, dummy, dummy, None)
    assert rc != 0 and "cells exceed" in smd.last_error()
    for bad in (np.array([np.inf, 100.0, 100.0]), np.array([np.nan, 100.0, 100.0]), np.array([1e300, 1e300, 1e300]),
                np.array([-10.0, 100.0, 100.0])):
        rc = n(dummy, dummy, 1000, bad.ctypes.data, 2.0, 6, dummy, dummy, None)
        assert rc != 0, bad
