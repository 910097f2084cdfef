"""smd_pair_forces_static: the non-bonded forces for callers that cannot
allocate device memory (another framework owns the device memory, or the
calling loop must not take cudaMalloc's implicit device synchronisation).

The entry point keeps its cell-list scratch in a fixed array inside the
library, so every call reuses the previous call's contents.  Two calls in a
row on different systems must each agree with smd_compute_pair_forces, the
allocating entry point, to the plain-FP64 tolerance used for forces (1e-12 of
max |F|).  This file is collected last on purpose.
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


def test_static_forces_match_allocating_entry_point():
    torch = pytest.importorskip("torch")
    for case in ("bil400", "ves300"):  # different sizes and grids, one after the other
        g = load_golden(case)
        s = smd.System(mpd_from_golden(g), precision=smd.PLAIN_FP64)
        want = s.forces(pair_only=True)
        s.close()
        got = _static_forces(torch, g)
        err = np.abs(got - want).max() / np.abs(want).max()
        assert err <= 1e-12, (case, err)


def test_static_rejects_sizes_beyond_its_maximum():
    n = smd.lib().smd_pair_forces_static  # validation happens before any device work
    box = np.array([100.0, 100.0, 100.0])
    dummy = ctypes.c_void_p(16)
    rc = n(dummy, dummy, 40000, box.ctypes.data, 2.0, 6, dummy, dummy, None)
    assert rc != 0 and "static maximum" in smd.last_error()
    big = np.array([500.0, 500.0, 500.0])
    rc = n(dummy, dummy, 1000, big.ctypes.data, 2.0, 6, dummy, dummy, None)
    assert rc != 0 and "cells exceed" in smd.last_error()
