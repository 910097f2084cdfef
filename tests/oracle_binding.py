"""ctypes binding of the CPU oracle (oracle/_build/libsmd_oracle.so) for tests.

The oracle is the checker: tests call it beside the CUDA library and compare.
"""
import ctypes as C
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_build", "libsmd_oracle.so")
MD = os.path.join(ROOT, "oracle", "_build", "md_oracle")

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)


def _d(a):
    return np.ascontiguousarray(a, np.float64).ctypes.data_as(D)


def _i(a):
    return np.ascontiguousarray(a, np.int32).ctypes.data_as(I)


class Oracle:
    def __init__(self, path=LIB):
        L = C.CDLL(path)
        L.orc_mt_fill53.argtypes = [C.c_uint32, C.c_int, D]
        L.orc_cell_keys.argtypes = [C.c_int, D, D, C.c_double, I]
        L.orc_pair_list.argtypes = [C.c_int, D, D, C.c_double, I, C.c_long]
        L.orc_pair_list.restype = C.c_long
        L.orc_pair_force.argtypes = [C.c_int, D, I, D, C.c_double, C.c_int, D, D]
        L.orc_pair_potential.argtypes = [C.c_int, D, I, D, C.c_double, C.c_int, D]
        L.orc_pair_potential.restype = C.c_double
        L.orc_pair_dpotential.argtypes = [C.c_int, D, I, D, C.c_double, C.c_int, D, D]
        L.orc_pair_dpotential.restype = C.c_double
        L.orc_chain_force.argtypes = [D, D, C.c_int, C.c_int, C.c_int, D, D]
        L.orc_chain_potential.argtypes = [D, D, C.c_int, C.c_int, C.c_int, D]
        L.orc_chain_potential.restype = C.c_double
        L.orc_chain_dpotential.argtypes = [D, D, C.c_int, C.c_int, C.c_int, D, D]
        L.orc_chain_dpotential.restype = C.c_double
        for f in ("orc_bead_force",):
            getattr(L, f).argtypes = [C.c_int, D, I, D, C.c_int, C.c_int, I, D, D]
        L.orc_bead_potential.argtypes = [C.c_int, D, I, D, C.c_int, C.c_int, I, D]
        L.orc_bead_potential.restype = C.c_double
        L.orc_bead_dpotential.argtypes = [C.c_int, D, I, D, C.c_int, C.c_int, I, D, D]
        L.orc_bead_dpotential.restype = C.c_double
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads(1)
        L.orc_md_run.argtypes = [C.c_char_p, C.c_int]
        L.orc_md_time.argtypes = [C.c_char_p, C.c_int, C.c_int]
        L.orc_md_time.restype = C.c_double
        self.L = L

    def rand53(self, seed, n):
        out = np.zeros(n)
        self.L.orc_mt_fill53(seed, n, out.ctypes.data_as(D))
        return out

    def cell_keys(self, pos, box, rc):
        pos = np.ascontiguousarray(pos, np.float64)
        k = np.zeros(len(pos), np.int32)
        self.L.orc_cell_keys(len(pos), _d(pos), _d(box), rc, k.ctypes.data_as(I))
        return k

    def pair_list(self, pos, box, rc):
        pos = np.ascontiguousarray(pos, np.float64)
        n = self.L.orc_pair_list(len(pos), _d(pos), _d(box), rc, None, 0)
        out = np.zeros((max(n, 1), 2), np.int32)
        self.L.orc_pair_list(len(pos), _d(pos), _d(box), rc, out.ctypes.data_as(I), n)
        return out[:n]

    def forces(self, g, pair_only=False):
        """Conservative accelerations as CellOpt::computeForce + doChainForce
        (+ doBeadForce) compute them on the golden case's state."""
        pos = np.ascontiguousarray(g["pos"], np.float64)
        typ = np.ascontiguousarray(g["type"], np.int32)
        acc = np.zeros_like(pos)
        nT = int(g["n_types"])
        self.L.orc_pair_force(len(pos), pos.ctypes.data_as(D), typ.ctypes.data_as(I), _d(g["box"]),
                              float(g["cutoff"]), nT, _d(g["fconst"]), acc.ctypes.data_as(D))
        if pair_only:
            return acc
        for b, c in zip(g["chain_blocks"], g["chain_consts"]):
            self.L.orc_chain_force(pos.ctypes.data_as(D), _d(g["box"]), int(b[0]), int(b[1]), int(b[2]), _d(c),
                                   acc.ctypes.data_as(D))
        si = g.get("sphere_index")
        if si is not None and len(si):
            self.L.orc_bead_force(len(pos), pos.ctypes.data_as(D), typ.ctypes.data_as(I), _d(g["box"]), nT,
                                  len(si), _i(si), _d(g["sphere_consts"]), acc.ctypes.data_as(D))
        return acc

    def energies(self, g, scale=None):
        pos = np.ascontiguousarray(g["pos"], np.float64)
        typ = np.ascontiguousarray(g["type"], np.int32)
        nT = int(g["n_types"])
        args = (len(pos), pos.ctypes.data_as(D), typ.ctypes.data_as(I), _d(g["box"]), float(g["cutoff"]), nT,
                _d(g["uconst"]))
        if scale is None:
            pair = self.L.orc_pair_potential(*args)
        else:
            pair = self.L.orc_pair_dpotential(*args, _d(scale))
        bonded = 0.0
        for b, c in zip(g["chain_blocks"], g["chain_consts"]):
            a = (pos.ctypes.data_as(D), _d(g["box"]), int(b[0]), int(b[1]), int(b[2]), _d(c))
            bonded += self.L.orc_chain_potential(*a) if scale is None else self.L.orc_chain_dpotential(*a,
                                                                                                     _d(scale))
        bead = 0.0
        si = g.get("sphere_index")
        if si is not None and len(si):
            a = (len(pos), pos.ctypes.data_as(D), typ.ctypes.data_as(I), _d(g["box"]), nT, len(si), _i(si),
                 _d(g["sphere_consts"]))
            bead = self.L.orc_bead_potential(*a) if scale is None else self.L.orc_bead_dpotential(*a, _d(scale))
        return pair, bonded, bead


def load():
    return Oracle()
