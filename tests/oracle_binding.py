"""ctypes binding of the CPU oracle (oracle/_build/libsmd_oracle.so) for tests.

Tests call the oracle beside the CUDA library and compare the two.
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
        for f in ("orc_bond_force", "orc_bend_force"):
            getattr(L, f).argtypes = [D, D, C.c_int, I, D, D]
        for f in ("orc_bond_potential", "orc_bend_potential"):
            getattr(L, f).argtypes = [D, D, C.c_int, I, D]
            getattr(L, f).restype = C.c_double
        for f in ("orc_bond_dpotential", "orc_bend_dpotential"):
            getattr(L, f).argtypes = [D, D, C.c_int, I, D, D]
            getattr(L, f).restype = C.c_double
        L.orc_boundary_force.argtypes = [D, D, C.c_int, I, D, D]
        L.orc_boundary_potential.argtypes = [D, D, C.c_int, I, D]
        L.orc_boundary_potential.restype = C.c_double
        L.orc_floating_base_force.argtypes = [D, I, C.c_int, I, D, D]
        L.orc_floating_base_potential.argtypes = [D, I, C.c_int, I, D]
        L.orc_floating_base_potential.restype = C.c_double
        L.orc_zpower_force.argtypes = [D, C.c_int, I, D, D]
        L.orc_zpower_potential.argtypes = [D, C.c_int, I, D]
        L.orc_zpower_potential.restype = C.c_double
        L.orc_ztorque_force.argtypes = [D, D, C.c_int, I, D, D]
        L.orc_ztorque_potential.argtypes = [D, D, C.c_int, I, D]
        L.orc_ztorque_potential.restype = C.c_double
        L.orc_ball_force.argtypes = [D, D, C.c_int, I, D, D]
        L.orc_ball_potential.argtypes = [D, D, C.c_int, I, D]
        L.orc_ball_potential.restype = C.c_double
        L.orc_nanocore_force.argtypes = [C.c_int, D, D, C.c_int, I, D, D]
        L.orc_nanocore_potential.argtypes = [C.c_int, D, D, C.c_int, I, D]
        L.orc_nanocore_potential.restype = C.c_double
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
        for kind in ("bond", "bend"):
            for lst, c in self._residues(g, kind):
                getattr(self.L, f"orc_{kind}_force")(pos.ctypes.data_as(D), _d(g["box"]), len(lst), _i(lst), _d(c),
                                                    acc.ctypes.data_as(D))
        si = g.get("sphere_index")
        if si is not None and len(si):
            self.L.orc_bead_force(len(pos), pos.ctypes.data_as(D), typ.ctypes.data_as(I), _d(g["box"]), nT,
                                  len(si), _i(si), _d(g["sphere_consts"]), acc.ctypes.data_as(D))
        ci = g.get("core_index")
        if ci is not None and len(ci):
            self.L.orc_nanocore_force(len(pos), pos.ctypes.data_as(D), _d(g["box"]), len(ci), _i(ci),
                                      _d(np.ascontiguousarray(g["core_consts"]).ravel()), acc.ctypes.data_as(D))
        for kind, idx, c in self._field_residues(g):
            a = acc.ctypes.data_as(D)
            if kind == 11:
                self.L.orc_boundary_force(pos.ctypes.data_as(D), _d(g["box"]), len(idx), _i(idx), _d(c), a)
            elif kind == 15:
                self.L.orc_floating_base_force(pos.ctypes.data_as(D), typ.ctypes.data_as(I), len(idx), _i(idx),
                                               _d(c), a)
            elif kind == 16:
                self.L.orc_ztorque_force(pos.ctypes.data_as(D), _d(g["box"]), len(idx) // 3, _i(idx), _d(c), a)
            elif kind == 19:
                self.L.orc_ball_force(pos.ctypes.data_as(D), _d(g["box"]), len(idx) // 2, _i(idx), _d(c), a)
            else:
                self.L.orc_zpower_force(pos.ctypes.data_as(D), len(idx) // 2, _i(idx), _d(c), a)
        return acc

    @staticmethod
    def _field_residues(g):
        """External-field terms (kind, first, second; 8 constants each) back
        into residue calls: runs of one kind, with the index lists and
        constants the oracle's residue functions take (FLOATING_BASE: 6 per
        type, slot 0 starting with the potential's z offset; ZTORQUE: one
        one-bond chain {l, 1, 3} per term; ZPOWERPOTENTIAL: {k, 1} per term;
        BALL: the residue's bonds)."""
        f = g.get("fields")
        if f is None or len(f) == 0:
            return []
        f = np.asarray(f)
        fc = np.asarray(g["field_consts"])
        typ = np.asarray(g["type"])
        nT = int(g["n_types"])
        out, k0 = [], 0
        for k in range(1, len(f) + 1):
            if k < len(f) and f[k, 0] == f[k0, 0]:
                continue
            kind, run, cs = int(f[k0, 0]), f[k0:k], fc[k0:k]
            if kind == 11:
                idx, c = run[:, 1], cs[0, :4]
            elif kind == 15:
                idx = run[:, 1]
                c = np.zeros(6 * nT)
                for t, cc in zip(run[:, 1], cs):
                    c[6 * typ[t]:6 * typ[t] + 6] = cc[:6]
                c[0] = cs[0, 6]
            elif kind == 16:
                idx, c = np.stack([run[:, 1], np.ones(len(run), int), np.full(len(run), 3)], 1).ravel(), cs[0, :4]
            elif kind == 19:  # bonds {own first (constant 2), second}
                idx, c = np.stack([cs[:, 2].astype(int), run[:, 2]], 1).ravel(), cs[0, :2]
            else:
                idx, c = np.stack([run[:, 1], np.ones(len(run), int)], 1).ravel(), cs[0, :2]
            out.append((kind, np.ascontiguousarray(idx, np.int32), np.ascontiguousarray(c, np.float64)))
            k0 = k
        return out

    @staticmethod
    def _residues(g, kind):
        """BOND / BEND terms grouped into residues (runs of equal constants),
        in the order the .mpd lists them, as Blob::do*Force visits them."""
        lst = g.get(kind + "s")
        if lst is None or len(lst) == 0:
            return []
        cs = np.asarray(g[kind + "_consts"])
        out, k0 = [], 0
        for k in range(1, len(lst) + 1):
            if k == len(lst) or not np.array_equal(cs[k], cs[k0]):
                out.append((np.ascontiguousarray(lst[k0:k], np.int32), np.ascontiguousarray(cs[k0])))
                k0 = k
        return out

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
        for kind in ("bond", "bend"):
            for lst, c in self._residues(g, kind):
                a = (pos.ctypes.data_as(D), _d(g["box"]), len(lst), _i(lst), _d(c))
                bonded += (getattr(self.L, f"orc_{kind}_potential")(*a) if scale is None else
                           getattr(self.L, f"orc_{kind}_dpotential")(*a, _d(scale)))
        if scale is None:  # the external fields have no size-change term in the reference
            for kind, idx, c in self._field_residues(g):
                if kind == 11:
                    bonded += self.L.orc_boundary_potential(pos.ctypes.data_as(D), _d(g["box"]), len(idx), _i(idx),
                                                            _d(c))
                elif kind == 15:
                    bonded += self.L.orc_floating_base_potential(pos.ctypes.data_as(D), typ.ctypes.data_as(I),
                                                                 len(idx), _i(idx), _d(c))
                elif kind == 16:
                    bonded += self.L.orc_ztorque_potential(pos.ctypes.data_as(D), _d(g["box"]), len(idx) // 3,
                                                           _i(idx), _d(c))
                elif kind == 19:
                    bonded += self.L.orc_ball_potential(pos.ctypes.data_as(D), _d(g["box"]), len(idx) // 2,
                                                        _i(idx), _d(c))
                else:
                    bonded += self.L.orc_zpower_potential(pos.ctypes.data_as(D), len(idx) // 2, _i(idx), _d(c))
        bead = 0.0
        si = g.get("sphere_index")
        if si is not None and len(si):
            a = (len(pos), pos.ctypes.data_as(D), typ.ctypes.data_as(I), _d(g["box"]), nT, len(si), _i(si),
                 _d(g["sphere_consts"]))
            bead = self.L.orc_bead_potential(*a) if scale is None else self.L.orc_bead_dpotential(*a, _d(scale))
        ci = g.get("core_index")
        if ci is not None and len(ci) and scale is None:  # the reference drops its size-change term
            bead += self.L.orc_nanocore_potential(len(pos), pos.ctypes.data_as(D), _d(g["box"]), len(ci), _i(ci),
                                                  _d(np.ascontiguousarray(g["core_consts"]).ravel()))
        return pair, bonded, bead


def load():
    return Oracle()
