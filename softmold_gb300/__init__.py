"""softmold_gb300: GB300 implicit-solvent membrane MD step behind a C ABI.

This module is a thin ctypes mirror of include/softmold_gb300.h for tests,
benchmarks and scripting.  The compute path is the CUDA library
``_build/libsoftmold_gb300.so``; there is no CPU fallback: every call that
needs the device raises when the library or the GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "_build", "libsoftmold_gb300.so")
MD_EXE = os.path.join(PKG, "_build", "MD")
HEADER = os.path.join(ROOT, "include", "softmold_gb300.h")

PLAIN_FP64 = 0
MIXED = 1


class SmdError(RuntimeError):
    pass


class SystemDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("n_types", C.c_int),
        ("pos", C.POINTER(C.c_double)), ("vel", C.POINTER(C.c_double)), ("type", C.POINTER(C.c_int)),
        ("box", C.c_double * 3), ("cutoff", C.c_double),
        ("fconst", C.POINTER(C.c_double)), ("uconst", C.POINTER(C.c_double)),
        ("n_chain_blocks", C.c_int), ("chain_blocks", C.POINTER(C.c_int)),
        ("chain_consts", C.POINTER(C.c_double)),
        ("n_spheres", C.c_int), ("sphere_index", C.POINTER(C.c_int)),
        ("sphere_consts", C.POINTER(C.c_double)),
        ("dt", C.c_double), ("gamma", C.c_double), ("temperature", C.c_double),
        ("seed", C.c_uint32), ("tension", C.c_double), ("delta_lxy", C.c_double),
        ("resize_rate", C.c_int), ("first_step", C.c_int), ("skin", C.c_double),
        ("n_bonds", C.c_int), ("bonds", C.POINTER(C.c_int)), ("bond_consts", C.POINTER(C.c_double)),
        ("n_bends", C.c_int), ("bends", C.POINTER(C.c_int)), ("bend_consts", C.POINTER(C.c_double)),
        ("n_fields", C.c_int), ("fields", C.POINTER(C.c_int)), ("field_consts", C.POINTER(C.c_double)),
        ("sphere_nanocore", C.c_int),
    ]


class Energy(C.Structure):
    _fields_ = [("pair", C.c_double), ("bonded", C.c_double), ("sphere", C.c_double), ("kinetic", C.c_double)]


class Measurement(C.Structure):
    _fields_ = [("kinetic", C.c_double), ("lo", C.c_double * 3), ("hi", C.c_double * 3),
                ("bond_length_sum", C.c_double), ("n_bond", C.c_int),
                ("bend_cos_sum", C.c_double), ("bend_len0_sum", C.c_double), ("bend_len1_sum", C.c_double),
                ("n_bend", C.c_int), ("msd", C.c_int)]


class McStats(C.Structure):
    _fields_ = [("trials", C.c_long), ("accepted", C.c_long), ("last_dU", C.c_double)]


_lib = None

class AdjointSpec(C.Structure):
    _fields_ = [("steps", C.c_int), ("checkpoint_every", C.c_int), ("umin_types", C.c_int * 2),
                ("segment_local", C.c_int)]


class AdjointResult(C.Structure):
    _fields_ = [("mean_potential", C.c_double), ("grad", C.c_double * 3), ("mean_area_per_lipid", C.c_double),
                ("grad_area", C.c_double * 3)]


# name -> (restype, argtypes); every function declared in the header
_SIGS = {
    "smd_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "smd_device_count": (C.c_int, []),
    "smd_create": (C.c_int, [C.POINTER(SystemDesc), C.c_int, C.POINTER(C.c_void_p)]),
    "smd_create_batch": (C.c_int, [C.POINTER(SystemDesc), C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "smd_destroy": (None, [C.c_void_p]),
    "smd_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "smd_get_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "smd_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "smd_get_box": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "smd_set_box": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "smd_compute_forces": (C.c_int, [C.c_void_p, C.c_void_p]),
    "smd_compute_pair_forces": (C.c_int, [C.c_void_p, C.c_void_p]),
    "smd_compute_energy": (C.c_int, [C.c_void_p, C.c_void_p]),
    "smd_compute_dU": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "smd_cell_keys": (C.c_int, [C.c_void_p, C.c_void_p]),
    "smd_pair_list": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "smd_prepare": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "smd_advance": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "smd_mc_stats_get": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "smd_mc_log": (C.c_long, [C.c_void_p, C.c_int, C.c_long, C.c_long, C.c_void_p, C.c_void_p]),
    "smd_set_temperature": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int]),
    "smd_set_noise_once": (C.c_int, [C.c_void_p, C.c_void_p]),
    "smd_last_timing": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "smd_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "smd_sync": (C.c_int, [C.c_void_p]),
    "smd_use_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "smd_autotune": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "smd_set_tuning": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "smd_adjoint": (C.c_int, [C.c_void_p, C.POINTER(AdjointSpec), C.POINTER(AdjointResult)]),
    "smd_hessian_vector": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "smd_mpd_update_state": (C.c_int, [C.c_char_p, C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
    "smd_rebuild_count": (C.c_long, [C.c_void_p]),
    "smd_list_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "smd_synth_vesicle": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_double]),
    "smd_synth_bilayer": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                    C.c_double]),
    "smd_synth_vesicle_sphere": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                           C.c_double, C.c_double, C.c_double]),
    "smd_md_main": (C.c_int, [C.c_char_p, C.c_int]),
    "smd_pair_forces_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_int,
                                         C.c_void_p, C.c_void_p, C.c_void_p]),
    "smd_mpd_load": (C.c_int, [C.c_char_p, C.POINTER(SystemDesc), C.c_void_p, C.POINTER(C.c_void_p)]),
    "smd_mpd_free": (None, [C.c_void_p]),
    "smd_measure": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "smd_ke_histogram": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "smd_start_diffusion": (C.c_int, [C.c_void_p]),
    "smd_set_msd_groups": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
}


def declared_symbols() -> list[str]:
    """Function names declared in include/softmold_gb300.h."""
    import re
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|long|void)\s+\*?\s*(smd_\w+)\s*\(", text, re.M)))


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SmdError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(2048)
    lib().smd_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def _check(rc, what):
    if rc != 0:
        raise SmdError(f"{what} failed ({rc}): {last_error()}")


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


@dataclass
class Mpd:
    """The hot-path fields of an .mpd file."""
    n_types: int
    pos: np.ndarray          # (n,3)
    vel: np.ndarray          # (n,3)
    type: np.ndarray         # (n,)
    box: np.ndarray          # (3,)
    cutoff: float
    fconst: np.ndarray
    uconst: np.ndarray
    chain_blocks: np.ndarray  # (k,3)
    chain_consts: np.ndarray  # (k,4)
    dt: float
    gamma: float
    temperature: float
    seed: int
    tension: float
    delta_lxy: float
    initial_time: float
    final_time: float
    sphere_index: np.ndarray | None = None
    sphere_consts: np.ndarray | None = None
    bonds: np.ndarray | None = None        # (k,2) BOND residue terms
    bond_consts: np.ndarray | None = None  # (k,2) l0, k per term
    bends: np.ndarray | None = None        # (k,3) BEND residue terms
    bend_consts: np.ndarray | None = None  # (k,2) a, k per term
    # external-field residues as terms: (kind, first, second) with kind the
    # .mpd molecule type (11 BOUNDARY, 15 FLOATING_BASE, 16 ZTORQUE, 17
    # ZPOWERPOTENTIAL, 19 BALL) and second = -1 for one-bead terms; 8
    # constants each
    fields: np.ndarray | None = None        # (k,3)
    field_consts: np.ndarray | None = None  # (k,8)
    # NANOCORE residue: core bead indices and 22 constants per core
    core_index: np.ndarray | None = None    # (k,)
    core_consts: np.ndarray | None = None   # (k,22)


class MpdRun(C.Structure):
    _fields_ = [("initial_time", C.c_double), ("final_time", C.c_double), ("store_interval", C.c_double),
                ("measure_interval", C.c_double), ("initial_temp", C.c_double), ("final_temp", C.c_double),
                ("temp_step_interval", C.c_double), ("n_bead_residues", C.c_int), ("per_type_gamma", C.c_int)]


def read_mpd(path: str) -> Mpd:
    """Reads an .mpd through the library's reader and residue expansion
    (smd_mpd_load: Blob::input, include/system.h:589-1314, expanded into the
    terms the device step takes exactly as the `MD` executable does)."""
    d = SystemDesc()
    run = MpdRun()
    owner = C.c_void_p()
    _check(lib().smd_mpd_load(path.encode(), C.byref(d), C.byref(run), C.byref(owner)), f"smd_mpd_load({path})")
    try:
        n, nT = d.n, d.n_types

        def arr(ptr, count, dtype, shape=None):
            if count <= 0 or not ptr:
                return np.zeros(shape if shape else (0,), dtype)
            a = np.ctypeslib.as_array(ptr, shape=(count,)).astype(dtype, copy=True)
            return a.reshape(shape) if shape else a

        sph = arr(d.sphere_index, d.n_spheres, np.int32) if d.n_spheres > 0 else None
        sph_c = None
        if d.n_spheres > 0:
            sph_c = arr(d.sphere_consts, 22 * (d.n_spheres if d.sphere_nanocore else nT * nT), np.float64)
        return Mpd(n_types=nT, pos=arr(d.pos, 3 * n, np.float64, (n, 3)), vel=arr(d.vel, 3 * n, np.float64, (n, 3)),
                   type=arr(d.type, n, np.int32), box=np.array(d.box[:]), cutoff=d.cutoff,
                   fconst=arr(d.fconst, 6 * nT * nT, np.float64), uconst=arr(d.uconst, 6 * nT * nT, np.float64),
                   chain_blocks=arr(d.chain_blocks, 3 * d.n_chain_blocks, np.int32, (d.n_chain_blocks, 3)),
                   chain_consts=arr(d.chain_consts, 4 * d.n_chain_blocks, np.float64, (d.n_chain_blocks, 4)),
                   dt=d.dt, gamma=d.gamma, temperature=d.temperature, seed=int(d.seed), tension=d.tension,
                   delta_lxy=d.delta_lxy, initial_time=run.initial_time, final_time=run.final_time,
                   sphere_index=None if d.sphere_nanocore else sph,
                   sphere_consts=None if d.sphere_nanocore else sph_c,
                   bonds=arr(d.bonds, 2 * d.n_bonds, np.int32, (d.n_bonds, 2)) if d.n_bonds else None,
                   bond_consts=arr(d.bond_consts, 2 * d.n_bonds, np.float64, (d.n_bonds, 2)) if d.n_bonds else None,
                   bends=arr(d.bends, 3 * d.n_bends, np.int32, (d.n_bends, 3)) if d.n_bends else None,
                   bend_consts=arr(d.bend_consts, 2 * d.n_bends, np.float64, (d.n_bends, 2)) if d.n_bends else None,
                   fields=arr(d.fields, 3 * d.n_fields, np.int32, (d.n_fields, 3)) if d.n_fields else None,
                   field_consts=arr(d.field_consts, 8 * d.n_fields, np.float64, (d.n_fields, 8)) if d.n_fields
                   else None,
                   core_index=sph if d.sphere_nanocore else None,
                   core_consts=sph_c.reshape(-1, 22) if d.sphere_nanocore else None)
    finally:
        lib().smd_mpd_free(owner)


class System:
    """One handle of the C ABI: one system or a batch of replicas."""

    def __init__(self, systems: Mpd | list[Mpd], precision: int = MIXED, skin: float = 0.5):
        systems = systems if isinstance(systems, list) else [systems]
        self._keep = []
        descs = (SystemDesc * len(systems))()
        for k, m in enumerate(systems):
            arrs = dict(pos=np.ascontiguousarray(m.pos, np.float64), vel=np.ascontiguousarray(m.vel, np.float64),
                        type=np.ascontiguousarray(m.type, np.int32), fc=np.ascontiguousarray(m.fconst, np.float64),
                        uc=np.ascontiguousarray(m.uconst, np.float64),
                        cb=np.ascontiguousarray(m.chain_blocks, np.int32),
                        cc=np.ascontiguousarray(m.chain_consts, np.float64))
            has_bead = m.sphere_index is not None and len(m.sphere_index) > 0
            has_core = m.core_index is not None and len(m.core_index) > 0
            if has_bead and has_core:
                raise SmdError("a BEAD and a NANOCORE residue in one system are not supported on the GPU step")
            if has_bead:
                arrs["si"] = np.ascontiguousarray(m.sphere_index, np.int32)
                arrs["sc"] = np.ascontiguousarray(m.sphere_consts, np.float64)
            elif has_core:
                arrs["si"] = np.ascontiguousarray(m.core_index, np.int32)
                arrs["sc"] = np.ascontiguousarray(np.asarray(m.core_consts, np.float64).ravel())
            self._keep.append(arrs)
            d = descs[k]
            d.n = len(m.type)
            d.n_types = m.n_types
            d.pos, d.vel, d.type = _dp(arrs["pos"]), _dp(arrs["vel"]), _ip(arrs["type"])
            for a in range(3):
                d.box[a] = float(m.box[a])
            d.cutoff = m.cutoff
            d.fconst, d.uconst = _dp(arrs["fc"]), _dp(arrs["uc"])
            d.n_chain_blocks = len(arrs["cb"])
            d.chain_blocks, d.chain_consts = _ip(arrs["cb"]), _dp(arrs["cc"])
            if "si" in arrs:
                d.n_spheres = len(arrs["si"])
                d.sphere_index, d.sphere_consts = _ip(arrs["si"]), _dp(arrs["sc"])
                d.sphere_nanocore = 1 if has_core else 0
            else:
                d.n_spheres = 0
            for key, lk, ck in (("bonds", "bl", "bc"), ("bends", "el", "ec")):
                lst = getattr(m, key, None)
                if lst is not None and len(lst) > 0:
                    arrs[lk] = np.ascontiguousarray(lst, np.int32)
                    arrs[ck] = np.ascontiguousarray(getattr(m, key[:-1] + "_consts"), np.float64)
            if "bl" in arrs:
                d.n_bonds, d.bonds, d.bond_consts = len(arrs["bl"]), _ip(arrs["bl"]), _dp(arrs["bc"])
            if "el" in arrs:
                d.n_bends, d.bends, d.bend_consts = len(arrs["el"]), _ip(arrs["el"]), _dp(arrs["ec"])
            if m.fields is not None and len(m.fields) > 0:
                arrs["fl"] = np.ascontiguousarray(m.fields, np.int32)
                arrs["fcs"] = np.ascontiguousarray(m.field_consts, np.float64)
                d.n_fields, d.fields, d.field_consts = len(arrs["fl"]), _ip(arrs["fl"]), _dp(arrs["fcs"])
            d.dt, d.gamma, d.temperature = m.dt, m.gamma, m.temperature
            d.seed = m.seed & 0xffffffff
            d.tension, d.delta_lxy = m.tension, m.delta_lxy
            d.resize_rate = 8
            d.first_step = int(m.initial_time / m.dt + 1e-7) if m.dt > 0 else 0  # the library refuses dt <= 0
            d.skin = skin
        h = C.c_void_p()
        _check(lib().smd_create_batch(descs, len(systems), precision, C.byref(h)), "smd_create_batch")
        self.h = h
        self.n = sum(len(m.type) for m in systems)
        self.n_rep = len(systems)
        self.precision = precision
        self._msd_groups = 0

    def close(self):
        if getattr(self, "h", None):
            lib().smd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def state(self, pos=None, vel=None):
        """Positions and velocities in input order, (n, 3) FP64.  `pos` / `vel`
        may be given as C-contiguous (n, 3) float64 arrays (pinned host memory
        for the fastest copy) to be filled in place."""
        p = np.empty((self.n, 3)) if pos is None else pos
        v = np.empty((self.n, 3)) if vel is None else vel
        for a in (p, v):
            if a.dtype != np.float64 or a.shape != (self.n, 3) or not a.flags.c_contiguous:
                raise ValueError("state buffers must be C-contiguous (n, 3) float64")
        _check(lib().smd_get_state(self.h, p.ctypes.data, v.ctypes.data), "smd_get_state")
        return p, v

    def _sized(self, a, size, what):
        """`a` as a C-contiguous float64 array of `size` values: the library
        reads exactly that many from the pointer it gets."""
        out = np.ascontiguousarray(a, np.float64)
        if out.size != size:
            raise ValueError(f"{what} must hold {size} values, got {out.size}")
        return out

    def set_state(self, pos=None, vel=None):
        pp = None if pos is None else self._sized(pos, 3 * self.n, "positions")
        vv = None if vel is None else self._sized(vel, 3 * self.n, "velocities")
        _check(lib().smd_set_state(self.h, None if pp is None else pp.ctypes.data,
                                   None if vv is None else vv.ctypes.data), "smd_set_state")

    def box(self, replica=0):
        b = np.zeros(3)
        _check(lib().smd_get_box(self.h, replica, b.ctypes.data), "smd_get_box")
        return b

    def set_box(self, box, replica=0):
        b = self._sized(box, 3, "box")
        _check(lib().smd_set_box(self.h, replica, b.ctypes.data), "smd_set_box")

    def forces(self, pair_only=False):
        f = np.zeros((self.n, 3))
        fn = lib().smd_compute_pair_forces if pair_only else lib().smd_compute_forces
        _check(fn(self.h, f.ctypes.data), "smd_compute_forces")
        return f

    def energy(self):
        e = (Energy * self.n_rep)()
        _check(lib().smd_compute_energy(self.h, e), "smd_compute_energy")
        return [dict(pair=x.pair, bonded=x.bonded, sphere=x.sphere, kinetic=x.kinetic) for x in e]

    def dU(self, scale):
        s = self._sized(scale, 3, "scale")
        out = np.zeros(self.n_rep)
        _check(lib().smd_compute_dU(self.h, s.ctypes.data, out.ctypes.data), "smd_compute_dU")
        return out

    def cell_keys(self):
        k = np.zeros(self.n, np.int32)
        _check(lib().smd_cell_keys(self.h, k.ctypes.data), "smd_cell_keys")
        return k

    def pair_list(self):
        cnt = C.c_size_t(0)
        _check(lib().smd_pair_list(self.h, None, 0, C.byref(cnt)), "smd_pair_list")
        out = np.zeros((max(cnt.value, 1), 2), np.int32)
        _check(lib().smd_pair_list(self.h, out.ctypes.data, cnt.value, C.byref(cnt)), "smd_pair_list")
        return out[:cnt.value]

    def prepare(self, do_second=False, energy=False):
        e = Energy()
        _check(lib().smd_prepare(self.h, 1 if do_second else 0, C.byref(e) if energy else None), "smd_prepare")
        return dict(pair=e.pair, bonded=e.bonded, sphere=e.sphere, kinetic=e.kinetic) if energy else None

    def advance(self, steps, stop_at_measure=False, asynchronous=False):
        flags = (1 if stop_at_measure else 0) | (2 if asynchronous else 0)
        _check(lib().smd_advance(self.h, int(steps), flags), "smd_advance")

    def sync(self):
        _check(lib().smd_sync(self.h), "smd_sync")

    def adjoint(self, steps, checkpoint_every=20, umin_types=(3, 3), segment_local=False):
        """smd_adjoint: J = mean potential over the next `steps` loop steps and
        dJ/d(Umin(a,b), kbond, kbend); the handle ends `steps` steps later."""
        spec = AdjointSpec(int(steps), int(checkpoint_every), (C.c_int * 2)(*umin_types),
                           1 if segment_local else 0)
        res = AdjointResult()
        _check(lib().smd_adjoint(self.h, C.byref(spec), C.byref(res)), "smd_adjoint")
        return dict(mean_potential=res.mean_potential, grad=np.array(res.grad[:]),
                    mean_area_per_lipid=res.mean_area_per_lipid, grad_area=np.array(res.grad_area[:]))

    def hessian_vector(self, w):
        ww = self._sized(w, 3 * self.n, "w")
        out = np.zeros((self.n, 3))
        _check(lib().smd_hessian_vector(self.h, ww.ctypes.data, out.ctypes.data), "smd_hessian_vector")
        return out

    def autotune(self, force=False):
        """smd_autotune: (lanes per bead, list kernel, [list ms x3, pair-pass ms x3])."""
        lanes, kern = C.c_int(0), C.c_int(0)
        ms = (C.c_float * 6)()
        _check(lib().smd_autotune(self.h, 1 if force else 0, C.byref(lanes), C.byref(kern), ms), "smd_autotune")
        return lanes.value, kern.value, list(ms)

    def set_tuning(self, lanes, list_kernel):
        _check(lib().smd_set_tuning(self.h, int(lanes), int(list_kernel)), "smd_set_tuning")

    def use_graphs(self, on=True):
        _check(lib().smd_use_graphs(self.h, 1 if on else 0), "smd_use_graphs")

    def profile(self, on=True):
        _check(lib().smd_profile(self.h, 1 if on else 0), "smd_profile")

    def timing(self):
        """(step-kernel ms, step-kernel launches, total launches)."""
        ms = C.c_double(0)
        k = C.c_long(0)
        n = C.c_long(0)
        _check(lib().smd_last_timing(self.h, C.byref(ms), C.byref(k), C.byref(n)), "smd_last_timing")
        return ms.value, k.value, n.value

    def set_noise_once(self, psi):
        p = self._sized(psi, 3 * self.n, "psi")
        _check(lib().smd_set_noise_once(self.h, p.ctypes.data), "smd_set_noise_once")

    def set_stream(self, stream_handle: int | None):
        _check(lib().smd_set_stream(self.h, C.c_void_p(stream_handle) if stream_handle else None),
               "smd_set_stream")

    def mc_stats(self, replica=0):
        s = McStats()
        _check(lib().smd_mc_stats_get(self.h, replica, C.byref(s)), "smd_mc_stats_get")
        return dict(trials=s.trials, accepted=s.accepted, last_dU=s.last_dU)

    def measure(self, n_groups=0):
        """smd_measure on a handle stopped at a measure step: the reductions
        of the .dat files as a dict (and 'msd_sum' per group while diffusion
        is tracked)."""
        m = Measurement()
        # the library writes one sum per group the handle holds
        msd = np.zeros(max(self._msd_groups, 1))
        _check(lib().smd_measure(self.h, C.byref(m), msd.ctypes.data if n_groups else None), "smd_measure")
        out = dict(kinetic=m.kinetic, lo=np.array(m.lo[:]), hi=np.array(m.hi[:]), bond_length_sum=m.bond_length_sum,
                   n_bond=m.n_bond, bend_cos_sum=m.bend_cos_sum, bend_len0_sum=m.bend_len0_sum,
                   bend_len1_sum=m.bend_len1_sum, n_bend=m.n_bend, msd=bool(m.msd))
        if m.msd:
            out["msd_sum"] = msd[:n_groups].copy()
        return out

    def ke_histogram(self):
        n = C.c_size_t(0)
        _check(lib().smd_ke_histogram(self.h, None, 0, C.byref(n)), "smd_ke_histogram")
        out = np.zeros(max(n.value, 1), np.int64)
        _check(lib().smd_ke_histogram(self.h, out.ctypes.data, n.value, C.byref(n)), "smd_ke_histogram")
        return out[:n.value]

    def start_diffusion(self):
        _check(lib().smd_start_diffusion(self.h), "smd_start_diffusion")

    def set_msd_groups(self, offsets, beads):
        o = np.ascontiguousarray(offsets, np.int32).ravel()
        b = np.ascontiguousarray(beads, np.int32).ravel()
        # the library reads offsets[-1] bead indices
        if len(o) < 1 or int(o[-1]) != len(b):
            raise ValueError("offsets must end at len(beads)")
        _check(lib().smd_set_msd_groups(self.h, len(o) - 1, o.ctypes.data, b.ctypes.data if len(b) else None),
               "smd_set_msd_groups")
        self._msd_groups = len(o) - 1

    def launches(self):
        return self.timing()[2]

    def rebuilds(self):
        return lib().smd_rebuild_count(self.h)

    def list_state(self):
        d = C.c_double(0)
        sl = C.c_double(0)
        _check(lib().smd_list_state(self.h, C.byref(d), C.byref(sl)), "smd_list_state")
        return d.value, sl.value


def mpd_update_state(in_path, out_path, pos, vel, box, time):
    """Rewrites in_path's state into out_path (smd_mpd_update_state); pos and
    vel hold the file's nParticles x 3 values, which the library reads."""
    import re
    with open(in_path) as f:
        got = re.search(r"(?:^|\s)nParticles\s+(\d+)", f.read())
    n3 = 3 * int(got.group(1)) if got else -1
    p = np.ascontiguousarray(pos, np.float64)
    v = np.ascontiguousarray(vel, np.float64)
    b = np.ascontiguousarray(box, np.float64)
    if p.size != n3 or v.size != n3 or b.size != 3:
        raise ValueError(f"positions and velocities must hold {n3} values (nParticles x 3) and box 3")
    _check(lib().smd_mpd_update_state(in_path.encode(), out_path.encode(), p.ctypes.data, v.ctypes.data,
                                      b.ctypes.data, float(time)), "smd_mpd_update_state")


def synth_vesicle(path, seed, n_lipids, density=3.45, box=400.0):
    _check(lib().smd_synth_vesicle(path.encode(), seed, n_lipids, density, box), "smd_synth_vesicle")


def synth_bilayer(path, seed, n_lipids, density=3.45, zsize=40.0, delta_lxy=0.01, tension=0.0):
    _check(lib().smd_synth_bilayer(path.encode(), seed, n_lipids, density, zsize, delta_lxy, tension),
           "smd_synth_bilayer")


def synth_vesicle_sphere(path, seed, n_lipids, density, box, radius=5.0, head_umin=-10.0, head_umax=10.0,
                         gap=2.0, other_umax=10.0):
    _check(lib().smd_synth_vesicle_sphere(path.encode(), seed, n_lipids, density, box, radius, head_umin,
                                          head_umax, gap, other_umax), "smd_synth_vesicle_sphere")
