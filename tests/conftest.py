import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library)")


@pytest.fixture(scope="session")
def built():
    """Builds the CUDA library (nvcc cross-compiles without a GPU) and the oracle."""
    from softmold_gb300 import build
    build.build_all()
    return True


@pytest.fixture(scope="session")
def oracle(built):
    import oracle_binding
    return oracle_binding.load()


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(params=["ves300", "bil400"])
def golden_case(request):
    return request.param, load_golden(request.param)


def mpd_from_golden(g):
    """softmold_gb300.Mpd view of a golden case."""
    import softmold_gb300 as smd
    return smd.Mpd(n_types=int(g["n_types"]), pos=g["pos"], vel=g["vel"], type=g["type"].astype(np.int32),
                   box=g["box"], cutoff=float(g["cutoff"]), fconst=g["fconst"], uconst=g["uconst"],
                   chain_blocks=g["chain_blocks"].astype(np.int32), chain_consts=g["chain_consts"],
                   dt=float(g["dt"]), gamma=float(g["gamma"]), temperature=float(g["temperature"]),
                   seed=int(g["seed"]), tension=float(g["tension"]), delta_lxy=float(g["delta_lxy"]),
                   initial_time=0.0, final_time=1.0,
                   sphere_index=g["sphere_index"].astype(np.int32) if len(g.get("sphere_index", [])) else None,
                   sphere_consts=g["sphere_consts"] if len(g.get("sphere_index", [])) else None,
                   bonds=g["bonds"].astype(np.int32) if len(g.get("bonds", [])) else None,
                   bond_consts=g["bond_consts"] if len(g.get("bonds", [])) else None,
                   bends=g["bends"].astype(np.int32) if len(g.get("bends", [])) else None,
                   bend_consts=g["bend_consts"] if len(g.get("bends", [])) else None,
                   fields=g["fields"].astype(np.int32) if len(g.get("fields", [])) else None,
                   field_consts=g["field_consts"] if len(g.get("fields", [])) else None,
                   core_index=g["core_index"].astype(np.int32) if len(g.get("core_index", [])) else None,
                   core_consts=g["core_consts"] if len(g.get("core_index", [])) else None)
