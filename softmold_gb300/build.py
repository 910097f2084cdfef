"""Build recipe for the GB300 library, the `MD` executable and the oracle.

Products (all git-ignored, rebuilt on each machine):
  softmold_gb300/_build/libsoftmold_gb300.so   CUDA sm_103a kernels + C ABI
  softmold_gb300/_build/MD                     drop-in `MD <name>` executable
  oracle/_build/libsmd_oracle.so, md_oracle    CPU oracle (test infrastructure)
  oracle/_ref/*                                reference tools, only where the
                                               reference sources are present
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_OUT = os.path.join(ORACLE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SRC = ["mpd_io.cpp", "mpd_desc.cpp", "observables.cpp", "synth.cpp", "md_driver.cpp", "abi_host.cpp"]
CU_SRC = ["smd_api.cu", "smd_static.cu"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _run(cmd, cwd=ROOT):
    p = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "softmold_gb300.h"))
    return files


def build_library(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, "libsoftmold_gb300.so")
    exe = os.path.join(OUT, "MD")
    deps = _deps()
    if not force and _newer(lib, deps) and _newer(exe, deps + [lib]):
        return lib
    nvcc = _nvcc()
    jobs = []
    objs = []
    for f in CU_SRC:
        o = os.path.join(OUT, f + ".o")
        objs.append(o)
        jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-warn-spills", "-c", os.path.join(CSRC, f), "-o", o])
    for f in HOST_SRC:
        o = os.path.join(OUT, f + ".o")
        objs.append(o)
        jobs.append(["g++", *CXXFLAGS, "-c", os.path.join(CSRC, f), "-o", o])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(_run, jobs))
    _run([nvcc, *ARCH, "-shared", "-o", lib, *objs])
    _run(["g++", "-O2", "-std=c++17", os.path.join(CSRC, "md_main.cpp"), "-o", exe,
          "-L" + OUT, "-lsoftmold_gb300", "-Wl,-rpath," + OUT])
    return lib


def build_oracle(force: bool = False) -> str:
    """CPU oracle (test infrastructure): restated reference step + MD driver."""
    os.makedirs(ORACLE_OUT, exist_ok=True)
    lib = os.path.join(ORACLE_OUT, "libsmd_oracle.so")
    exe = os.path.join(ORACLE_OUT, "md_oracle")
    srcs = [os.path.join(ORACLE, "smd_oracle.cpp"), os.path.join(ORACLE, "md_oracle.cpp"),
            os.path.join(CSRC, "mpd_io.cpp"), os.path.join(CSRC, "observables.cpp")]
    deps = srcs + [os.path.join(ORACLE, "smd_oracle.h"), os.path.join(ORACLE, "md_oracle_main.cpp"),
                   os.path.join(CSRC, "mpd_io.h"), os.path.join(CSRC, "observables.h")]
    if not force and _newer(lib, deps) and _newer(exe, deps):
        return lib
    flags = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off"]
    jobs = [["g++", *flags, "-shared", *srcs, "-o", lib],
            ["g++", *flags, *srcs, os.path.join(ORACLE, "md_oracle_main.cpp"), "-o", exe]]
    with ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, jobs))
    return lib


def reference_root(ref_root: str | None = None) -> str | None:
    """The reference checkout: the argument, else $SMD_REFERENCE_ROOT, else a
    directory named `reference` beside this repository; None when none of
    them holds the reference's MD.cpp."""
    for cand in (ref_root, os.environ.get("SMD_REFERENCE_ROOT"), os.path.join(os.path.dirname(ROOT), "reference")):
        if cand and os.path.exists(os.path.join(cand, "MD.cpp")):
            return cand
    return None


def build_reference_tools(ref_root: str | None = None) -> bool:
    """Compiles the reference's own tools into oracle/_ref (only where present)."""
    root = reference_root(ref_root)
    if root is None:
        return False
    _run(["bash", os.path.join(ORACLE, "build_ref.sh"), root])
    return True


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, force)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", os.path.join(OUT, "libsoftmold_gb300.so"))
