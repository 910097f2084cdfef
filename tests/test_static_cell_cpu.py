"""Index safety of smd_pair_forces_static, checked on the CPU.

The allocation-free entry point takes raw device arrays from another
framework, so its kernels derive cell indices from values nobody has
checked.  The cell and type functions they use live in a header that plain
C++ compiles (softmold_gb300/csrc/smd_static_cell.h); this test compiles it
with g++ and checks that every input, including NaN, infinities and
coordinates far outside the box, gives a cell inside the grid, that the
reference's cell (include/algorithms/cellOpt.h:532-539) is kept for
coordinates in [0, L], and that non-finite coordinates and out-of-range
types are flagged.  No kernel runs: out-of-range values are never sent to
the GPU.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER_DIR = os.path.join(ROOT, "softmold_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include "smd_static_cell.h"
int main(int argc, char** argv) {
  // argv: n cs, then coordinates; prints "cell flags" per coordinate
  const int n = std::atoi(argv[1]);
  const double cs = std::strtod(argv[2], nullptr);
  for (int k = 3; k < argc; ++k) {
    int flags = 0;
    const int c = smd_static::cell_coord(std::strtod(argv[k], nullptr), cs, n, &flags);
    std::printf("%d %d\n", c, flags);
  }
  const int types[] = {-1, 0, 5, 6, 1 << 30};
  for (int t : types) std::printf("type %d %d\n", t, smd_static::type_ok(t, 6) ? 1 : 0);
  return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("static_cell")
    src = d / "drv.cpp"
    src.write_text(DRIVER)
    exe = d / "drv"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", HEADER_DIR, str(src), "-o", str(exe)],
                   check=True)
    return str(exe)


def _cells(driver, n, cs, values):
    out = subprocess.run([driver, str(n), repr(cs), *[repr(float(v)) for v in values]], check=True,
                         capture_output=True, text=True).stdout.split("\n")
    cells = [tuple(map(int, line.split())) for line in out if line and not line.startswith("type")]
    types = [tuple(map(int, line.split()[1:])) for line in out if line.startswith("type")]
    return cells, types


def test_every_coordinate_gives_a_cell_inside_the_grid(driver):
    n, L = 10, 20.0
    cs = L / n
    cases = {
        0.0: (0, 0), L: (n - 1, 0), 19.999: (n - 1, 0), -0.5: (0, 0), -3.0: (0, 0),
        L + cs: (n - 1, 0),  # the reference's x >= n -> n-1 fix-up alone would give n here
        L + 2.5 * cs: (n - 1, 0), 1e300: (n - 1, 0), -1e300: (0, 0),
        float("nan"): (0, 1), float("inf"): (0, 1), float("-inf"): (0, 1),
    }
    got, _ = _cells(driver, n, cs, list(cases))
    for (v, want), g in zip(cases.items(), got):
        assert g == want, (v, g, want)
        assert 0 <= g[0] < n


def test_reference_cell_kept_inside_the_box(driver):
    rng = np.random.default_rng(7)
    for n, L in ((3, 6.5), (10, 20.0), (38, 76.14), (95, 190.3)):
        cs = L / n
        xs = np.concatenate([rng.uniform(0.0, L, 400), [0.0, L, cs, 2 * cs, L - cs, np.nextafter(L, 0.0)]])
        got, _ = _cells(driver, n, cs, xs)
        for x, (c, flags) in zip(xs, got):
            q = int(x / cs)  # CellOpt::build: int(p/cellSize), then x >= n -> n-1
            q = q - 1 if q >= n else q
            assert (c, flags) == (q, 0), (x, c, q)


def test_out_of_range_types_are_flagged(driver):
    _, types = _cells(driver, 4, 1.0, [])
    assert dict(types) == {-1: 0, 0: 1, 5: 1, 6: 0, 1 << 30: 0}
