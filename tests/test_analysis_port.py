"""The restatement of analysis/structureFactorFrames.cpp used by the
statistical parity checks: its arithmetic against an analytic mode and a
direct Fourier sum, and its frame/size pairing against a hand-worked case."""
import numpy as np
from analysis_obs import frame_sizes, frame_spectrum


def _ring_count(n, m):
    """Grid entries of ring m under the tool's fold (index >= n/2 -> n - index)."""
    c = 0
    for j in range(n * n):
        ix, iy = j % n, j // n
        ix = n - ix if ix >= n // 2 else ix
        iy = n - iy if iy >= n // 2 else iy
        c += int(np.sqrt(ix * ix + iy * iy)) == m
    return c


def _cell_centres(n, box):
    cx, cy = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    x = (cx.ravel() + 0.5) * box[0] / n
    y = (cy.ravel() + 0.5) * box[1] / n
    return x, y


def test_cosine_mode_lands_in_its_ring():
    """z = A cos(2 pi m x / Lx), one bead per cell: the two +-m coefficients
    have |H| = A nx ny / 2, so ring m holds A^2 nx ny / 2 over its entries."""
    n, m, A = 16, 3, 0.7
    box = np.array([20.0, 20.0, 30.0])
    x, y = _cell_centres(n, box)
    z = 15.0 + A * np.cos(2 * np.pi * m * x / box[0])
    xyz = np.stack([x, y, z], 1)
    sf = frame_spectrum(np.full(len(x), 2), xyz, box, n, n, [2])
    want = A * A * n * n / 2 / _ring_count(n, m)
    assert np.isclose(sf[m - 1], want, rtol=1e-12)
    others = np.delete(sf, m - 1)
    assert np.abs(others).max() < 1e-20 * want + 1e-24


def test_spectrum_equals_direct_fourier_sum():
    rng = np.random.default_rng(5)
    n = 8
    box = np.array([9.0, 9.0, 20.0])
    x, y = _cell_centres(n, box)
    # two beads of the selected type per cell and one of another type
    xyz = np.concatenate([np.stack([x, y, rng.normal(10, 0.3, len(x))], 1),
                          np.stack([x, y, rng.normal(10, 0.3, len(x))], 1),
                          np.stack([x, y, rng.normal(10, 3.0, len(x))], 1)])
    types = np.array([2] * (2 * len(x)) + [3] * len(x))
    sf = frame_spectrum(types, xyz, box, n, n, [2])
    # the height map by hand, laid out as the tool's hash c.x + c.y n
    sel = xyz[types == 2]
    h = np.zeros(n * n)
    for cx in range(n):
        for cy in range(n):
            inside = (np.floor(sel[:, 0] / (box[0] / n)) == cx) & (np.floor(sel[:, 1] / (box[1] / n)) == cy)
            h[cx + cy * n] = sel[inside, 2].mean() - sel[:, 2].mean()
    g = h.reshape(n, n)  # read as [nx][ny]
    power = np.zeros(n * n)
    for k1 in range(n):
        for k2 in range(n):
            s = sum(g[a, b] * np.exp(-2j * np.pi * (k1 * a / n + k2 * b / n)) for a in range(n) for b in range(n))
            power[k1 * n + k2] = abs(s) ** 2 * (box[0] / n) * (box[1] / n) / (box[0] * box[1])
    for m in range(1, n // 2):
        tot = 0.0
        for j in range(n * n):
            ix, iy = j % n, j // n
            ix = n - ix if ix >= n // 2 else ix
            iy = n - iy if iy >= n // 2 else iy
            if int(np.sqrt(ix * ix + iy * iy)) == m:
                tot += power[j]
        assert np.isclose(sf[m - 1], tot / _ring_count(n, m), rtol=1e-10)


def test_frame_size_pairing():
    """Sizes measured every 0.5 from t = 0.5, frames stored every 1: the
    clock starts at 0.5 (that row consumed); frame 0 then reads on to 1.0,
    frame 1 (clock 1.5) to 1.5, frame 2 (clock 2.5) to 2.5, frame 3 past the
    end keeps the last row."""
    sizes = np.array([[0.5, 10, 10, 5], [1.0, 11, 11, 5], [1.5, 12, 12, 5], [2.0, 13, 13, 5],
                      [2.5, 14, 14, 5]], float)
    t, b = frame_sizes(sizes, 4, 1.0)
    assert np.allclose(t, [0.5, 1.5, 2.5, 3.5])
    assert np.allclose(b[:, 0], [11, 12, 14, 14])


def test_width_of_two_flat_leaflets():
    """Heads of two flat leaflets at z0 +- h in every column: each column's
    standard deviation is h (equal counts), whatever the column grid."""
    from analysis_obs import frame_width
    rng = np.random.default_rng(1)
    box = np.array([20.0, 20.0, 30.0])
    n = 2000
    x = rng.uniform(0, box[0], n)
    y = rng.uniform(0, box[1], n)
    z = np.where(np.arange(n) % 2 == 0, 15.0 + 2.5, 15.0 - 2.5)
    types = np.full(n, 2)
    xyz = np.stack([x, y, z], 1)
    # pair each upper head with a lower one in the same column
    xyz[1::2, :2] = xyz[0::2, :2]
    w = frame_width(types, xyz, box, 2, 2.0, [2])
    assert abs(w - 2.5) < 1e-9
    # other types are ignored; along x the same beads have a uniform spread
    types2 = types.copy()
    types2[:10] = 3
    assert frame_width(types2, xyz, box, 2, 2.0, [3]) > 0.0
    wx = frame_width(types, xyz, box, 0, 4.0, [2])
    assert 0.0 < wx < box[0] / np.sqrt(12.0) + 1e-9


def test_width_columns_follow_the_tools_quirk():
    """The second axis takes its column count from the first axis's length:
    a 20 x 10 box with cutoff 2 has 10 x 10 columns of 2 x 1."""
    from analysis_obs import frame_width
    box = np.array([20.0, 10.0, 30.0])
    # one column holds beads at y 0.2 and 0.7 (same 1-wide column) with z 10, 12
    xyz = np.array([[1.0, 0.2, 10.0], [1.0, 0.7, 12.0], [1.0, 1.2, 20.0]])
    types = np.array([2, 2, 2])
    # columns: (0, 0) holds two beads (std 1), (0, 1) one bead (std 0)
    assert abs(frame_width(types, xyz, box, 2, 2.0, [2]) - 0.5) < 1e-12
