"""Post-processing observables of the reference's analysis tools, restated for
the statistical parity checks.  Test infrastructure: only tests import it.

structure_factor_frames restates analysis/structureFactorFrames.cpp (the
height-fluctuation spectrum of a membrane from its frames_ and size_ files).
That tool links FFTW, which this image does not have, so the restatement is
checked against a direct discrete Fourier sum and an analytic mode instead of
against the tool's own output.

width_frames restates analysis/avgThicknessFrames.cpp (the membrane's width
along one axis: the standard deviation of the selected beads' coordinate in
columns of the other two axes, averaged over the columns and the frames).
The tool's column index is broken as written (avgThicknessFrames.cpp:149-150
assigns the x index twice, from the raw coordinate, and leaves the y index
uninitialised, so its output is undefined), and its column count along the
second axis is taken from the first axis's length (:134-135).  The
restatement keeps the second quirk and computes the column index the tool
evidently intends, floor(coordinate / column side); it is checked against a
hand-worked case instead of the tool's output.
"""
from __future__ import annotations

import numpy as np


def read_frames(path):
    """frames_<name>.xyz as a list of (types, xyz) arrays
    (include/fileFormats/xyzFormat.h: `N`, a comment line, `type x y z` lines)."""
    lines = open(path).read().split("\n")
    out = []
    k = 0
    while k < len(lines) and lines[k].strip():
        n = int(lines[k])
        a = np.array([ln.split() for ln in lines[k + 2:k + 2 + n]], dtype=float)
        out.append((a[:, 0].astype(int), a[:, 1:4]))
        k += n + 2
    return out


def read_sizes(path):
    """size_<name>.dat rows (time, Lx, Ly, Lz)."""
    return np.loadtxt(path, ndmin=2)


def frame_sizes(sizes, n_frames, store_interval):
    """The clock and box of each frame, read as structureFactorFrames.cpp:52-64,
    89-99 reads them: the first row with a non-negative time starts the clock
    and is consumed; for each frame the tool reads on (from a time of 0) while
    the last time read is below the clock, keeps the last row read, and then
    advances the clock by the store interval.  Rows past the end keep the last
    box."""
    times = np.empty(n_frames)
    boxes = np.empty((n_frames, 3))
    row = 0
    while row < len(sizes) - 1 and sizes[row, 0] < 0:
        row += 1
    t = sizes[row, 0]
    cur = sizes[row, 1:4]
    row += 1
    for f in range(n_frames):
        s_time = 0.0
        while s_time < t and row < len(sizes):
            s_time = sizes[row, 0]
            cur = sizes[row, 1:4]
            row += 1
        times[f] = t
        boxes[f] = cur
        t += store_interval
    return times, boxes


def frame_spectrum(types, xyz, box, nx, ny, select):
    """One frame of structureFactorFrames.cpp:100-180: the mean z of the
    selected beads per (x, y) grid cell less the selection's mean z, its 2-D
    forward DFT (unnormalised, as FFTW_FORWARD), and |h(q)|^2 (rx ry)/(Lx Ly)
    averaged over rings of integer |q| index.  Returns the ring sums' averages
    for ring 1 .. nx/2 - 1 and their counts."""
    rx, ry = box[0] / nx, box[1] / ny
    keep = np.isin(types, select)
    p = xyz[keep]
    cx = np.minimum(np.floor(p[:, 0] / rx).astype(int), nx - 1)
    cy = np.minimum(np.floor(p[:, 1] / ry).astype(int), ny - 1)
    h = np.zeros(nx * ny)
    cnt = np.zeros(nx * ny)
    np.add.at(h, cx + cy * nx, p[:, 2])
    np.add.at(cnt, cx + cy * nx, 1.0)
    avg_z = p[:, 2].mean() if len(p) else 0.0
    filled = cnt != 0
    h[filled] = h[filled] / cnt[filled] - avg_z
    # FFTW's dft_2d(nx, ny) reads the buffer row-major as [nx][ny]
    H = np.fft.fft2(h.reshape(nx, ny)).ravel()
    power = (H.real ** 2 + H.imag ** 2) * (rx * ry) / (box[0] * box[1])
    j = np.arange(nx * ny)
    ix = j % nx
    iy = j // ny
    ix = np.where(ix >= nx // 2, nx - ix, ix)
    iy = np.where(iy >= ny // 2, ny - iy, iy)
    qq = np.sqrt((ix * ix + iy * iy).astype(float)).astype(int)
    sf = np.bincount(qq, weights=power, minlength=nx + 1)[:nx]
    count = np.bincount(qq, minlength=nx + 1)[:nx].astype(float)
    rings = np.arange(1, nx // 2)
    return np.where(count[rings] != 0, sf[rings] / np.maximum(count[rings], 1), 0.0)


def structure_factor_frames(frames_path, size_path, store_interval, from_time, nx, ny, select):
    """structureFactorFrames.cpp as a whole, per frame: returns (q, per-frame
    spectra [frames x rings]).  The tool prints q and the mean over frames."""
    frames = read_frames(frames_path)
    times, boxes = frame_sizes(read_sizes(size_path), len(frames), store_interval)
    spectra, lx = [], []
    for (types, xyz), t, box in zip(frames, times, boxes):
        if t >= from_time:
            spectra.append(frame_spectrum(types, xyz, box, nx, ny, select))
            lx.append(box[0])
    q = np.arange(1, nx // 2) * 2.0 * np.pi / np.mean(lx)
    return q, np.array(spectra)


def frame_width(types, xyz, box, dimension, cutoff, select):
    """One frame of avgThicknessFrames.cpp:127-170: columns of side
    (Lx / int(Lx / cutoff), Ly / int(Lx / cutoff)) over the two axes after
    `dimension`; in each column the selected beads' mean and mean square of
    coordinate `dimension`; the square root of their difference summed over
    the columns (0 for an empty one) and divided by the number of non-empty
    columns."""
    a1, a2 = (dimension + 1) % 3, (dimension + 2) % 3
    nsx = int(box[0] / cutoff)
    nsy = int(box[0] / cutoff)  # the tool's ns.y comes from size.x
    csx, csy = box[0] / nsx, box[1] / nsy
    keep = np.isin(types, select)
    p = xyz[keep]
    cx = np.minimum(np.floor(p[:, a1] / csx).astype(int), nsx - 1)
    cy = np.minimum(np.floor(p[:, a2] / csy).astype(int), nsy - 1)
    cell = cx + cy * nsx
    cnt = np.bincount(cell, minlength=nsx * nsy).astype(float)
    s1 = np.bincount(cell, weights=p[:, dimension], minlength=nsx * nsy)
    s2 = np.bincount(cell, weights=p[:, dimension] ** 2, minlength=nsx * nsy)
    filled = cnt != 0
    avg = s1[filled] / cnt[filled]
    avg2 = s2[filled] / cnt[filled]
    total = np.sqrt(avg2 - avg * avg).sum()
    return total / filled.sum() if filled.any() else 0.0


def width_frames(frames_path, size_path, store_interval, from_time, dimension, cutoff, select):
    """avgThicknessFrames.cpp as a whole: per-frame widths from `from_time` on
    (the tool prints their mean and population standard deviation); frames
    and boxes are paired as structureFactorFrames pairs them (:87-124)."""
    frames = read_frames(frames_path)
    times, boxes = frame_sizes(read_sizes(size_path), len(frames), store_interval)
    return np.array([frame_width(types, xyz, box, dimension, cutoff, select)
                     for (types, xyz), t, box in zip(frames, times, boxes) if t >= from_time])
