"""Patchy-saturation models and the raw float32 model-file format.

* ``reference_pattern(k)``: the six deterministic circle-packing layers of
  patchymodel.m (patchy:17-260): circles of radius r = 8 cells on a pitch of
  2r (or multiples) in a 240-row layer placed at rows 2001-2240 of a
  2800 x 5000 background; IDs 1 = background, 2 = inside a circle,
  3 = layer host (patchy:33-46).
* ``random_patches(...)``: seeded random circular gas patches with a target
  areal fraction (the patchy workloads of the benchmark configurations).
* ``write_bin`` / ``read_bin``: raw little-endian float32 grids as arr2bin.m
  writes them (arr2bin:4-14).  patchymodel.m reshapes column-major before
  calling arr2bin (patchy:50-51), so its files are z-fastest, while the
  solver's driver reads x-fastest (cu:685): ``order`` says which.
"""
from __future__ import annotations

import numpy as np

LINGX, LINGY, MODY, R = 5000, 240, 2800, 8     # patchy:4-8

# (start_x, step_x, start_y, step_y) of each circle lattice, in units of r and
# diameters, per pattern (patchy:17, 57, 92, 128-137, 172-181, 215-224)
_LATTICES = {
    1: [(1, 1, 1, 1)],
    2: [(1, 2, 1, 2)],
    3: [(1, 4, 1, 2)],
    4: [(1, 2, 1, 2), (3, 2, 3, 2)],
    5: [(1, 2, 3, 2), (1, 1, 1, 2)],
    6: [(1, 4, 1, 2), (5, 4, 3, 2)],
}


def _layer(pattern, lingx=LINGX, lingy=LINGY, r=R):
    """The 240 x 5000 patch layer of one pattern, IDs 2 (circle) / 3 (host)."""
    dia = 2 * r
    yy, xx = np.mgrid[1:lingy + 1, 1:lingx + 1]          # meshgrid(1:lingx, 1:lingy)
    hit = np.zeros((lingy, lingx), bool)
    for sx, stx, sy, sty in _LATTICES[pattern]:
        # MATLAB i = sx*r+1 : stx*dia : lingx, j = sy*r+1 : sty*dia : lingy
        for i in range(sx * r + 1, lingx + 1, stx * dia):
            x0, x1 = max(i - r, 1), min(i + r, lingx)
            for j in range(sy * r + 1, lingy + 1, sty * dia):
                y0, y1 = max(j - r, 1), min(j + r, lingy)
                sub = (xx[y0 - 1:y1, x0 - 1:x1] - i) ** 2 + (yy[y0 - 1:y1, x0 - 1:x1] - j) ** 2 <= r * r
                hit[y0 - 1:y1, x0 - 1:x1] |= sub
    return np.where(hit, 2.0, 3.0).astype(np.float32)


def reference_pattern(pattern):
    """2800 x 5000 medium-ID model of pattern 1..6 (rows are z, columns x)."""
    if pattern not in _LATTICES:
        raise ValueError("pattern must be 1..6")
    model = np.ones((MODY, LINGX), np.float32)
    model[2000:2000 + LINGY, :] = _layer(pattern)         # rows 2001..2240 (1-based)
    return model


def random_patches(shape, dx, fraction=0.10, r_min=2.0, r_max=10.0, seed=0, margin=0):
    """uint8 IDs (0 = background, 1 = patch) with seeded random circles.

    Radii are uniform in [r_min, r_max] metres, centres uniform over the grid
    minus ``margin`` cells on every side; circles are added until the patch
    cells reach ``fraction`` of the grid area.
    """
    nz, nx = shape
    rng = np.random.default_rng(seed)
    ids = np.zeros(shape, np.uint8)
    target = fraction * nz * nx
    count = 0
    zlo, zhi, xlo, xhi = margin, nz - margin, margin, nx - margin
    guard = 0
    while count < target and guard < 10_000_000:
        guard += 1
        rc = rng.uniform(r_min, r_max) / dx
        cz, cx = rng.uniform(zlo, zhi), rng.uniform(xlo, xhi)
        z0, z1 = max(int(np.floor(cz - rc)), 0), min(int(np.ceil(cz + rc)) + 1, nz)
        x0, x1 = max(int(np.floor(cx - rc)), 0), min(int(np.ceil(cx + rc)) + 1, nx)
        if z0 >= z1 or x0 >= x1:
            continue
        zz, xx = np.mgrid[z0:z1, x0:x1]
        disk = (zz - cz) ** 2 + (xx - cx) ** 2 <= rc * rc
        sub = ids[z0:z1, x0:x1]
        count += int(np.count_nonzero(disk & (sub == 0)))
        sub[disk] = 1
    return ids


def write_bin(path, grid2d, order="x"):
    """Raw float32 little-endian; order 'x' = x fastest (cu:685), 'z' = z fastest (patchy:50)."""
    a = np.asarray(grid2d, dtype="<f4")
    data = a if order == "x" else a.T
    np.ascontiguousarray(data).tofile(path)


def read_bin(path, nx, nz, order="x"):
    """Read an (nz, nx) grid written x-fastest or z-fastest; raises on a short file."""
    raw = np.fromfile(path, dtype="<f4")
    if raw.size < nx * nz:
        raise ValueError("%s: %d floats, expected %d" % (path, raw.size, nx * nz))
    raw = raw[:nx * nz]
    return raw.reshape(nz, nx) if order == "x" else raw.reshape(nx, nz).T.copy()
