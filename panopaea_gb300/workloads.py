"""Seeded synthetic inputs for the benchmark configurations (numpy only, so
every process that builds them gets identical arrays).

* :func:`filtered_noise_velocity` -- faces i.i.d. N(0, 1) (seeded), low-pass
  filtered by 3 passes of a 3x3x3 box filter per face array, scaled to
  max|u| = umax, boundary faces zeroed (solid walls);
* :func:`filtered_noise_density` -- a cell field built the same way, mapped
  affinely onto [0, 1];
* :func:`gaussian_blob_2d` -- exp(-|x - c|^2 / (2 sigma^2)), c and sigma as
  fractions of the domain, peak 1.
"""

import numpy as np


def _box3(a, passes=3):
    """`passes` passes of a 3-wide box filter along every axis (edge values
    repeated at the borders)."""
    a = np.asarray(a, np.float32)
    for _ in range(passes):
        for ax in range(a.ndim):
            pad = [(0, 0)] * a.ndim
            pad[ax] = (1, 1)
            p = np.pad(a, pad, mode="edge")
            n = a.shape[ax]
            sl = lambda s, e: tuple(slice(s, e) if i == ax else slice(None) for i in range(a.ndim))  # noqa: E731
            a = (p[sl(0, n)] + p[sl(1, n + 1)] + p[sl(2, n + 2)]) * np.float32(1.0 / 3.0)
    return a


def face_shapes(dims):
    if len(dims) == 2:
        h, w = dims
        return [(h + 1, w), (h, w + 1)]
    d, h, w = dims
    return [(d + 1, h, w), (d, h + 1, w), (d, h, w + 1)]


def num_faces(dims):
    return sum(int(np.prod(s)) for s in face_shapes(dims))


def zero_walls(parts):
    """Zero the domain-boundary faces of each face part (normal axis ends)."""
    nd = parts[0].ndim
    for ax, part in enumerate(parts):  # part k is normal to axis k ((z,) y, x order)
        idx0 = tuple(0 if i == ax else slice(None) for i in range(nd))
        idx1 = tuple(-1 if i == ax else slice(None) for i in range(nd))
        part[idx0] = 0.0
        part[idx1] = 0.0
    return parts


def filtered_noise_velocity(dims, seed=2, umax=2.0, passes=3, dtype=np.float32):
    rng = np.random.default_rng(seed)
    parts = [_box3(rng.standard_normal(s, dtype=np.float32), passes) for s in face_shapes(dims)]
    zero_walls(parts)
    m = max(np.abs(p).max() for p in parts)
    parts = [p * (umax / m) for p in parts]
    return np.concatenate([p.ravel() for p in parts]).astype(dtype)


def filtered_noise_density(dims, seed=3, passes=3, dtype=np.float32):
    rng = np.random.default_rng(seed)
    a = _box3(rng.standard_normal(dims, dtype=np.float32), passes)
    a = (a - a.min()) / (a.max() - a.min())
    return a.astype(dtype)


def gaussian_blob_2d(dims, center=(0.5, 0.15), sigma=0.04, dtype=np.float32):
    """center = (x, y) fractions (y up), sigma a fraction of the larger side."""
    h, w = dims
    s = sigma * max(h, w)
    y, x = np.mgrid[0:h, 0:w]
    cx, cy = center[0] * w, center[1] * h
    return np.exp(-(((x + 0.5 - cx) ** 2 + (y + 0.5 - cy) ** 2) / (2 * s * s))).astype(dtype)


# Named workloads: dims, dt and the fields they start from.
WORKLOADS = {
    # 3D MAC grid 256^3, filtered-noise velocity (max |u| = 2 cells/step, so
    # dt = 1), walls, one step of trilinear advection + 7-point projection
    # to relative residual 1e-6.
    "precision_3d_256": dict(dims=(256, 256, 256), dt=1.0, rel_tol=1e-6, buoyancy=0.0, cpu=True, compare="plain"),
    # 2D plume 256^2: blob at (0.5, 0.15), sigma 0.04, buoyancy 1, dt 0.5, 1e-5.
    "plume_2d_256": dict(dims=(256, 256), dt=0.5, rel_tol=1e-5, buoyancy=1.0, cpu=True, compare="plain"),
    # Large single grid 512^3: solid sphere r = 64 at the centre, smoke from a
    # bottom-centre disk of radius 32 (density 1), buoyancy 1, velocity from
    # rest, trilinear advection, projection to 1e-6 by MG-PCG (chosen) and by
    # Jacobi-PCG (the comparison).
    "sphere_3d_512": dict(dims=(512, 512, 512), dt=0.5, rel_tol=1e-6, buoyancy=1.0, cpu=False, compare="jacobi",
                          sphere_r=64, disk_r=32),
}


def sphere_plume(dims, sphere_r=64, disk_r=32, disk_h=4):
    """Cell mask of a solid sphere at the centre and the source field of a
    smoke disk (density 1) on the bottom (y = 0 side), both centred in x
    and z; radii and thickness scale with min(dims) / 512."""
    d, h, w = dims
    sc = min(dims) / 512.0
    z, y, x = np.ogrid[0:d, 0:h, 0:w]
    zc, yc, xc = z + 0.5 - d / 2, y + 0.5 - h / 2, x + 0.5 - w / 2
    r = sphere_r * sc
    mask = ((zc * zc + yc * yc + xc * xc) < r * r).astype(np.uint8)
    rd = disk_r * sc
    src = (((zc * zc + xc * xc) < rd * rd) & (y < max(1, int(round(disk_h * max(sc, 0.25)))))).astype(np.float32)
    return mask, np.broadcast_to(src, dims).astype(np.float32)


def batch_grids(count=512, seed=3, sides=tuple(range(64, 513, 32)), max_circles=8, rmin=4, rmax=32, sigma=4.0):
    """The batching configuration: `count` 2D grids, each side drawn
    uniformly from `sides` (non-square allowed), 0..max_circles solid
    circles of radius rmin..rmax cells, and a Gaussian smoke source (peak 1,
    `sigma` cells) at a random cell adjacent to the domain boundary.
    Returns (dims, cell_masks, sources) as lists of numpy arrays."""
    rng = np.random.default_rng(seed)
    dims, masks, sources = [], [], []
    for _ in range(count):
        h, w = int(rng.choice(sides)), int(rng.choice(sides))
        y, x = np.mgrid[0:h, 0:w]
        m = np.zeros((h, w), np.uint8)
        for _ in range(int(rng.integers(0, max_circles + 1))):
            r = rng.uniform(rmin, rmax)
            cy, cx = rng.uniform(0, h), rng.uniform(0, w)
            m |= (((y + 0.5 - cy) ** 2 + (x + 0.5 - cx) ** 2) < r * r).astype(np.uint8)
        side = int(rng.integers(0, 4))  # bottom, top, left, right
        if side < 2:
            sy, sx = (0 if side == 0 else h - 1), int(rng.integers(0, w))
        else:
            sy, sx = int(rng.integers(0, h)), (0 if side == 2 else w - 1)
        m[max(0, sy - 2):sy + 3, max(0, sx - 2):sx + 3] = 0  # keep the source cell fluid
        src = np.exp(-((y - sy) ** 2 + (x - sx) ** 2) / (2 * sigma * sigma)).astype(np.float32)
        src[m > 0] = 0.0
        dims.append((h, w))
        masks.append(m)
        sources.append(src)
    return dims, masks, sources


def initial_state(name, dims=None):
    """(vel, density) host arrays for a named workload (dims overridable)."""
    spec = WORKLOADS[name]
    dims = tuple(dims or spec["dims"])
    if name.startswith("sphere_3d"):
        return np.zeros(num_faces(dims), np.float32), np.zeros(dims, np.float32)
    if name.startswith("plume_2d"):
        vel = np.zeros(num_faces(dims), np.float32)
        rho = gaussian_blob_2d(dims)
        return vel, rho
    return filtered_noise_velocity(dims), filtered_noise_density(dims)
