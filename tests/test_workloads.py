"""The seeded synthetic inputs of the benchmark configurations
(panopaea_gb300.workloads), checked on the CPU at reduced sizes: the shapes,
value ranges and boundary conditions each configuration states, and that
every process building them gets the same arrays."""

import numpy as np

from panopaea_gb300 import workloads as W


def parts_of(vel, dims):
    out, o = [], 0
    for s in W.face_shapes(dims):
        n = int(np.prod(s))
        out.append(vel[o:o + n].reshape(s))
        o += n
    assert o == vel.size
    return out


def test_filtered_noise_velocity_3d():
    dims = (12, 10, 14)
    vel, rho = W.initial_state("precision_3d_256", dims)
    assert vel.dtype == np.float32 and vel.size == W.num_faces(dims)
    assert abs(np.abs(vel).max() - 2.0) < 1e-6  # max|u| = 2 cells/step at dt = 1
    for ax, p in enumerate(parts_of(vel, dims)):  # part k is normal to axis k: its two end slabs are walls
        assert not p.take(0, axis=ax).any() and not p.take(-1, axis=ax).any()
    assert rho.shape == dims and rho.min() == 0.0 and abs(rho.max() - 1.0) < 1e-6
    v2, r2 = W.initial_state("precision_3d_256", dims)
    assert np.array_equal(vel, v2) and np.array_equal(rho, r2)


def test_plume_2d_blob():
    dims = (64, 64)
    vel, rho = W.initial_state("plume_2d_256", dims)
    assert not vel.any() and vel.size == W.num_faces(dims)
    y, x = np.unravel_index(np.argmax(rho), dims)
    # centre (x, y) = (0.5, 0.15) of the domain, cell centres at +0.5
    assert abs(x + 0.5 - 0.5 * 64) <= 0.5 and abs(y + 0.5 - 0.15 * 64) <= 0.5
    assert 0.9 < rho.max() <= 1.0


def test_sphere_plume_geometry():
    dims = (64, 48, 64)
    mask, src = W.sphere_plume(dims)
    d, h, w = dims
    assert mask[d // 2, h // 2, w // 2] == 1 and mask[0, 0, 0] == 0
    assert np.array_equal(mask, mask[::-1, :, :]) and np.array_equal(mask, mask[:, :, ::-1])
    assert src.max() == 1.0 and not src[:, h // 2:, :].any()  # the disk sits on the y = 0 side
    assert not (src.astype(bool) & mask.astype(bool)).any()


def test_batch_grids():
    dims, masks, srcs = W.batch_grids(24)
    sides = set(range(64, 513, 32))
    for (h, w), m, s in zip(dims, masks, srcs):
        assert h in sides and w in sides and m.shape == (h, w) and s.shape == (h, w)
        sy, sx = np.unravel_index(np.argmax(s), s.shape)
        assert s[sy, sx] == 1.0 and m[sy, sx] == 0  # the source cell is fluid
        assert sy in (0, h - 1) or sx in (0, w - 1)  # and adjacent to the boundary
        assert not s[m > 0].any()
    d2, m2, s2 = W.batch_grids(24)
    assert d2 == dims and all(np.array_equal(a, b) for a, b in zip(m2, masks))
