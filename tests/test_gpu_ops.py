"""GPU parity of every operator against the oracle: bit-exact (same float
operations in the same order), 2D and 3D, f32 and f64, with and without
solid faces, odd and small sizes, back-traces far outside the grid.
Also the reference's own golden vectors run through the GPU API."""

import numpy as np
import pytest
import torch

from conftest import rng, seed_of

pytestmark = pytest.mark.gpu

DIMS_2D = [(5, 5), (3, 7), (2, 2), (64, 48), (257, 130), (1, 6), (7, 1)]
DIMS_3D = [(2, 2, 2), (4, 5, 6), (17, 9, 33), (40, 36, 32)]
DTYPES = [np.float32, np.float64]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.data.cpu().numpy()


def make_grid(pg, dims):
    return pg.Grid2d(dims) if len(dims) == 2 else pg.Grid3d(dims)


def faces(pg, g, a):
    return pg.Simplex1(g, dev(a))


def cells(pg, g, a):
    return pg.Simplex2(g, dev(a))


def same(a, b):
    assert a.dtype == b.dtype and a.shape == b.shape
    ok = np.array_equal(a, b, equal_nan=True)
    if not ok:
        bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))))
        raise AssertionError("%d mismatches, first at %s: %r vs %r" % (len(bad), bad[0], a[tuple(bad[0])],
                                                                       b[tuple(bad[0])]))


# ---------------------------------------------------------------------------
# The reference's golden tests (dec/grid.rs:428-515) through the GPU API.

def test_golden_divergence_gpu(pg, golden):
    d = golden["grid_2d_divergence"]
    g = pg.Grid2d((5, 5))
    vel = g.new_simplex_1(torch.float32)
    vy, vx = vel.split_mut()
    vy.copy_(torch.tensor(d["velocities_y"], dtype=torch.float32))
    vx.copy_(torch.tensor(d["velocities_x"], dtype=torch.float32))
    vel_primal = g.new_simplex_1(torch.float32)
    div = g.new_simplex_2(torch.float32)
    g.hodge_1_dual(vel_primal, vel)
    g.derivative_1_primal(div, vel_primal)
    ref = np.array(d["div_ref"], np.float32).reshape(5, 5)
    assert np.all(np.abs(host(div) - ref) < d["eps"])


def test_golden_laplacian_gpu(pg, golden):
    lc = golden["grid_2d_laplacian"]
    g = pg.Grid2d((3, 3))
    faces_primal = pg.Simplex2(g, torch.tensor(lc["faces_primal"], dtype=torch.float64).cuda())
    faces_dual = g.new_simplex_2(torch.float64)
    edges_dual = g.new_simplex_1(torch.float64)
    edges_primal = g.new_simplex_1(torch.float64)
    lap = g.new_simplex_2(torch.float64)
    g.hodge_2_primal(faces_dual, faces_primal)
    g.derivative_0_dual(edges_dual, faces_dual)
    g.hodge_1_dual(edges_primal, edges_dual)
    g.derivative_1_primal(lap, edges_primal)
    ref = np.array(lc["laplacian_ref"]).reshape(3, 3)
    assert np.all(np.abs(host(lap) - ref) < lc["eps"])
    fused = g.new_simplex_2(torch.float64)
    g.laplacian(fused, faces_primal, 1.0)
    same(host(fused), host(lap))


# ---------------------------------------------------------------------------

@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("dims", DIMS_2D)
def test_dec_ops_2d(pg, oracle, dims, dtype):
    r = rng(seed_of((dims, str(dtype))))
    g = make_grid(pg, dims)
    nf = oracle.num_faces(dims)
    e = r.standard_normal(nf).astype(dtype)
    p = r.standard_normal(dims).astype(dtype)
    out = faces(pg, g, np.zeros(nf, dtype))
    g.hodge_1_dual(out, faces(pg, g, e))
    same(host(out), oracle.hodge_1_dual(e, dims))
    g.hodge_1_primal(out, faces(pg, g, e))
    same(host(out), oracle.hodge_1_primal(e, dims))
    c = cells(pg, g, np.zeros(dims, dtype))
    g.derivative_1_primal(c, faces(pg, g, e))
    same(host(c), oracle.derivative_1_primal(e, dims))
    g.hodge_2_primal(c, cells(pg, g, p))
    same(host(c), p)
    # derivative_0_dual leaves boundary faces untouched
    init = r.standard_normal(nf).astype(dtype)
    out = faces(pg, g, init)
    g.derivative_0_dual(out, cells(pg, g, p))
    same(host(out), oracle.derivative_0_dual(p, dims, edges=init))


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("masked", [False, True])
@pytest.mark.parametrize("dims", DIMS_2D + DIMS_3D)
def test_laplacian_rhs_project(pg, oracle, dims, dtype, masked):
    r = rng(seed_of((dims, str(dtype), masked)))
    g = make_grid(pg, dims)
    nf = oracle.num_faces(dims)
    fs = (r.random(nf) < 0.2).astype(np.uint8) if masked else None
    if masked:
        g.set_solid_faces(fs)
    p = r.standard_normal(dims).astype(dtype)
    vel = r.standard_normal(nf).astype(dtype)
    dt = 0.37
    out = cells(pg, g, np.zeros(dims, dtype))
    g.laplacian(out, cells(pg, g, p), dt)
    same(host(out), oracle.laplacian(p, dt, dims, fs))
    g.divergence_rhs(out, faces(pg, g, vel))
    same(host(out), oracle.divergence_rhs(vel, dims, fs))
    for zero_solid in (False, True):
        v = faces(pg, g, vel)
        g.project(v, cells(pg, g, p), dt, zero_solid=zero_solid)
        same(host(v), oracle.project(vel, p, dt, dims, fs, zero_solid=zero_solid))
    v = faces(pg, g, vel)
    g.walls(v)
    same(host(v), oracle.walls(vel, dims))
    if masked:
        v = faces(pg, g, vel)
        g.mask_solid_faces(v)
        same(host(v), oracle.mask_faces(vel, fs))


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("dims", [d for d in DIMS_2D + DIMS_3D if min(d) >= 2] + [(300, 270), (3, 260, 5)])
@pytest.mark.parametrize("speed", [0.3, 3.0, 400.0])
def test_advection(pg, oracle, dims, dtype, speed):
    """advect / advect_mac bit-exact, including back-traces far outside the
    grid (speed 400) and the float clamp rule for sides >= 257."""
    r = rng(seed_of((dims, str(dtype), speed)))
    g = make_grid(pg, dims)
    nf = oracle.num_faces(dims)
    vel = (speed * r.standard_normal(nf)).astype(dtype)
    q = r.standard_normal(dims).astype(dtype)
    qf = r.standard_normal(nf).astype(dtype)
    dt = 0.61
    out = cells(pg, g, np.zeros(dims, dtype))
    pg.advect(out, cells(pg, g, q), dt, faces(pg, g, vel))
    same(host(out), oracle.advect(q, dt, vel, dims))
    outf = faces(pg, g, np.zeros(nf, dtype))
    pg.advect_mac(outf, faces(pg, g, qf), dt, faces(pg, g, vel))
    same(host(outf), oracle.advect_mac(qf, dt, vel, dims))
    # self-advection as in examples/dec_fluid.rs:60
    v = faces(pg, g, vel)
    pg.advect_mac(outf, v, dt, v)
    same(host(outf), oracle.advect_mac(vel, dt, vel, dims))


@pytest.mark.parametrize("dims", [(70, 50, 90), (33, 17, 65), (9, 40, 100)])
def test_self_advection_3d_mixed_speeds(pg, oracle, dims):
    """3D self-advection of a smooth field with sparse fast faces and NaN
    velocities, at sizes with many blocks: bit-exact against the oracle."""
    r = rng(seed_of(("staged", dims)))
    g = make_grid(pg, dims)
    nf = oracle.num_faces(dims)
    # smooth part (|v| dt up to ~2.5 cells) plus sparse fast faces and NaNs
    t = np.arange(nf, dtype=np.float64)
    vel = (2.5 * np.sin(t * 0.0007) + 0.2 * r.standard_normal(nf)).astype(np.float32)
    vel[r.integers(0, nf, nf // 50)] = 9.0
    vel[r.integers(0, nf, nf // 500)] = np.nan
    dt = 0.9
    v = faces(pg, g, vel)
    out = faces(pg, g, np.zeros(nf, np.float32))
    pg.advect_mac(out, v, dt, v)
    same(host(out), oracle.advect_mac(vel, dt, vel, dims))


def test_advection_nonfinite(pg, oracle):
    """NaN / inf velocities follow the reference's f64::max/min rules."""
    dims = (9, 11)
    r = rng(11)
    g = make_grid(pg, dims)
    nf = oracle.num_faces(dims)
    vel = r.standard_normal(nf).astype(np.float32)
    vel[::7] = np.nan
    q = r.standard_normal(dims).astype(np.float32)
    out = cells(pg, g, np.zeros(dims, np.float32))
    pg.advect(out, cells(pg, g, q), 0.5, faces(pg, g, vel))
    same(host(out), oracle.advect(q, 0.5, vel, dims))
    outf = faces(pg, g, np.zeros(nf, np.float32))
    qf = r.standard_normal(nf).astype(np.float32)
    pg.advect_mac(outf, faces(pg, g, qf), 0.5, faces(pg, g, vel))
    same(host(outf), oracle.advect_mac(qf, 0.5, vel, dims))


def test_solid_cells_rule(pg, oracle):
    dims = (6, 7, 8)
    r = rng(12)
    cs = (r.random(dims) < 0.2).astype(np.uint8)
    g = make_grid(pg, dims)
    g.set_solid_cells(cs)
    fs = oracle.cell_mask_to_faces(cs)
    p = r.standard_normal(dims).astype(np.float32)
    out = cells(pg, g, np.zeros(dims, np.float32))
    g.laplacian(out, cells(pg, g, p), 1.0)
    same(host(out), oracle.laplacian(p, 1.0, dims, fs))


def test_bad_shapes(pg):
    from panopaea_gb300 import _native as N

    g = pg.Grid2d((1, 5))
    a = g.new_simplex_2()
    v = g.new_simplex_1()
    with pytest.raises(N.PgError) as ei:
        pg.advect(g.new_simplex_2(), a, 0.1, v)
    assert ei.value.status == N.PG_BAD_ARG
    g3 = pg.Grid3d((2, 3, 4))
    with pytest.raises(N.PgError):
        g3.hodge_1_dual(g3.new_simplex_1(), g3.new_simplex_1())
    with pytest.raises(N.PgError):
        pg.advect(a, a, 0.1, v)  # dst aliases src
