"""Second-order limited advection of a cell scalar (MacCormack, BFECC) on the
GPU against the oracle's restatement: bit-exact per call (same float
operations in the same order, first-order passes shared with ``advect``),
2D and 3D, f32 and f64, slow and far-out-of-grid back-traces; and the whole
step with ``advect_scheme`` against the oracle's step."""

import numpy as np
import pytest
import torch

from conftest import rng, seed_of
from test_gpu_ops import cells, faces, host, make_grid, same
from test_gpu_step import gpu_state, rel_linf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("dims", [(2, 2), (5, 7), (64, 48), (300, 270), (2, 2, 2), (17, 9, 33), (40, 36, 32)])
@pytest.mark.parametrize("speed", [0.3, 3.0, 400.0])
def test_advect2_bit_exact(pg, oracle, dims, dtype, scheme, speed):
    r = rng(seed_of((dims, str(dtype), scheme, speed)))
    g = make_grid(pg, dims)
    nf = oracle.num_faces(dims)
    vel = (speed * r.standard_normal(nf)).astype(dtype)
    q = r.standard_normal(dims).astype(dtype)
    dt = 0.61
    out = cells(pg, g, np.zeros(dims, dtype))
    pg.advect2(out, cells(pg, g, q), dt, faces(pg, g, vel), scheme)
    same(host(out), oracle.advect2(q, dt, vel, dims, scheme))


def test_advect2_limiter_keeps_range(pg, oracle):
    """A blob translated 40 steps: the limited schemes never leave [0, 1]
    and keep the peak well above the first-order scheme's."""
    h, w = 48, 64
    y, x = np.mgrid[0:h, 0:w]
    q0 = np.exp(-((x - 16.0) ** 2 + (y - 24.0) ** 2) / 18.0).astype(np.float32)
    vel = np.zeros(oracle.num_faces((h, w)), np.float32)
    vel[(h + 1) * w:] = 0.37
    g = pg.Grid2d((h, w))
    v = faces(pg, g, vel)
    peaks = {}
    for scheme in (0, 1, 2):
        a, b = cells(pg, g, q0), cells(pg, g, np.zeros_like(q0))
        for _ in range(40):
            if scheme == 0:
                pg.advect(b, a, 1.0, v)
            else:
                pg.advect2(b, a, 1.0, v, scheme)
            a, b = b, a
        out = host(a)
        assert out.min() >= 0.0 and out.max() <= 1.0
        peaks[scheme] = out.max()
    assert peaks[1] > peaks[0] + 0.1 and peaks[2] > peaks[0] + 0.1


def test_advect2_bad_args(pg):
    g = pg.Grid2d((8, 8))
    q = g.new_simplex_2(torch.float32)
    out = g.new_simplex_2(q.data.dtype)
    v = g.new_simplex_1(q.data.dtype)
    for bad in (0, 3, -1):
        with pytest.raises(pg.PgError):
            pg.advect2(out, q, 0.5, v, bad)
    with pytest.raises(pg.PgError):
        pg.advect2(q, q, 0.5, v, 1)


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("dims", [(96, 80), (20, 24, 28)])
def test_step_with_advect_scheme(pg, oracle, dims, scheme):
    """f64 steps with second-order density advection, buoyancy, walls,
    Jacobi PCG to relative 1e-10: the PCG dot products differ only in
    summation order, so fields agree to 1e-9 relative."""
    r = rng(seed_of((dims, scheme)))
    nf = oracle.num_faces(dims)
    vel = oracle.walls((0.3 * r.standard_normal(nf)).astype(np.float64), dims)
    rho = r.random(dims)
    p = np.zeros(dims)
    g = make_grid(pg, dims)
    gv, gr, gp = gpu_state(pg, g, vel, rho, p)
    solver = pg.SolverConfig(precond=1, rel_stop=True, rel_tol=1e-10, max_iter=20000)
    cfg = pg.StepConfig(dt=0.4, buoyancy=0.5, source_enabled=False, walls_after_advect=True,
                        advect_scheme=scheme, solver=solver)
    prm = oracle.step_params(dt=0.4, buoyancy=0.5, walls_after_advect=True, precond=1, rel_stop=True,
                             rel_tol=1e-10, max_iter=20000, advect_scheme=scheme)
    for i in range(3):
        st_o = oracle.step(vel, rho, p, dims, prm)
        st_g = pg.step(g, cfg, gv, gr, gp)
        assert st_g["status"] == 0 and st_o.converged
        assert rel_linf(host(gr), rho) < 1e-9, i
        assert rel_linf(host(gv), vel) < 1e-9, i
