"""BF16-stored density: the advection kernel bit-exact against the oracle
(the FP32 advection of the widened values, rounded to nearest even), and
the whole step with a BF16 density against the oracle's step with the
density rounded to BF16 after every write."""

import numpy as np
import pytest
import torch

from conftest import rng, seed_of
from test_gpu_ops import dev, faces, host, make_grid
from test_gpu_step import gaussian_blob, rel_linf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(2, 2), (5, 7), (64, 48), (300, 270), (2, 2, 2), (17, 9, 33), (40, 36, 32)])
@pytest.mark.parametrize("speed", [0.3, 3.0, 400.0])
def test_advect_bf16_bit_exact(pg, oracle, dims, speed):
    r = rng(seed_of((dims, speed, "bf16")))
    g = make_grid(pg, dims)
    nf = oracle.num_faces(dims)
    vel = (speed * r.standard_normal(nf)).astype(np.float32)
    q = oracle.bf16_bits(r.standard_normal(dims).astype(np.float32))
    src = pg.Simplex2(g, dev(q.view(np.int16)).view(torch.bfloat16))
    out = g.new_simplex_2(torch.bfloat16)
    pg.fluid.advect_bf16(out, src, 0.61, faces(pg, g, vel))
    got = host(pg.Simplex2(g, out.data.view(torch.int16))).view(np.uint16)
    want = oracle.advect_bf16(q, 0.61, vel, dims)
    assert np.array_equal(got, want), np.argwhere(got != want)[:3]


def test_step_bf16_density_matches_oracle(pg, oracle):
    """The 256^2 plume (buoyancy 1, dt 0.5, walls, relative 1e-5) for 6 steps
    with BF16 density: within 2e-3 relative of the oracle's BF16-density
    step, and every density value a BF16 value."""
    oracle.set_dot64(True)
    try:
        dims = (256, 256)
        nf = oracle.num_faces(dims)
        vel = np.zeros(nf, np.float32)
        rho = oracle.bits_to_f32(oracle.bf16_bits(gaussian_blob(dims, (0.15, 0.5), 0.04).astype(np.float32)))
        p = np.zeros(dims, np.float32)
        g = pg.Grid2d(dims)
        gv, gp = pg.Simplex1(g, dev(vel)), pg.Simplex2(g, dev(p))
        gr = pg.Simplex2(g, dev(rho).to(torch.bfloat16))
        solver = pg.SolverConfig(rel_stop=True, rel_tol=1e-5, max_iter=10000)
        cfg = pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                            zero_solid_after_project=True, solver=solver)
        prm = oracle.step_params(dt=0.5, buoyancy=1.0, walls_after_advect=True, zero_solid_after_project=True,
                                 rel_stop=True, rel_tol=1e-5, max_iter=10000, density_bf16=True)
        for i in range(6):
            st_o = oracle.step(vel, rho, p, dims, prm)
            st_g = pg.step(g, cfg, gv, gr, gp)
            assert st_g["status"] == 0 and st_o.converged
            gr32 = gr.data.float().cpu().numpy()
            assert np.array_equal(oracle.bits_to_f32(oracle.bf16_bits(gr32)), gr32)
            assert np.array_equal(oracle.bits_to_f32(oracle.bf16_bits(rho)), rho)
            assert rel_linf(gr32, rho) < 2e-3, i
            assert rel_linf(host(gv), vel) < 2e-3, i
    finally:
        oracle.set_dot64(False)


def test_bf16_density_tracks_fp32_density(pg, oracle):
    """Same 3D filtered-noise state stepped with FP32 and with BF16 density
    (MG-PCG in refinement to 1e-6): density within 1% and velocity within
    1% relative L-inf after 4 steps -- BF16 keeps 8 bits of mantissa, so the
    difference is the accumulated storage rounding, not a solver effect."""
    from panopaea_gb300 import workloads as W

    dims = (48, 40, 56)
    vel0 = W.filtered_noise_velocity(dims, seed=5)
    rho0 = oracle.bits_to_f32(oracle.bf16_bits(W.filtered_noise_density(dims, seed=6)))
    out = {}
    for dt_ in (torch.float32, torch.bfloat16):
        g = pg.Grid3d(dims)
        gv, gp = pg.Simplex1(g, dev(vel0.copy())), g.new_simplex_2()
        gr = pg.Simplex2(g, dev(rho0.copy()).to(dt_))
        cfg = pg.StepConfig(dt=1.0, buoyancy=0.5, source_enabled=False, walls_after_advect=True,
                            zero_solid_after_project=True,
                            solver=pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=20000, refine=4))
        for _ in range(4):
            assert pg.step(g, cfg, gv, gr, gp)["status"] == 0
        out[dt_] = (host(gv), gr.data.float().cpu().numpy())
    assert rel_linf(out[torch.bfloat16][1], out[torch.float32][1]) < 1e-2
    assert rel_linf(out[torch.bfloat16][0], out[torch.float32][0]) < 1e-2
