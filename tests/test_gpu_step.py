"""The whole fluid step on the GPU against the oracle's restatement of
examples/dec_fluid.rs:46-141.

Per-operator parity is bit-exact (test_gpu_ops); across steps the PCG's
dot-product rounding differs (FP64 on the GPU), so fields are compared with
a relative L-inf tolerance stated in each test."""

import numpy as np
import pytest
import torch

from conftest import rng
from test_gpu_ops import dev, host

pytestmark = pytest.mark.gpu


def gpu_state(pg, g, vel, rho, p):
    return pg.Simplex1(g, dev(vel)), pg.Simplex2(g, dev(rho)), pg.Simplex2(g, dev(p))


def rel_linf(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-9), (np.float32, 2e-3)])
def test_reference_configuration(pg, oracle, dtype, tol):
    """examples/dec_fluid.rs as written: 128x128, dt 0.05, absolute
    threshold 0.1, 100 iterations, inflow box (rows 5..20, cols 54..64),
    the face obstacle of :71-78.  6 steps."""
    dims = (128, 128)
    nf = oracle.num_faces(dims)
    vel = np.zeros(nf, dtype)
    rho = np.zeros(dims, dtype)
    p = np.zeros(dims, dtype)
    fs = oracle.reference_face_mask(dims)
    g = pg.Grid2d(dims)
    g.set_solid_faces(fs)
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    gv, gr, gp = gpu_state(pg, g, vel, rho, p)
    cfg = pg.StepConfig()  # the reference's defaults
    prm = oracle.step_params(source=((0, 5, 54), (1, 20, 64)))
    for i in range(6):
        st_o = oracle.step(vel, rho, p, dims, prm, fs)
        st_g = pg.step(g, cfg, gv, gr, gp)
        assert abs(st_g["iterations"] - st_o.iterations) <= (0 if dtype == np.float64 else 3), i
        assert rel_linf(host(gv), vel) < tol, i
        assert rel_linf(host(gr), rho) < tol, i
    assert gv.data.dtype == tdt


def gaussian_blob(dims, center, sigma_frac):
    h, w = dims
    L = max(h, w)
    y, x = np.mgrid[0:h, 0:w]
    cy, cx = center[0] * h, center[1] * w
    s = sigma_frac * L
    return np.exp(-(((x + 0.5 - cx) ** 2 + (y + 0.5 - cy) ** 2) / (2 * s * s)))


def test_plume_2d_matches_oracle(pg, oracle):
    """The 2D plume (256x256, f32, walls, Gaussian blob at (0.5, 0.15),
    sigma 0.04, buoyancy 1, dt 0.5, PCG to relative 1e-5): 8 steps, fields
    within 2e-3 relative L-inf of the oracle, divergence below the solve
    tolerance after every step.  The oracle accumulates its dot products in
    double here, as the library does; with the reference's f32 sums its CG
    needs ~15% more iterations on this case."""
    oracle.set_dot64(True)
    try:
        _plume(pg, oracle)
    finally:
        oracle.set_dot64(False)


def test_plume_2d_50_steps_per_step(pg, oracle):
    """The 2D plume over 50 steps, each GPU step against the oracle step
    taken from the same input state (the GPU's state after the previous
    step), so the comparison measures one step's difference at every stage
    of the flow rather than the chaotic growth of earlier ones: velocity and
    density within 2e-4 relative L-inf (measured worst 3.4e-5 on GB300), the
    same iteration count within 5%, and the projected divergence within the
    solve's FP32 floor after every step."""
    oracle.set_dot64(True)
    try:
        dims = (256, 256)
        nf = oracle.num_faces(dims)
        g = pg.Grid2d(dims)
        gv, gr, gp = gpu_state(pg, g, np.zeros(nf, np.float32),
                               gaussian_blob(dims, (0.15, 0.5), 0.04).astype(np.float32), np.zeros(dims, np.float32))
        cfg = pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                            zero_solid_after_project=True,
                            solver=pg.SolverConfig(rel_stop=True, rel_tol=1e-5, max_iter=10000))
        prm = oracle.step_params(dt=0.5, buoyancy=1.0, walls_after_advect=True, zero_solid_after_project=True,
                                 rel_stop=True, rel_tol=1e-5, max_iter=10000)
        worst = 0.0
        for i in range(50):
            vel, rho, p = host(gv).copy(), host(gr).copy(), host(gp).copy()
            st_o = oracle.step(vel, rho, p, dims, prm)
            st_g = pg.step(g, cfg, gv, gr, gp)
            assert st_g["status"] == 0 and st_o.converged, i
            assert abs(st_g["iterations"] - st_o.iterations) <= max(3, 0.05 * st_o.iterations), i
            e = max(rel_linf(host(gr), rho), rel_linf(host(gv), vel))
            worst = max(worst, e)
            print("step", i, "iterations", st_g["iterations"], st_o.iterations, "rel L-inf %.2e" % e)
            assert e < 2e-4, (i, e)
            div = oracle.divergence_rhs(host(gv).astype(np.float64), dims)
            assert np.abs(div).max() <= 2e-3 * st_g["b_max"], i
        print("worst %.2e" % worst)
    finally:
        oracle.set_dot64(False)


def _plume(pg, oracle):
    dims = (256, 256)
    nf = oracle.num_faces(dims)
    vel = np.zeros(nf, np.float32)
    rho = gaussian_blob(dims, (0.15, 0.5), 0.04).astype(np.float32)
    p = np.zeros(dims, np.float32)
    g = pg.Grid2d(dims)
    gv, gr, gp = gpu_state(pg, g, vel, rho, p)
    solver = pg.SolverConfig(rel_stop=True, rel_tol=1e-5, max_iter=10000)
    cfg = pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                        zero_solid_after_project=True, solver=solver)
    prm = oracle.step_params(dt=0.5, buoyancy=1.0, walls_after_advect=True, zero_solid_after_project=True,
                             rel_stop=True, rel_tol=1e-5, max_iter=10000)
    for i in range(8):
        st_o = oracle.step(vel, rho, p, dims, prm)
        st_g = pg.step(g, cfg, gv, gr, gp)
        assert st_g["status"] == 0 and st_o.converged
        assert abs(st_g["iterations"] - st_o.iterations) <= max(3, 0.05 * st_o.iterations)
        assert rel_linf(host(gr), rho) < 2e-3, i
        assert rel_linf(host(gv), vel) < 2e-3, i
        # Plain FP32 PCG (the reference algorithm in FP32 storage): the
        # recursive residual meets 1e-5 relative, but the true residual --
        # the projected divergence -- drifts from it by FP32 rounding over
        # ~700 iterations and settles near 1e-3 relative on this case.  The
        # refined form below is the one that meets the tolerance.
        div = oracle.divergence_rhs(host(gv).astype(np.float64), dims)
        assert np.abs(div).max() <= 2e-3 * st_g["b_max"]


@pytest.mark.parametrize("precond", [0, 2])
def test_plume_2d_refined_divergence(pg, oracle, precond):
    """The same plume with FP64 residual refinement (plain CG or MG-PCG
    inside): after every step the projected field's max divergence is below
    the relative tolerance times ||b||inf, measured in FP64 by the oracle's
    operator -- the bound FP32 storage alone cannot meet."""
    dims = (256, 256)
    nf = oracle.num_faces(dims)
    vel = np.zeros(nf, np.float32)
    rho = gaussian_blob(dims, (0.15, 0.5), 0.04).astype(np.float32)
    g = pg.Grid2d(dims)
    gv, gr, gp = gpu_state(pg, g, vel, rho, np.zeros(dims, np.float32))
    tol = 1e-5
    solver = pg.SolverConfig(precond=precond, rel_stop=True, rel_tol=tol, max_iter=10000, refine=5)
    cfg = pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                        zero_solid_after_project=True, solver=solver)
    for i in range(6):
        st = pg.step(g, cfg, gv, gr, gp)
        assert st["status"] == 0, (i, st)
        div = oracle.divergence_rhs(host(gv).astype(np.float64), dims)
        # the velocity itself is FP32: allow its rounding on top
        assert np.abs(div).max() <= tol * st["b_max"] + 4 * 2.0 ** -24 * np.abs(host(gv)).max(), i


def test_headline_256_cubed_divergence(pg, oracle):
    """The benchmarked configuration at its full size: 256^3, filtered-noise
    velocity (max|u| = 2 cells/step, dt 1), walls, MG-PCG in double-float
    refinement to relative 1e-6.  After each of 2 steps the solve reports
    status 0 within 8 iterations, and the projected velocity's max
    divergence, computed in FP64 by the oracle's operator, is below
    1e-6 ||b||inf plus the FP32 rounding of the 6 faces of a cell."""
    from panopaea_gb300 import workloads as W

    dims = (256, 256, 256)
    vel, rho = W.initial_state("precision_3d_256", dims)
    g = pg.Grid3d(dims)
    gv, gr, gp = gpu_state(pg, g, vel, rho, np.zeros(dims, np.float32))
    solver = pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=20000, refine=4)
    cfg = pg.StepConfig(dt=1.0, buoyancy=0.0, source_enabled=False, walls_after_advect=True,
                        zero_solid_after_project=True, solver=solver)
    for i in range(2):
        st = pg.step(g, cfg, gv, gr, gp)
        assert st["status"] == 0 and st["iterations"] <= 8, (i, st)
        v = host(gv)
        div = oracle.divergence_rhs(v.astype(np.float64), dims)
        assert np.abs(div).max() <= 1e-6 * st["b_max"] + 6 * 2.0 ** -24 * np.abs(v).max(), i


def test_step_3d_matches_oracle(pg, oracle):
    """3D step (extension), 48x40x36 with a solid box, buoyancy, Jacobi PCG
    to 1e-5: 3 steps within 2e-3 relative L-inf."""
    dims = (36, 40, 48)
    r = rng(21)
    nf = oracle.num_faces(dims)
    vel = oracle.walls((0.5 * r.standard_normal(nf)).astype(np.float32), dims)
    rho = r.random(dims).astype(np.float32)
    p = np.zeros(dims, np.float32)
    cs = np.zeros(dims, np.uint8)
    cs[10:20, 12:22, 20:30] = 1
    fs = oracle.cell_mask_to_faces(cs)
    g = pg.Grid3d(dims)
    g.set_solid_cells(cs)
    gv, gr, gp = gpu_state(pg, g, vel, rho, p)
    solver = pg.SolverConfig(precond=1, rel_stop=True, rel_tol=1e-5, max_iter=10000)
    cfg = pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                        zero_solid_after_project=True, solver=solver)
    prm = oracle.step_params(dt=0.5, buoyancy=1.0, walls_after_advect=True, zero_solid_after_project=True,
                             precond=1, rel_stop=True, rel_tol=1e-5, max_iter=10000)
    for i in range(3):
        oracle.step(vel, rho, p, dims, prm, fs)
        st = pg.step(g, cfg, gv, gr, gp)
        assert st["status"] == 0
        assert rel_linf(host(gr), rho) < 2e-3, i
        assert rel_linf(host(gv), vel) < 2e-3, i


def test_source_box_and_field(pg, oracle):
    dims = (5, 24, 20)
    r = rng(5)
    nf = oracle.num_faces(dims)
    vel = np.zeros(nf, np.float64)
    rho = np.zeros(dims)
    p = np.zeros(dims)
    src = r.random(dims) * (r.random(dims) < 0.1)
    g = pg.Grid3d(dims)
    gv, gr, gp = gpu_state(pg, g, vel, rho, p)
    cfg = pg.StepConfig(dt=0.3, source_lo=(1, 2, 3), source_hi=(3, 6, 9), source_density=0.7, source_vy=2.0,
                        source_field=pg.Simplex2(g, dev(src)),
                        solver=pg.SolverConfig(rel_stop=True, rel_tol=1e-10, max_iter=5000))
    prm = oracle.step_params(dt=0.3, source=((1, 2, 3), (3, 6, 9)), source_density=0.7, source_vy=2.0,
                             source_field=src, rel_stop=True, rel_tol=1e-10, max_iter=5000)
    for _ in range(2):
        oracle.step(vel, rho, p, dims, prm)
        pg.step(g, cfg, gv, gr, gp)
    assert rel_linf(host(gr), rho) < 1e-9
    assert rel_linf(host(gv), vel) < 1e-8
