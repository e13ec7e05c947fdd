"""Batched 2D grids (pg_batch_*): every grid of a batch advanced in one
launch per stage must match the same grid stepped alone -- bit for bit in
advection, -div and projection (shared per-sample arithmetic), within CG
rounding overall (the per-grid reductions run in a different order).  The
batched multigrid preconditioner is checked the same way against the
single-grid MG-PCG, and by the divergence its projection leaves."""

import numpy as np
import pytest
import torch

from conftest import rng

pytestmark = pytest.mark.gpu

DIMS = [(2, 3), (7, 5), (33, 64), (64, 33), (96, 128), (17, 9), (128, 128), (40, 200)]


def make_case(seed=0):
    r = rng(seed)
    masks, vels, rhos, srcs = [], [], [], []
    from panopaea_gb300 import workloads as W

    for i, (h, w) in enumerate(DIMS):
        m = np.zeros((h, w), np.uint8)
        if i % 2 == 1 and h > 6 and w > 6:
            m[h // 3:h // 3 + 3, w // 3:w // 3 + 3] = 1
        masks.append(m)
        parts = [r.standard_normal(s).astype(np.float32) for s in W.face_shapes((h, w))]
        W.zero_walls(parts)
        vels.append(np.concatenate([p.ravel() for p in parts]))
        rhos.append(r.random((h, w)).astype(np.float32))
        s = np.zeros((h, w), np.float32)
        s[0, 0] = 0.9
        srcs.append(s)
    return masks, vels, rhos, srcs


def config(pg, precond):
    return pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                         zero_solid_after_project=True,
                         solver=pg.SolverConfig(precond=precond, rel_stop=True, rel_tol=1e-5, max_iter=20000))


@pytest.mark.parametrize("precond", [0, 1, 2])
def test_batch_matches_single_grids(pg, precond):
    masks, vels, rhos, srcs = make_case()
    B = pg.Batch2d(DIMS)
    B.set_solid_cells(masks)
    v = torch.from_numpy(B.pack_faces(vels)).cuda()
    rho = torch.from_numpy(B.pack_cells(rhos)).cuda()
    p = B.new_cells()
    src = torch.from_numpy(B.pack_cells(srcs)).cuda()
    cfg = config(pg, precond)
    for _ in range(3):
        stats = B.step(cfg, v, rho, p, source_field=src)
    torch.cuda.synchronize()
    for i, (h, w) in enumerate(DIMS):
        g = pg.Grid2d((h, w))
        g.set_solid_cells(masks[i])
        gv = pg.Simplex1(g, torch.from_numpy(vels[i].copy()).cuda())
        gr = pg.Simplex2(g, torch.from_numpy(rhos[i].copy()).cuda())
        gp = g.new_simplex_2()
        c1 = config(pg, precond)
        c1.source_field = pg.Simplex2(g, torch.from_numpy(srcs[i]).cuda())
        for _ in range(3):
            st1 = pg.step(g, c1, gv, gr, gp)
        torch.cuda.synchronize()
        bv = B.faces_of(v, i).cpu().numpy()
        br = B.cells_of(rho, i).cpu().numpy()
        sv = gv.data.cpu().numpy()
        sr = gr.data.cpu().numpy()
        scale_v = max(np.abs(sv).max(), 1e-6)
        assert np.abs(bv - sv).max() <= 1e-3 * scale_v, (i, h, w)
        assert np.abs(br - sr).max() <= 1e-3 * max(np.abs(sr).max(), 1e-6), (i, h, w)
        assert stats[i]["status"] == 0
        if precond == 2 and min(h, w) > 2 and h * w > 64:
            # same hierarchy and V-cycle as the single-grid MG
            assert abs(stats[i]["iterations"] - st1["iterations"]) <= 2, (i, stats[i], st1)
        elif precond == 2:
            # too small to coarsen: the batch solves level 0 with the coarse
            # solver, the single grid with symmetric sweeps
            assert stats[i]["iterations"] <= max(8, 2 * st1["iterations"]), (i, stats[i], st1)
        else:
            assert abs(stats[i]["iterations"] - st1["iterations"]) <= max(3, 0.1 * st1["iterations"]), (i, stats[i], st1)


def test_batch_first_step_fields_bit_exact(pg):
    """With a zero velocity the CG is trivial (b = 0): the step reduces to
    the shared per-sample kernels, so batch and single grid agree exactly."""
    masks, vels, rhos, srcs = make_case(1)
    B = pg.Batch2d(DIMS)
    v = B.new_faces()
    rho = torch.from_numpy(B.pack_cells(rhos)).cuda()
    p = B.new_cells()
    cfg = pg.StepConfig(dt=0.5, source_enabled=False, walls_after_advect=True,
                        solver=pg.SolverConfig(rel_stop=True, rel_tol=1e-5))
    B.step(cfg, v, rho, p)
    for i, (h, w) in enumerate(DIMS):
        g = pg.Grid2d((h, w))
        gv, gr, gp = g.new_simplex_1(), pg.Simplex2(g, torch.from_numpy(rhos[i].copy()).cuda()), g.new_simplex_2()
        pg.step(g, cfg, gv, gr, gp)
        assert torch.equal(B.cells_of(rho, i), gr.data), i
        assert torch.equal(B.faces_of(v, i), gv.data), i


@pytest.mark.parametrize("precond", [0, 2])
def test_batch_graph_loop_equals_host_loop(pg, precond):
    lib = pg.load()
    masks, vels, rhos, srcs = make_case(2)
    outs = []
    for profiled in (False, True):
        B = pg.Batch2d(DIMS)
        B.set_solid_cells(masks)
        v = torch.from_numpy(B.pack_faces(vels)).cuda()
        rho = torch.from_numpy(B.pack_cells(rhos)).cuda()
        p = B.new_cells()
        lib.pg_profile_enable(int(profiled))
        try:
            st = B.step(config(pg, precond), v, rho, p)
        finally:
            lib.pg_profile_enable(0)
        outs.append((st, v.cpu(), p.cpu()))
    assert [s["iterations"] for s in outs[0][0]] == [s["iterations"] for s in outs[1][0]]
    assert torch.equal(outs[0][1], outs[1][1]) and torch.equal(outs[0][2], outs[1][2])


def test_batch_tiles_and_autotune(pg, tmp_path):
    masks, vels, rhos, srcs = make_case(3)
    cache = str(tmp_path / "tune.txt")
    B = pg.Batch2d(DIMS)
    shape = B.autotune(cache)
    assert shape[0] * shape[1] % 32 == 0 and shape[0] * shape[1] <= 256
    assert open(cache).read().split()[1:4] == [str(shape[0]), str(shape[1]), str(int(shape[2]))]
    B2 = pg.Batch2d(DIMS)
    assert B2.autotune(cache) == shape  # read back from the cache
    # every tile shape gives the same answer up to CG reduction order
    ref = None
    for tx, ty, fu in [(32, 8, True), (16, 16, False), (64, 2, True)]:
        B2.set_tile(tx, ty, fu)
        B2.set_solid_cells(masks)
        v = torch.from_numpy(B2.pack_faces(vels)).cuda()
        rho = torch.from_numpy(B2.pack_cells(rhos)).cuda()
        p = B2.new_cells()
        B2.step(config(pg, 1), v, rho, p)
        out = v.cpu().numpy()
        if ref is None:
            ref = out
        else:
            assert np.abs(out - ref).max() <= 1e-3 * np.abs(ref).max()


def test_batch_rejections(pg):
    from panopaea_gb300 import _native as N

    B = pg.Batch2d([(8, 8), (9, 7)])
    v, rho, p = B.new_faces(), B.new_cells(), B.new_cells()
    for solver in (pg.SolverConfig(precond=5), pg.SolverConfig(refine=2)):
        with pytest.raises(N.PgError) as ei:
            B.step(pg.StepConfig(source_enabled=False, solver=solver), v, rho, p)
        assert ei.value.status == N.PG_BAD_ARG
    with pytest.raises(N.PgError):
        pg.Batch2d([(1, 8)])


def test_batch_mg_projection_divergence(pg, oracle):
    """The batched multigrid configuration on 24 grids of 64..256 cells per
    side with solid circles (several grids have isolated fluid pockets):
    every grid converges to relative 1e-6 in a few iterations, and the
    projected velocity's divergence (FP64, oracle operator) is below 1e-5 of
    the right-hand side's max plus 4e-6 of max |u|: the batch solves in FP32
    without refinement, so the FP32 rounding of the pressure and of the
    velocity bounds what the projection can remove."""
    from panopaea_gb300 import workloads as W

    dims, masks, srcs = W.batch_grids(24, seed=11, sides=tuple(range(64, 257, 32)))
    B = pg.Batch2d(dims)
    B.set_solid_cells(masks)
    v, rho, p = B.new_faces(), B.new_cells(), B.new_cells()
    src = torch.from_numpy(B.pack_cells(srcs)).cuda()
    cfg = pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                        zero_solid_after_project=True,
                        solver=pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=1000))
    for _ in range(4):
        stats = B.step(cfg, v, rho, p, source_field=src)
    torch.cuda.synchronize()
    for i, d in enumerate(dims):
        assert stats[i]["status"] == 0 and stats[i]["iterations"] <= 30, (i, stats[i])
        fs = oracle.cell_mask_to_faces(masks[i])
        vel = B.faces_of(v, i).cpu().numpy().astype(np.float64)
        div = oracle.divergence_rhs(vel, d, fs)
        assert np.abs(div).max() <= 1e-5 * stats[i]["b_max"] + 4e-6 * np.abs(vel).max(), (i, d)


def test_batch_mg_long_run_converges(pg):
    """The 512-grid batch configuration for 12 steps with MG: every grid
    converges in every step (a single-component grid whose rounding-level
    inconsistent constant mode used to stall the solve at step 9)."""
    import torch

    from panopaea_gb300 import workloads as W

    dims, masks, srcs = W.batch_grids(512)
    B = pg.Batch2d(dims)
    B.set_solid_cells(masks)
    v, rho, p = B.new_faces(), B.new_cells(), B.new_cells()
    src = torch.from_numpy(B.pack_cells(srcs)).cuda()
    cfg = pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                        zero_solid_after_project=True,
                        solver=pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=400))
    for k in range(12):
        st = B.step(cfg, v, rho, p, source_field=src)
        bad = [(i, s["iterations"], s["status"]) for i, s in enumerate(st) if s["status"] != 0 or s["iterations"] > 12]
        assert not bad, (k, bad[:5])


@pytest.mark.parametrize("precond", [1, 2])
def test_batch_steps_against_fp64_oracle(pg, oracle, precond):
    """Each batched step against the oracle's all-FP64 step (FP64 fields,
    FP64 Jacobi-PCG to relative 1e-10) taken from the same input state (the
    batch's state after the previous step), on 6 grids of 64..192 cells per
    side with solid circles and boundary sources: the batch solves in FP32
    to relative 1e-6 without refinement, so its projected velocity may differ
    by the FP32 solve's error -- within 2e-4 of max |u| per grid (measured
    at most 6.5e-5) -- and the density, advected in FP32 by the previous
    velocity, by the FP32 rounding of back-traced positions of up to ~200
    cells (~1e-5 cells) times the sources' gradient -- within 2e-5 of max rho
    (measured at most 3.2e-6)."""
    from panopaea_gb300 import workloads as W

    dims, masks, srcs = W.batch_grids(6, seed=21, sides=tuple(range(64, 193, 32)))
    B = pg.Batch2d(dims)
    B.set_solid_cells(masks)
    v, rho, p = B.new_faces(), B.new_cells(), B.new_cells()
    src = torch.from_numpy(B.pack_cells(srcs)).cuda()
    cfg = pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                        zero_solid_after_project=True,
                        solver=pg.SolverConfig(precond=precond, rel_stop=True, rel_tol=1e-6, max_iter=5000))
    fss = [oracle.cell_mask_to_faces(m) for m in masks]
    worst_v = worst_r = 0.0
    for step in range(3):
        torch.cuda.synchronize()
        ins = [(B.faces_of(v, i).cpu().numpy().astype(np.float64), B.cells_of(rho, i).cpu().numpy().astype(np.float64),
                B.cells_of(p, i).cpu().numpy().astype(np.float64)) for i in range(len(dims))]
        st = B.step(cfg, v, rho, p, source_field=src)
        torch.cuda.synchronize()
        for i, d in enumerate(dims):
            vel, r64, p64 = ins[i]
            prm = oracle.step_params(dt=0.5, buoyancy=1.0, walls_after_advect=True, zero_solid_after_project=True,
                                     precond=1, rel_stop=True, rel_tol=1e-10, max_iter=100000,
                                     source_field=srcs[i].astype(np.float64))
            so = oracle.step(vel, r64, p64, d, prm, fss[i])
            assert so.converged and st[i]["status"] == 0, (step, i)
            gv = B.faces_of(v, i).cpu().numpy().astype(np.float64)
            gr = B.cells_of(rho, i).cpu().numpy().astype(np.float64)
            ev = np.abs(gv - vel).max() / max(np.abs(vel).max(), 1e-30)
            er = np.abs(gr - r64).max() / max(np.abs(r64).max(), 1e-30)
            worst_v, worst_r = max(worst_v, ev), max(worst_r, er)
            assert ev <= 2e-4 and er <= 2e-5, (step, i, d, ev, er)
    print("worst velocity %.2e density %.2e" % (worst_v, worst_r))
