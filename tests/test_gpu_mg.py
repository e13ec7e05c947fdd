"""Multigrid-preconditioned CG (an extension behind pcg.rs:4-6
`Preconditioner`): converges in a grid-size-independent handful of
iterations, to the same solution as the oracle's CG, with obstacles, odd and
anisotropic shapes, in 2D and 3D."""

import numpy as np
import pytest

from conftest import rng, seed_of
from test_gpu_ops import cells, faces, host, make_grid

pytestmark = pytest.mark.gpu


def solve_case(pg, oracle, dims, obstacle, precond, tol, refine=0):
    r = rng(seed_of(dims, obstacle))
    nf = oracle.num_faces(dims)
    cs = None
    g = make_grid(pg, dims)
    if obstacle:
        idx = np.indices(dims).astype(np.float64)
        ctr = np.array([(n - 1) / 2 for n in dims]).reshape((-1,) + (1,) * len(dims))
        cs = (((idx - ctr) ** 2).sum(0) < (min(dims) / 5.0) ** 2).astype(np.uint8)
        g.set_solid_cells(cs)
    fs = oracle.cell_mask_to_faces(cs) if obstacle else None
    vel = oracle.walls(r.standard_normal(nf).astype(np.float32), dims)
    b = g.new_simplex_2()
    g.divergence_rhs(b, faces(pg, g, vel))
    x = g.new_simplex_2()
    st = pg.solve_pressure(g, x, b, 0.5, pg.SolverConfig(precond=precond, rel_stop=True, rel_tol=tol,
                                                         max_iter=20000, refine=refine))
    bh = host(b).astype(np.float64)
    xh = host(x).astype(np.float64)
    true_r = np.abs(bh - oracle.laplacian(xh, 0.5, dims, fs)).max() / np.abs(bh).max()
    return st, xh, bh, true_r, fs


@pytest.mark.parametrize("dims", [(64, 64), (256, 256), (200, 131), (33, 47, 29), (64, 64, 64), (128, 128, 128),
                                  (16, 64, 40), (256, 16)])
@pytest.mark.parametrize("obstacle", [False, True])
def test_mgpcg_converges_fast(pg, oracle, dims, obstacle):
    st, x, b, true_r, fs = solve_case(pg, oracle, dims, obstacle, 2, 1e-5)
    assert st["status"] == 0, st
    assert st["iterations"] <= 30, st
    # FP32 storage: the true residual is within the FP32 floor of x
    floor = 16 * 2.0 ** -24 * 0.5 * np.abs(x).max() / np.abs(b).max()
    assert true_r <= 20e-5 + floor


@pytest.mark.parametrize("dims", [(128, 128), (48, 40, 36)])
def test_mgpcg_matches_plain_cg_solution(pg, oracle, dims):
    """Same projected velocity as plain CG run to the same tolerance (the
    pressure is unique up to a constant; its gradient on open faces is
    unique -- across closed faces it sees the constant, since solid cells
    stay at 0)."""
    st_mg, x_mg, b, _, fs = solve_case(pg, oracle, dims, True, 2, 1e-7, refine=4)
    st_cg, x_cg, _, _, _ = solve_case(pg, oracle, dims, True, 0, 1e-7, refine=4)
    assert st_mg["status"] == 0 and st_cg["status"] == 0
    assert st_mg["iterations"] * 5 < st_cg["iterations"]
    g_mg = oracle.mask_faces(oracle.derivative_0_dual(x_mg, dims), fs)
    g_cg = oracle.mask_faces(oracle.derivative_0_dual(x_cg, dims), fs)
    assert np.abs(g_mg - g_cg).max() <= 1e-4 * np.abs(g_cg).max()


@pytest.mark.parametrize("dims", [(256, 256), (96, 96, 96)])
def test_refined_mgpcg_reaches_1e6(pg, oracle, dims):
    st, x, b, true_r, _ = solve_case(pg, oracle, dims, True, 2, 1e-6, refine=5)
    assert st["status"] == 0 and st["true_residual_max"] <= 1e-6 * st["b_max"], st
    assert st["iterations"] <= 60


def test_mg_rejected_for_f64(pg):
    """MG is an FP32 preconditioner: an f64 step asking for it is refused."""
    import torch

    from panopaea_gb300 import _native as N

    g = pg.Grid2d((16, 16))
    vel, rho, p = g.new_simplex_1(torch.float64), g.new_simplex_2(torch.float64), g.new_simplex_2(torch.float64)
    rho.data[4, 4] = 1.0
    vel.data[40] = 1.0
    cfg = pg.StepConfig(dt=0.5, source_enabled=False, solver=pg.SolverConfig(precond=2, rel_stop=True))
    with pytest.raises(N.PgError) as ei:
        pg.step(g, cfg, vel, rho, p)
    assert ei.value.status == N.PG_BAD_ARG
    # b = 0 takes the early out before any preconditioner runs
    st = pg.solve_pressure(g, g.new_simplex_2(), g.new_simplex_2(), 1.0, pg.SolverConfig(precond=2, rel_stop=True))
    assert st["status"] == 0 and st["iterations"] == 0


def test_profile_counters(pg):
    lib = pg.load()
    import ctypes as C

    n0 = lib.pg_kernel_launches()
    g = pg.Grid3d((8, 8, 8))
    lib.pg_profile_reset()
    lib.pg_profile_enable(1)
    out = g.new_simplex_2()
    g.laplacian(out, g.new_simplex_2(), 1.0)
    lib.pg_profile_enable(0)
    assert lib.pg_kernel_launches() > n0
    names = [lib.pg_profile_kind_name(k).decode() for k in range(lib.pg_profile_num_kinds())]
    t = C.c_double()
    n = C.c_int64()
    lib.pg_profile_read(names.index("dec_op"), C.byref(t), C.byref(n))
    assert n.value >= 1 and t.value > 0
    ta, na = C.c_double(), C.c_int64()
    lib.pg_profile_read_active(names.index("dec_op"), C.byref(ta), C.byref(na))
    assert 1 <= na.value <= n.value and 0 < ta.value <= t.value


def test_profile_active_skips_exit_at_entry_launches(pg, oracle):
    """The host-polled CG loop (profiling mode) launches iterations past its
    stop test; they exit at entry, and the active count leaves them out."""
    import ctypes as C

    lib = pg.load()
    names = [lib.pg_profile_kind_name(k).decode() for k in range(lib.pg_profile_num_kinds())]
    lib.pg_profile_reset()
    lib.pg_profile_enable(1)
    try:
        st, *_ = solve_case(pg, oracle, (192, 192, 192), False, 2, 1e-5)  # real launches >> exit-at-entry ones
    finally:
        lib.pg_profile_enable(0)
    k = names.index("cg_update")  # a plain kernel: its exit-at-entry launches take microseconds
    t, n, ta, na = C.c_double(), C.c_int64(), C.c_double(), C.c_int64()
    lib.pg_profile_read(k, C.byref(t), C.byref(n))
    lib.pg_profile_read_active(k, C.byref(ta), C.byref(na))
    assert st["status"] == 0
    assert na.value == st["iterations"] <= n.value, (na.value, n.value, st["iterations"])


@pytest.mark.parametrize("precond", [0, 1, 2])
def test_graph_loop_equals_stream_loop(pg, oracle, precond):
    """The device-side CUDA-graph loop and the host-polled stream loop run
    the same deterministic kernels: identical iterates, bit for bit."""
    lib = pg.load()
    dims = (40, 36, 44)
    outs = []
    for profiled in (False, True):  # profiling forces the stream loop
        lib.pg_profile_enable(int(profiled))
        try:
            st, x, b, true_r, _ = solve_case(pg, oracle, dims, True, precond, 1e-6)
        finally:
            lib.pg_profile_enable(0)
        outs.append((st, x))
    (s0, x0), (s1, x1) = outs
    assert s0["status"] == s1["status"] == 0
    assert s0["iterations"] == s1["iterations"]
    assert np.array_equal(x0, x1)


@pytest.mark.parametrize("dims", [(256, 256), (64, 64, 64)])
def test_double_float_refinement_matches_native_fp64(pg, oracle, dims):
    """The double-float (FP32-pair) residual / accumulation reaches the same
    FP64 tolerance as native FP64 arithmetic, with the same solution to
    FP32 accuracy."""
    res = []
    for native in (False, True):
        r = rng(seed_of(dims, "df"))
        nf = oracle.num_faces(dims)
        vel = oracle.walls(r.standard_normal(nf).astype(np.float32), dims)
        g = make_grid(pg, dims)
        b = g.new_simplex_2()
        g.divergence_rhs(b, faces(pg, g, vel))
        x = g.new_simplex_2()
        st = pg.solve_pressure(g, x, b, 0.5, pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=2000,
                                                             refine=5, fp64_native=native))
        assert st["status"] == 0 and st["true_residual_max"] <= 1e-6 * st["b_max"], (native, st)
        bh = host(b).astype(np.float64)
        xh = host(x).astype(np.float64)
        # independent FP64 check of the returned (FP32-rounded) solution
        tr = np.abs(bh - oracle.laplacian(xh, 0.5, dims)).max() / np.abs(bh).max()
        res.append((xh - xh.mean(), tr))
    (xa, ta), (xb, tb) = res
    assert np.abs(xa - xb).max() <= 1e-5 * np.abs(xb).max()


@pytest.mark.parametrize("dims", [(64, 160), (24, 40, 32)])
def test_mg_with_isolated_pockets(pg, oracle, dims):
    """Solid walls cutting off small fluid pockets: on a pocket the
    right-hand side sums to zero only up to FP32 rounding, which a plain
    V-cycle turns into a diverging search direction.  With the pocket
    projection the MG-PCG converges in a few iterations, agrees with
    Jacobi-PCG, and leaves a divergence-free projection, in 2D and 3D."""
    r = rng(seed_of(dims))
    cs = np.zeros(dims, np.uint8)
    if len(dims) == 2:
        cs[10:22, 20] = cs[10:22, 30] = 1          # a 12 x 9 pocket
        cs[10, 20:31] = cs[21, 20:31] = 1
        cs[40, :] = 1                              # a wall cutting the grid in two
        cs[50:53, 100:103] = 1
    else:
        cs[4:12, 5:15, 6:16] = 1                   # a hollow box: its inside is a pocket
        cs[5:11, 6:14, 7:15] = 0
        cs[:, 30, :] = 1                           # a wall cutting the grid in two
    fs = oracle.cell_mask_to_faces(cs)
    g = make_grid(pg, dims)
    g.set_solid_cells(cs)
    nf = oracle.num_faces(dims)
    vel = oracle.mask_faces(oracle.walls(r.standard_normal(nf), dims), fs).astype(np.float32)
    b = oracle.divergence_rhs(vel.astype(np.float64), dims, fs).astype(np.float32)
    out = {}
    for precond in (1, 2):
        x = g.new_simplex_2()
        st = pg.solve_pressure(g, x, cells(pg, g, b), 1.0,
                               pg.SolverConfig(precond=precond, rel_stop=True, rel_tol=1e-6, max_iter=20000, refine=4))
        assert st["status"] == 0, (precond, st)
        assert st["true_residual_max"] <= 1e-6 * st["b_max"]
        out[precond] = (st, host(x).astype(np.float64))
    assert out[2][0]["iterations"] <= 40
    # the solutions agree up to a constant per fluid component: compare gradients
    ga = oracle.mask_faces(oracle.derivative_0_dual(out[1][1], dims), fs)
    gb = oracle.mask_faces(oracle.derivative_0_dual(out[2][1], dims), fs)
    assert np.abs(ga - gb).max() <= 1e-4 * np.abs(ga).max()
    # the whole step on the same mask with MG stays finite and divergence-free
    gv = faces(pg, g, vel)
    gr, gp = cells(pg, g, r.random(dims).astype(np.float32)), g.new_simplex_2()
    cfg = pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                        zero_solid_after_project=True,
                        solver=pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=20000, refine=4))
    for _ in range(4):
        st = pg.step(g, cfg, gv, gr, gp)
        assert st["status"] == 0
    v = host(gv).astype(np.float64)
    assert np.isfinite(v).all()
    assert np.abs(oracle.divergence_rhs(v, dims, fs)).max() <= 1e-5 * st["b_max"] + 1e-6 * np.abs(v).max()


def _launches(lib, fn, kind):
    import ctypes as C

    names = [lib.pg_profile_kind_name(k).decode() for k in range(lib.pg_profile_num_kinds())]
    lib.pg_profile_reset()
    lib.pg_profile_enable(1)
    try:
        out = fn()
    finally:
        lib.pg_profile_enable(0)
    t, n = C.c_double(), C.c_int64()
    lib.pg_profile_read(names.index(kind), C.byref(t), C.byref(n))
    return out, n.value


def _pair_launches(lib, fn):
    return _launches(lib, fn, "mg_pair")


@pytest.mark.parametrize("dims", [(20, 24, 80), (37, 19, 48), (64, 64, 64)])
@pytest.mark.parametrize("nsmooth", [1, 2, 3])
def test_fused_pairs_equal_half_sweeps(pg, oracle, dims, nsmooth, monkeypatch):
    """The fine-level fused red-black pairs (TMA-staged z-march, rows of a
    multiple of 16 cells) compute the same V-cycle as separate half-sweeps:
    the same iterations and the same solution, on ragged tiles, with an
    obstacle, for 1-3 sweeps."""
    lib = pg.load()
    r = rng(seed_of(dims, nsmooth))
    idx = np.indices(dims).astype(np.float64)
    ctr = np.array([(n - 1) / 2 for n in dims]).reshape((-1, 1, 1, 1))
    cs = (((idx - ctr) ** 2).sum(0) < (min(dims) / 4.0) ** 2).astype(np.uint8)
    nf = oracle.num_faces(dims)
    vel = oracle.walls(r.standard_normal(nf).astype(np.float32), dims)
    res = {}
    for pairs in ("1", "0"):
        monkeypatch.setenv("PG_MG_PAIRS", pairs)
        g = make_grid(pg, dims)  # a new grid builds its hierarchy under the switch
        g.set_solid_cells(cs)
        b = g.new_simplex_2()
        g.divergence_rhs(b, faces(pg, g, vel))
        x = g.new_simplex_2()
        cfg = pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=2000, refine=4, mg_smooth=nsmooth)
        st, n_pair = _pair_launches(lib, lambda: pg.solve_pressure(g, x, b, 0.5, cfg))
        assert st["status"] == 0 and st["true_residual_max"] <= 1e-6 * st["b_max"], (pairs, st)
        res[pairs] = (st, host(x).astype(np.float64), n_pair)
    (s1, x1, n1), (s0, x0, n0) = res["1"], res["0"]
    assert n1 > 0 and n0 == 0, (n1, n0)
    assert s1["iterations"] == s0["iterations"]
    assert np.abs(x1 - x0).max() <= 1e-6 * np.abs(x0).max()


@pytest.mark.parametrize("dims", [(224, 96), (48, 40, 64)])
@pytest.mark.parametrize("offset", [1e-9, 1e-8])
def test_mg_one_component_constant_mode(pg, oracle, dims, offset):
    """A closed grid's operator is singular (constants); FP32 rounding leaves
    a right-hand side a little inconsistent (here: a consistent divergence
    plus offset * max|b| on every cell, the size FP32 sums leave).  The
    V-cycle's coarse sweeps amplify that constant part of r into z; unless
    z's mean on the fluid is removed, it swamps A p near the 1e-6 target and
    plain MG-PCG stalls or breaks down.  With the lazy projection the solve
    converges in a few iterations, without refinement."""
    r = rng(seed_of(dims, offset))
    nf = oracle.num_faces(dims)
    vel = oracle.walls(r.standard_normal(nf), dims)
    b64 = oracle.divergence_rhs(vel, dims)
    b = (b64 + offset * np.abs(b64).max()).astype(np.float32)
    g = make_grid(pg, dims)
    x = g.new_simplex_2()
    st = pg.solve_pressure(g, x, cells(pg, g, b), 1.0,
                           pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=500))
    assert st["status"] == 0 and st["iterations"] <= 12, st
    xh = host(x).astype(np.float64)
    bh = b.astype(np.float64)
    true_r = np.abs(bh - oracle.laplacian(xh, 1.0, dims)).max() / np.abs(bh).max()
    floor = 16 * 2.0 ** -24 * np.abs(xh).max() / np.abs(bh).max()  # FP32 storage of x
    assert true_r <= 5e-6 + floor, (true_r, floor)


@pytest.mark.parametrize("dims", [(20, 24, 80), (64, 64, 64), (96, 40, 112), (128, 128, 128)])
def test_tma_restriction_equals_plain_kernel(pg, oracle, dims, monkeypatch):
    """The fine-level restriction of 3D grids with even sides, TMA-staged
    (a 64 x 16 fine tile per block, coarse planes walked in z), against the
    plain kernel (PG_MG_RESTRICT_TMA=0): every child residual is formed and
    summed in the same order, so the solves are bit-identical -- on ragged
    tiles, with an obstacle."""
    r = rng(seed_of(dims, "restrict"))
    idx = np.indices(dims).astype(np.float64)
    ctr = np.array([(n - 1) / 2 for n in dims]).reshape((-1, 1, 1, 1))
    cs = (((idx - ctr) ** 2).sum(0) < (min(dims) / 4.0) ** 2).astype(np.uint8)
    nf = oracle.num_faces(dims)
    vel = oracle.walls(r.standard_normal(nf).astype(np.float32), dims)
    res = {}
    for on in ("1", "0"):
        monkeypatch.setenv("PG_MG_RESTRICT_TMA", on)
        g = make_grid(pg, dims)  # a new grid builds its hierarchy under the switch
        g.set_solid_cells(cs)
        b = g.new_simplex_2()
        g.divergence_rhs(b, faces(pg, g, vel))
        x = g.new_simplex_2()
        st = pg.solve_pressure(g, x, b, 0.5, pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6,
                                                             max_iter=2000, refine=4))
        assert st["status"] == 0 and st["true_residual_max"] <= 1e-6 * st["b_max"], (on, st)
        res[on] = (st, host(x))
    (s1, x1), (s0, x0) = res["1"], res["0"]
    assert s1["iterations"] == s0["iterations"]
    assert np.array_equal(x1, x0)


@pytest.mark.parametrize("dims", [(64, 64, 64), (96, 64, 80), (48, 40, 64), (20, 24, 80), (128, 128, 128)])
@pytest.mark.parametrize("nsmooth", [1, 2])
def test_cluster_tail_equals_per_level_kernels(pg, oracle, dims, nsmooth, monkeypatch):
    """The cluster tail (levels of at most 32768 cells in one thread-block
    cluster: z slabs per rank in distributed shared memory, the smallest
    levels in rank 0) computes every cell with the per-level kernels' and the
    single-block tail's formulas: the solves are bit-identical with
    PG_MG_CTAIL=0, on shapes whose slabs leave ranks empty, with an
    obstacle, for 1 and 2 sweeps."""
    lib = pg.load()
    r = rng(seed_of(dims, nsmooth, "ctail"))
    idx = np.indices(dims).astype(np.float64)
    ctr = np.array([(n - 1) / 2 for n in dims]).reshape((-1, 1, 1, 1))
    cs = (((idx - ctr) ** 2).sum(0) < (min(dims) / 4.0) ** 2).astype(np.uint8)
    nf = oracle.num_faces(dims)
    vel = oracle.walls(r.standard_normal(nf).astype(np.float32), dims)
    res = {}
    for on in ("1", "0"):
        monkeypatch.setenv("PG_MG_CTAIL", on)
        g = make_grid(pg, dims)  # a new grid builds its hierarchy under the switch
        g.set_solid_cells(cs)
        b = g.new_simplex_2()
        g.divergence_rhs(b, faces(pg, g, vel))
        x = g.new_simplex_2()
        cfg = pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=2000, refine=4, mg_smooth=nsmooth)
        st, n_coarse = _launches(lib, lambda: pg.solve_pressure(g, x, b, 0.5, cfg), "mg_smooth_coarse")
        assert st["status"] == 0 and st["true_residual_max"] <= 1e-6 * st["b_max"], (on, st)
        res[on] = (st, host(x), n_coarse)
    (s1, x1, n1), (s0, x0, n0) = res["1"], res["0"]
    assert n1 < n0, (n1, n0)  # the cluster took over the half-sweeps of its top level
    assert s1["iterations"] == s0["iterations"]
    assert np.array_equal(x1, x0)


def test_vcycle_graph_timing(pg):
    """pg_debug_mg_vcycle_ms replays one V-cycle and its coarse part as CUDA
    graphs: both times are positive and the coarse part is the smaller."""
    import ctypes as C

    lib = pg.load()
    g = make_grid(pg, (64, 64, 64))
    full, coarse = C.c_double(), C.c_double()
    assert lib.pg_debug_mg_vcycle_ms(g.handle, C.c_double(0.5), 2, 5, C.byref(full), C.byref(coarse)) == 0
    assert 0.0 < coarse.value < full.value, (full.value, coarse.value)
