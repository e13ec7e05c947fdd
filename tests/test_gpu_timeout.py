"""The bounded device-side waits give up cleanly.

The only waits inside this library's kernels are the TMA pipeline-stage
waits of the 3D z-marching kernels (the CG SpMV, the multigrid fine-level
pairs, the refinement residual): one thread polls an mbarrier with a poll
and time budget; when it gives up, the block waits (bounded) for the copies
it has in flight, sets PG_TIMEOUT and stops the solve.  The test hook
pg_debug_set_stage_wait_polls(0) makes every stage wait give up at once --
no fault, no hang: every copy that was issued still lands -- so the whole
path runs and its status is checked; the next solve, with the budget
restored, succeeds."""

import numpy as np
import pytest

from conftest import rng
from test_gpu_ops import faces, host, make_grid

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precond", [0, 1, 2])
def test_stage_wait_give_up_reports_timeout(pg, oracle, precond):
    from panopaea_gb300 import _native as N

    lib = N.load()
    dims = (24, 40, 64)  # rows of a multiple of 16 cells: the TMA-staged kernels run
    r = rng(31 + precond)
    vel = oracle.walls(r.standard_normal(oracle.num_faces(dims)).astype(np.float32), dims)
    g = make_grid(pg, dims)
    b = g.new_simplex_2()
    g.divergence_rhs(b, faces(pg, g, vel))
    x = g.new_simplex_2()
    cfg = pg.SolverConfig(precond=precond, rel_stop=True, rel_tol=1e-5, max_iter=20000)
    default = lib.pg_debug_stage_wait_polls_default()
    assert default > 0
    assert lib.pg_debug_set_stage_wait_polls(0) == N.PG_OK
    try:
        with pytest.raises(N.PgError) as ei:
            pg.solve_pressure(g, x, b, 0.5, cfg)
        assert ei.value.status == N.PG_TIMEOUT
        assert "PG_TIMEOUT" in str(ei.value) or lib.pg_status_string(N.PG_TIMEOUT) == b"PG_TIMEOUT"
    finally:
        assert lib.pg_debug_set_stage_wait_polls(default) == N.PG_OK
    st = pg.solve_pressure(g, x, b, 0.5, cfg)
    assert st["status"] == 0, st
    bh = host(b).astype(np.float64)
    true_r = np.abs(bh - oracle.laplacian(host(x).astype(np.float64), 0.5, dims)).max()
    assert true_r <= 20e-5 * np.abs(bh).max()
