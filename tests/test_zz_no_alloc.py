"""pg_pcg_noalloc_f32 -- the PCG for callers that cannot allocate device
memory (their device memory is owned by a host framework's pool or arena,
or they run time-critical loops where cudaMalloc/cudaFree would synchronise
the device) -- called through the C ABI and checked against pg_pcg_f32 on
the same inputs, on two calls in a row.  Its scratch is a fixed device array
inside the library, shared by every call.

This file is named so that pytest collects it last."""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

# Face-open bits of the allocation-free entry point's geometry argument.
XLO, XHI, YLO, YHI, ZLO, ZHI = 1, 2, 4, 8, 16, 32


def face_bits(cell_solid):
    """One byte per cell: a face is open iff it is interior and neither
    adjacent cell is solid."""
    cs = np.asarray(cell_solid, bool)
    if cs.ndim == 2:
        cs = cs[None]
        nd = 2
    else:
        nd = 3
    d, h, w = cs.shape
    f = np.zeros(cs.shape, np.uint8)
    fluid = ~cs
    for ax, (lo, hi) in zip((2, 1, 0), ((XLO, XHI), (YLO, YHI), (ZLO, ZHI))):
        if nd == 2 and ax == 0:
            continue
        n = cs.shape[ax]
        idx = np.arange(n).reshape([-1 if a == ax else 1 for a in range(3)])
        prev = np.roll(fluid, 1, axis=ax)
        nxt = np.roll(fluid, -1, axis=ax)
        f |= np.where((idx > 0) & fluid & prev, lo, 0).astype(np.uint8)
        f |= np.where((idx < n - 1) & fluid & nxt, hi, 0).astype(np.uint8)
    return f.reshape(cs.shape if nd == 3 else cs.shape[1:])


def ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def rhs(pg, grid, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    vel = pg.Simplex1(grid, torch.randn(grid.num_elem_1(), device="cuda", generator=g))
    grid.walls(vel)
    b = grid.new_simplex_2()
    grid.divergence_rhs(b, vel)
    return b


def solve_reference_entry(pg, grid, b, precond, max_iter, thr, dt):
    x, r, aux, s = (grid.new_simplex_2() for _ in range(4))
    pre = pg.JACOBI if precond else pg.IDENTITY
    st = pg.precond_conjugate_gradient(pre, x, b, max_iter, thr, r, aux, s, pg.LaplacianOperator(grid, dt))
    torch.cuda.synchronize()
    return [t.data.clone() for t in (x, r, aux, s)], st


def solve_noalloc(lib, N, dims, flags_dev, b, precond, max_iter, thr, dt):
    nd = len(dims)
    d, h, w = (1,) + tuple(dims) if nd == 2 else tuple(dims)
    x, r, aux, s = (torch.zeros(dims, dtype=torch.float32, device="cuda") for _ in range(4))
    st = N.PcgStats()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.pg_pcg_noalloc_f32(nd, d, h, w, ptr(flags_dev), precond, ptr(x), ptr(b.data), max_iter, C.c_double(thr),
                                ptr(r), ptr(aux), ptr(s), C.c_double(dt), stream, C.byref(st))
    torch.cuda.synchronize()
    return rc, [x, r, aux, s], st.as_dict()


@pytest.mark.parametrize("dims,masked,precond", [((96, 80), False, 0), ((64, 64), True, 1), ((24, 28, 32), True, 0),
                                                 ((40, 40, 40), False, 1)])
def test_noalloc_matches_pcg_on_two_calls(dims, masked, precond):
    import panopaea_gb300 as pg
    from panopaea_gb300 import _native as N

    lib = pg.load()
    grid = pg.Grid2d(dims) if len(dims) == 2 else pg.Grid3d(dims)
    flags_dev = None
    if masked:
        rng = np.random.default_rng(7)
        cs = (rng.random(dims) < 0.08).astype(np.uint8)
        grid.set_solid_cells(cs)
        flags_dev = torch.from_numpy(face_bits(cs)).cuda()
    dt = 0.5
    for call, seed in enumerate((11, 12)):  # two calls in a row share the scratch
        b = rhs(pg, grid, seed)
        thr = 1e-5 * float(b.data.abs().max())
        want, st_want = solve_reference_entry(pg, grid, b, precond, 5000, thr, dt)
        rc, got, st_got = solve_noalloc(lib, N, dims, flags_dev, b, precond, 5000, thr, dt)
        assert rc == N.PG_OK, (call, lib.pg_last_error())
        assert st_got["status"] == st_want["status"] == N.PG_OK
        assert st_got["iterations"] == st_want["iterations"], call
        for a, e in zip(got, want):
            torch.testing.assert_close(a, e, rtol=1e-6, atol=1e-6 * float(e.abs().max()) + 1e-30)


def test_noalloc_max_iterations_tail_and_rejections():
    import panopaea_gb300 as pg
    from panopaea_gb300 import _native as N

    lib = pg.load()
    dims = (20, 17)
    grid = pg.Grid2d(dims)
    b = rhs(pg, grid, 3)
    want, st_want = solve_reference_entry(pg, grid, b, 0, 7, 1e-30, 1.0)
    rc, got, st_got = solve_noalloc(lib, N, dims, None, b, 0, 7, 1e-30, 1.0)
    assert rc == N.PG_NOT_CONVERGED and st_got["iterations"] == 7 == st_want["iterations"]
    for a, e in zip(got, want):
        torch.testing.assert_close(a, e, rtol=1e-6, atol=1e-6 * float(e.abs().max()) + 1e-30)
    # a grid beyond the fixed scratch is refused before any GPU work
    big = torch.zeros(4, device="cuda")
    st = N.PcgStats()
    rc = lib.pg_pcg_noalloc_f32(2, 1, 1025, 1024, None, 0, ptr(big), ptr(big), 10, C.c_double(1e-6), ptr(big),
                                ptr(big), ptr(big), C.c_double(1.0), None, C.byref(st))
    assert rc == N.PG_BAD_ARG and b"1048576" in lib.pg_last_error()
    rc = lib.pg_pcg_noalloc_f32(2, 2, 8, 8, None, 0, ptr(big), ptr(big), 10, C.c_double(1e-6), ptr(big),
                                ptr(big), ptr(big), C.c_double(1.0), None, C.byref(st))
    assert rc == N.PG_BAD_ARG
