"""The oracle against the reference's own golden vectors, and its internal
consistency (CPU only).

Golden vectors: panopaea/src/dec/grid.rs:428-482 (grid_2d_divergence) and
:484-515 (grid_2d_laplacian), extracted verbatim by tests/golden/make_golden.py.
"""

import numpy as np
import pytest

from conftest import rng


def _div_case(g, dtype=np.float32):
    d = g["grid_2d_divergence"]
    vel = np.concatenate([np.array(d["velocities_y"], dtype).ravel(), np.array(d["velocities_x"], dtype).ravel()])
    return vel, np.array(d["div_ref"], dtype).reshape(5, 5), d["eps"]


def test_golden_divergence(golden, oracle):
    """grid.rs:467-481: hodge_1_dual then derivative_1_primal, f32, eps 1e-3."""
    vel, ref, eps = _div_case(golden)
    div = oracle.derivative_1_primal(oracle.hodge_1_dual(vel, (5, 5)), (5, 5))
    assert np.all(np.abs(div - ref) < eps)
    # fused RHS form: b = -div
    b = oracle.divergence_rhs(vel, (5, 5))
    assert np.array_equal(b, -div)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_golden_laplacian(golden, oracle, dtype):
    """grid.rs:494-514: *2, d0dual, *1^-1, d1primal composed, eps 1e-3."""
    lcase = golden["grid_2d_laplacian"]
    p = np.array(lcase["faces_primal"], dtype)
    ref = np.array(lcase["laplacian_ref"], dtype).reshape(3, 3)
    edges = oracle.derivative_0_dual(p.copy(), (3, 3))
    lap = oracle.derivative_1_primal(oracle.hodge_1_dual(edges, (3, 3)), (3, 3))
    assert np.all(np.abs(lap - ref) < lcase["eps"])
    # The fused closure (dt = 1) is the same operator, bit for bit.
    assert np.array_equal(oracle.laplacian(p, 1.0, (3, 3)), lap)


def test_hodge_pair_composes_to_minus_identity(oracle):
    """grid.rs:206-238: *1 flips vx, *1^-1 flips vy, so *1 *1^-1 = -1 (2D DEC)."""
    r = rng(1)
    dims = (7, 5)
    v = r.standard_normal(oracle.num_faces(dims)).astype(np.float32)
    assert np.array_equal(oracle.hodge_1_primal(oracle.hodge_1_dual(v, dims), dims), -v)


@pytest.mark.parametrize("dims", [(6, 9), (4, 5, 7)])
def test_laplacian_symmetric_and_nullspace(oracle, dims):
    r = rng(2)
    nf = oracle.num_faces(dims)
    solid = (r.random(nf) < 0.1).astype(np.uint8)
    u = r.standard_normal(dims)
    v = r.standard_normal(dims)
    au = oracle.laplacian(u, 0.5, dims, solid)
    av = oracle.laplacian(v, 0.5, dims, solid)
    assert abs(np.vdot(v, au) - np.vdot(u, av)) < 1e-9 * np.abs(au).sum()
    assert np.vdot(u, au) > 0
    # constants are in the null space (pure Neumann walls)
    assert np.abs(oracle.laplacian(np.ones(dims), 0.5, dims, solid)).max() == 0


@pytest.mark.parametrize("dims", [(12, 10), (6, 5, 7)])
def test_laplacian_equals_neg_div_grad(oracle, dims):
    """A p = -div(M grad p) * dt, from the separately restated operators."""
    r = rng(3)
    nf = oracle.num_faces(dims)
    solid = (r.random(nf) < 0.15).astype(np.uint8)
    p = r.standard_normal(dims)
    e = oracle.mask_faces(oracle.derivative_0_dual(p, dims), solid)  # e = -grad p on open interior faces
    b = oracle.divergence_rhs(e, dims)  # -div e
    lap = oracle.laplacian(p, 1.0, dims, solid)
    np.testing.assert_allclose(-b, lap, rtol=1e-12, atol=1e-12)


def test_pcg_converges_and_projection_is_divergence_free(oracle):
    r = rng(4)
    dims = (24, 20)
    dt = 0.5
    vel = r.standard_normal(oracle.num_faces(dims))
    vel = oracle.walls(vel, dims)
    b = oracle.divergence_rhs(vel, dims)
    thr = 1e-10 * np.abs(b).max()
    x, rr, aux, s, it, res, conv = oracle.pcg(b, dt, dims, 10000, thr)
    assert conv and res < thr
    # true residual
    assert np.abs(b - oracle.laplacian(x, dt, dims)).max() < 10 * thr
    out = oracle.project(vel, x, dt, dims)
    assert np.abs(oracle.divergence_rhs(out, dims)).max() < 10 * thr


def test_pcg_reference_semantics(oracle):
    """Early exit leaves x = 0; max_iterations bounds the operator count."""
    dims = (8, 8)
    b = np.zeros(dims)
    b[3, 3], b[4, 4] = 1.0, -1.0
    x, _, _, _, it, res, conv = oracle.pcg(b, 1.0, dims, 100, 2.0)
    assert it == 0 and conv and np.all(x == 0)
    x, _, _, _, it, res, conv = oracle.pcg(b, 1.0, dims, 3, 1e-12)
    assert it == 3 and not conv


def test_jacobi_matches_identity_solution(oracle):
    r = rng(5)
    dims = (5, 9, 8)
    vel = oracle.walls(r.standard_normal(oracle.num_faces(dims)), dims)
    b = oracle.divergence_rhs(vel, dims)
    thr = 1e-11 * np.abs(b).max()
    x0 = oracle.pcg(b, 0.5, dims, 5000, thr, precond=0)[0]
    x1, _, _, _, it1, _, conv1 = oracle.pcg(b, 0.5, dims, 5000, thr, precond=1)
    assert conv1
    np.testing.assert_allclose(x0 - x0.mean(), x1 - x1.mean(), atol=1e-8)


def test_advect_zero_velocity_is_identity(oracle):
    """Identity except the last row/column per axis: the clamp to n - 1.00001
    (dec_fluid.rs:194-195) blends 1e-5 of the neighbour in there."""
    r = rng(6)
    for dims in [(9, 7), (4, 6, 5)]:
        q = r.standard_normal(dims)
        vel = np.zeros(oracle.num_faces(dims))
        out = oracle.advect(q, 0.7, vel, dims)
        inner = tuple(slice(0, n - 1) for n in dims)
        assert np.array_equal(out[inner], q[inner])
        np.testing.assert_allclose(out, q, atol=1e-4 * np.abs(q).max())
        assert not np.array_equal(out, q)
        f = r.standard_normal(oracle.num_faces(dims))
        assert np.array_equal(oracle.advect_mac(f, 0.7, vel, dims), f)


def test_advect_integer_shift(oracle):
    """A uniform velocity of exactly one cell per step shifts the field."""
    h, w = 6, 9
    q = rng(7).standard_normal((h, w))
    vel = np.zeros(oracle.num_faces((h, w)))
    vel[(h + 1) * w:] = 1.0  # vx = 1
    out = oracle.advect(q, 1.0, vel, (h, w))
    # rows but the last (the n - 1.00001 clamp blends the last row)
    np.testing.assert_array_equal(out[:-1, 1:], q[:-1, :-1])
    np.testing.assert_array_equal(out[:-1, 0], q[:-1, 0])  # clamped at the wall


def test_reference_step_runs(oracle):
    """examples/dec_fluid.rs configuration: 128x128, f64, dt 0.05, thr 0.1,
    100 iterations, inflow box, face obstacle; a few steps stay finite."""
    dims = (128, 128)
    vel = np.zeros(oracle.num_faces(dims))
    rho = np.zeros(dims)
    p = np.zeros(dims)
    fs = oracle.reference_face_mask(dims)
    prm = oracle.step_params(source=((0, 5, 54), (1, 20, 64)))
    its = []
    for _ in range(3):
        st = oracle.step(vel, rho, p, dims, prm, fs)
        its.append(st.iterations)
    assert np.isfinite(vel).all() and np.isfinite(rho).all()
    assert rho.max() == pytest.approx(1.0, abs=1e-9) and its[-1] > 0


def test_cell_mask_rule(oracle):
    cs = np.zeros((4, 5), np.uint8)
    cs[1, 2] = 1
    fs = oracle.cell_mask_to_faces(cs)
    h, w = 4, 5
    vy = fs[:(h + 1) * w].reshape(h + 1, w)
    vx = fs[(h + 1) * w:].reshape(h, w + 1)
    assert vy[1, 2] and vy[2, 2] and vx[1, 2] and vx[1, 3]
    assert fs.sum() == 4


def test_second_order_advection_keeps_peaks(oracle):
    """Translating a Gaussian blob with a uniform velocity: MacCormack and
    BFECC keep its peak far better than the first-order scheme (the
    reference's), and never leave the initial value range (limiter)."""
    h, w = 48, 64
    y, x = np.mgrid[0:h, 0:w]
    q0 = np.exp(-((x - 16.0) ** 2 + (y - 24.0) ** 2) / (2 * 3.0 ** 2))
    vel = np.zeros(oracle.num_faces((h, w)))
    vel[(h + 1) * w:] = 0.37  # vx
    peaks = {}
    for scheme in (0, 1, 2):
        q = q0.copy()
        for _ in range(40):
            q = oracle.advect(q, 1.0, vel, (h, w)) if scheme == 0 else oracle.advect2(q, 1.0, vel, (h, w), scheme)
        assert q.min() >= -1e-12 and q.max() <= 1.0 + 1e-12
        peaks[scheme] = q.max()
    assert peaks[1] > peaks[0] + 0.1 and peaks[2] > peaks[0] + 0.1
