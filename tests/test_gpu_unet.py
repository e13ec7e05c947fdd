"""The learned pressure guess on the GPU: forward output, loss and every
weight gradient of the device network against the CPU oracle's bf16-storage
restatement; Adam; the initial-guess solver path; and what a trained network
gains over the same solver started from zero."""

import numpy as np
import pytest
import torch

from conftest import rng
from test_gpu_ops import dev, host

pytestmark = pytest.mark.gpu

CIN = [16, 16, 16, 32, 32, 64, 96, 32, 48, 16]
COUT = [16, 16, 32, 32, 64, 64, 32, 32, 16, 16]
OFFS = np.cumsum([0] + [27 * a * c for a, c in zip(CIN, COUT)])


def _case(pg, oracle, dims, seed):
    from panopaea_gb300 import learned, workloads

    r = rng(seed)
    g = pg.Grid3d(dims)
    mask = learned.box_obstacles(dims, r)
    g.set_solid_cells(mask)
    fs = oracle.cell_mask_to_faces(mask)
    b = r.standard_normal(dims).astype(np.float32)
    b[mask > 0] = 0
    # a smooth target, like a pressure field (the energy-norm loss applies
    # the Laplacian to the error, which would amplify white noise)
    pt = 10.0 * workloads._box3(r.standard_normal(dims).astype(np.float32), 3)
    pt[mask > 0] = 0
    params = learned.he_init(seed)
    return g, mask, fs, b, pt, params


@pytest.mark.parametrize("loss_kind", [0, 1])
@pytest.mark.parametrize("dims", [(16, 16, 16), (16, 32, 24), (32, 20, 16)])
def test_forward_and_gradients_match_oracle(pg, oracle, dims, loss_kind):
    """Raw output within 1% (relative L2) of the oracle; loss within 1e-3;
    every layer's weight gradient within 3% (MSE loss) / 8% (energy-norm
    loss) relative L2, with cosine similarity >= 0.998 / 0.99.  BF16
    storage: the two sides round the same values and differ only where FP32
    sums taken in another order land on the other side of a BF16 rounding
    boundary.  The bound is the gradient's own sensitivity: on the oracle, a
    1e-5 relative change of b moves the bf16-mode layer gradients by up to
    2.2% (MSE) and 7.7% (energy norm, whose Laplacian amplifies the
    flips)."""
    from panopaea_gb300 import learned

    g, mask, fs, b, pt, params = _case(pg, oracle, dims, seed=41 + dims[2])
    out_scale, dt = 3.0, 0.5
    net = learned.PressureNet(dims, params=params, out_scale=out_scale)
    net.set_loss(loss_kind)
    gb, gpt = pg.Simplex2(g, dev(b)), pg.Simplex2(g, dev(pt))
    x = g.new_simplex_2()
    net.forward(g, gb, dt, x)
    loss = net.accumulate(g, gb, gpt, dt)
    grads = net.get_grads()
    p_ref, loss_ref, g_ref = oracle.unet_run(params, out_scale, dt, dims, b, fs, pt, want_grad=True,
                                             loss_kind=loss_kind)
    p_gpu = host(x)
    assert np.linalg.norm(p_gpu - p_ref) <= 1e-2 * np.linalg.norm(p_ref)
    assert np.all(p_gpu[mask > 0] == 0)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    tol, cos_min = (3e-2, 0.998) if loss_kind == 0 else (8e-2, 0.99)
    for k in range(10):
        a, c = grads[OFFS[k]:OFFS[k + 1]], g_ref[OFFS[k]:OFFS[k + 1]]
        assert np.linalg.norm(a - c) <= tol * np.linalg.norm(c), (k, np.linalg.norm(a - c) / np.linalg.norm(c))
        assert np.vdot(a, c) >= cos_min * np.linalg.norm(a) * np.linalg.norm(c), k
    a, c = grads[OFFS[10]:], g_ref[OFFS[10]:]
    assert np.linalg.norm(a - c) <= 1e-2 * np.linalg.norm(c)
    # padded input channels of layer 0 get no gradient
    assert np.all(grads[:OFFS[1]].reshape(27, 16, 16)[:, 2:, :] == 0)


def test_guess_is_the_energy_optimal_step(pg, oracle):
    """guess = alpha * raw output with alpha = (d.b) / (d.Ad): the guess's
    energy functional x.Ax/2 - x.b is <= 0 (never worse than x = 0) and
    equals -(d.b)^2 / (2 d.Ad)."""
    from panopaea_gb300 import learned

    dims = (16, 16, 16)
    g, mask, fs, b, pt, params = _case(pg, oracle, dims, seed=47)
    net = learned.PressureNet(dims, params=params, out_scale=5.0)
    gb = pg.Simplex2(g, dev(b))
    d, x = g.new_simplex_2(), g.new_simplex_2()
    net.forward(g, gb, 0.7, d)
    net.guess(g, gb, 0.7, x)
    dd, xx = host(d).astype(np.float64), host(x).astype(np.float64)
    ad = oracle.laplacian(dd, 0.7, dims, fs)
    alpha = np.vdot(dd, b) / np.vdot(dd, ad)
    np.testing.assert_allclose(xx, alpha * dd, rtol=1e-4, atol=1e-6 * np.abs(xx).max())
    ax = oracle.laplacian(xx, 0.7, dims, fs)
    energy = 0.5 * np.vdot(xx, ax) - np.vdot(xx, b)
    assert energy <= 0 and energy == pytest.approx(-np.vdot(dd, b) ** 2 / (2 * np.vdot(dd, ad)), rel=1e-3)


def test_gradient_accumulation_and_adam(pg, oracle):
    """Two accumulations add; one Adam step matches the textbook update."""
    from panopaea_gb300 import learned

    dims = (16, 16, 16)
    g, mask, fs, b, pt, params = _case(pg, oracle, dims, seed=45)
    net = learned.PressureNet(dims, params=params, out_scale=2.0)
    gb, gpt = pg.Simplex2(g, dev(b)), pg.Simplex2(g, dev(pt))
    net.accumulate(g, gb, gpt, 1.0)
    g1 = net.get_grads()
    net.accumulate(g, gb, gpt, 1.0)
    g2 = net.get_grads()
    np.testing.assert_allclose(g2, 2 * g1, rtol=1e-5, atol=1e-12)
    lr, b1, b2, eps, gs = 1e-3, 0.9, 0.999, 1e-8, 0.5
    net.adam_step(lr=lr, beta1=b1, beta2=b2, eps=eps, grad_scale=gs)
    p1, _ = net.get_params()
    gg = g2.astype(np.float64) * gs
    m, v = (1 - b1) * gg, (1 - b2) * gg * gg
    want = params - lr * (m / (1 - b1)) / (np.sqrt(v / (1 - b2)) + eps)
    np.testing.assert_allclose(p1, want, rtol=1e-5, atol=1e-7)
    assert np.all(net.get_grads() == 0)


def test_initial_guess_solver_path(pg, oracle):
    """initial_guess: the exact solution as the guess needs no iteration;
    a perturbed one converges to the same tolerance; refine = 0 refuses."""
    from panopaea_gb300 import learned

    dims = (16, 16, 16)
    g = pg.Grid3d(dims)
    b, p, mask, st = learned.training_pair(g, seed=7)
    assert st["status"] == 0
    solver = pg.SolverConfig(rel_stop=True, rel_tol=1e-6, max_iter=20000, refine=8, initial_guess=True)
    x = pg.Simplex2(g, p.data.clone())
    st2 = pg.solve_pressure(g, x, b, 1.0, solver)
    assert st2["status"] == 0 and st2["iterations"] <= 0.2 * st["iterations"]
    x = pg.Simplex2(g, p.data + 0.01 * torch.randn_like(p.data) * p.data.abs().max())
    st3 = pg.solve_pressure(g, x, b, 1.0, solver)
    assert st3["status"] == 0 and 0 < st3["iterations"]
    assert st3["true_residual_max"] <= 1e-6 * st3["b_max"]
    with pytest.raises(pg.PgError):
        pg.solve_pressure(g, x, b, 1.0, pg.SolverConfig(refine=0, initial_guess=True))


def test_bad_shapes(pg):
    from panopaea_gb300 import learned

    for dims in [(15, 16, 16), (16, 16, 18), (8, 16, 16)]:
        with pytest.raises(pg.PgError):
            learned.PressureNet(dims)
    net = learned.PressureNet((16, 16, 16))
    g = pg.Grid3d((16, 16, 20))
    b = g.new_simplex_2()
    with pytest.raises(pg.PgError):
        net.guess(g, b, 1.0, g.new_simplex_2())


@pytest.fixture(scope="module")
def trained32(pg):
    """A network trained on 32^3 grids with 1-6 random boxes and
    filtered-noise divergence (energy-norm loss, 10 epochs, 384 pairs from
    the plain solver: FP64-refined CG to relative 1e-6), and 8 held-out
    grids."""
    from panopaea_gb300 import learned

    dims = (32, 32, 32)
    g = pg.Grid3d(dims)
    torch.manual_seed(0)
    pairs = [learned.training_pair(g, seed=1000 + i)[:3] for i in range(384)]
    held = [learned.training_pair(g, seed=5000 + i)[:3] for i in range(8)]
    scale = learned.estimate_out_scale(pairs, 1.0)
    net = learned.PressureNet(dims, out_scale=scale, seed=1)
    hist = learned.train(net, g, pairs, 1.0, epochs=10, batch=4, lr=1e-3)
    return g, net, held, hist


def test_trained_network_saves_iterations(pg, oracle, trained32):
    """Solve the 8 held-out grids from x = 0 and from the learned guess with
    the same solver and tolerance.  Both runs must meet the tolerance (the
    network changes the start, never the accuracy); the guess must save
    >= 5% of the CG iterations, and the guess with one learned correction
    round >= 10%."""
    from panopaea_gb300 import learned

    g, net, held, hist = trained32
    assert hist[-1] < 0.2 * hist[0]
    solver = pg.SolverConfig(rel_stop=True, rel_tol=1e-6, max_iter=20000, refine=8)
    it = {0: [], 1: [], 2: []}
    for b, _, mask in held:
        g.set_solid_cells(mask)
        x = g.new_simplex_2()
        runs = [pg.solve_pressure(g, x, b, 1.0, solver)]
        for corr in (0, 1):
            x = g.new_simplex_2()
            runs.append(learned.solve_with_guess(net, g, x, b, 1.0, solver, corrections=corr))
        for k, s in enumerate(runs):
            assert s["status"] == 0 and s["true_residual_max"] <= 1e-6 * s["b_max"]
            it[k].append(s["iterations"])
    print("CG iterations from zero %s, learned guess %s, guess + 1 correction %s" % (it[0], it[1], it[2]))
    assert np.mean(it[1]) <= 0.95 * np.mean(it[0])
    assert np.mean(it[2]) <= 0.90 * np.mean(it[0])


def test_learned_preconditioner_inside_cg(pg, oracle, trained32):
    """The trained network as a preconditioner correction inside the CG
    (flexible CG, z = a net(r) + D^-1 (r - a A net(r))) on the held-out
    grids, in FP64-class refinement to relative 1e-6: every solve meets the
    tolerance (checked in FP64 by the oracle's operator), and it needs fewer
    iterations than plain CG and than Jacobi-PCG on the same grids."""
    from panopaea_gb300 import learned

    g, net, held, _ = trained32
    dims = (32, 32, 32)
    its = {"plain": [], "jacobi": [], "learned": []}
    for b, _, mask in held:
        g.set_solid_cells(mask)
        fs = oracle.cell_mask_to_faces(mask)
        for name, precond in (("plain", 0), ("jacobi", 1)):
            x = g.new_simplex_2()
            st = pg.solve_pressure(g, x, b, 1.0, pg.SolverConfig(precond=precond, rel_stop=True, rel_tol=1e-6,
                                                                 max_iter=20000, refine=8))
            assert st["status"] == 0
            its[name].append(st["iterations"])
        x = g.new_simplex_2()
        st = learned.solve_learned_pcg(net, g, x, b, 1.0, pg.SolverConfig(rel_stop=True, rel_tol=1e-6,
                                                                          max_iter=20000, refine=8))
        assert st["status"] == 0 and st["true_residual_max"] <= 1e-6 * st["b_max"], st
        bh = host(b).astype(np.float64)
        true_r = np.abs(bh - oracle.laplacian(host(x).astype(np.float64), 1.0, dims, fs)).max()
        assert true_r <= 1e-5 * np.abs(bh).max()  # x returned in FP32
        its["learned"].append(st["iterations"])
    print("iterations: plain CG %s, Jacobi-PCG %s, learned preconditioner (flexible CG) %s" %
          (its["plain"], its["jacobi"], its["learned"]))
    assert np.mean(its["learned"]) < np.mean(its["jacobi"])
    assert np.mean(its["learned"]) < np.mean(its["plain"])


@pytest.mark.parametrize("dims", [(16, 16, 16), (32, 48, 40)])
def test_tensor_core_convs_equal_warp_mma(pg, oracle, dims, monkeypatch):
    """The convolutions on the fifth-generation tensor cores (tcgen05.mma,
    FP32 accumulators in tensor memory) against the warp-level mma.sync
    kernel (PG_UNET_TC=0): the same forward output and loss and every
    layer's weight gradient, to the BF16 storage rounding the two FP32
    summation orders can flip (the bounds of the oracle comparison: output
    1% and loss 1e-3, gradients 8% relative L2 with cosine >= 0.99); no
    tensor-core wait gave up."""
    from panopaea_gb300 import _native as N
    from panopaea_gb300 import learned

    g, mask, fs, b, pt, params = _case(pg, oracle, dims, seed=61 + dims[1])
    gb, gpt = pg.Simplex2(g, dev(b)), pg.Simplex2(g, dev(pt))
    res = {}
    for tc in ("1", "0"):
        monkeypatch.setenv("PG_UNET_TC", tc)
        net = learned.PressureNet(dims, params=params, out_scale=3.0)
        x = g.new_simplex_2()
        net.forward(g, gb, 0.5, x)
        loss = net.accumulate(g, gb, gpt, 0.5)
        assert N.load().pg_unet_check(net._h) == N.PG_OK
        res[tc] = (host(x), loss, net.get_grads())
    (x1, l1, g1), (x0, l0, g0) = res["1"], res["0"]
    assert np.linalg.norm(x1 - x0) <= 1e-2 * np.linalg.norm(x0)
    assert abs(l1 - l0) <= 1e-3 * l0
    for k in range(10):
        a, c = g1[OFFS[k]:OFFS[k + 1]], g0[OFFS[k]:OFFS[k + 1]]
        assert np.linalg.norm(a - c) <= 8e-2 * np.linalg.norm(c), (k, np.linalg.norm(a - c) / np.linalg.norm(c))
        assert np.vdot(a, c) >= 0.99 * np.linalg.norm(a) * np.linalg.norm(c), k
