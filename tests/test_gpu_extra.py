"""Device sparse products (sparse.rs) and the headless density image
(imgproc.rs + png.rs), bit-exact against the oracle."""

import numpy as np
import pytest
import torch

from conftest import rng

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_csr_and_diag_bit_exact(pg, oracle, dtype):
    from panopaea_gb300.sparse import DiagonalMatrix, SparseMatrix

    r = rng(3)
    rows, cols = 300, 250
    m = SparseMatrix((rows, cols), dtype)
    for _ in range(2000):
        m.insert((int(r.integers(rows)), int(r.integers(cols))), float(r.standard_normal()))
    x = torch.from_numpy(r.standard_normal(cols)).to(dtype).cuda()
    b = torch.empty(rows, dtype=dtype, device="cuda")
    m.mul_vec(b, x)
    rp, ci, d = m.to_csr_numpy()
    npd = np.float64 if dtype == torch.float64 else np.float32
    want = oracle.csr_mul_vec(rp, ci, d.astype(npd), x.cpu().numpy())
    assert np.array_equal(b.cpu().numpy(), want)
    a = torch.from_numpy(r.standard_normal(cols)).to(dtype).cuda()
    dm = DiagonalMatrix(cols, dtype, a)
    out = torch.empty_like(x)
    dm.mul_vec(out, x)
    assert np.array_equal(out.cpu().numpy(), oracle.diag_mul_vec(a.cpu().numpy(), x.cpu().numpy()))
    assert torch.equal((dm * dm).data, a * a)


def test_csr_laplacian_matches_operator(pg, oracle):
    """The masked Laplacian assembled as a SparseMatrix (rows = cells) gives
    the same product as the fused operator, to rounding."""
    from panopaea_gb300.sparse import SparseMatrix

    h, w = 12, 9
    m = SparseMatrix((h * w, h * w), torch.float64)
    for y in range(h):
        for x in range(w):
            i = y * w + x
            nb = [(y - 1, x), (y + 1, x), (y, x - 1), (y, x + 1)]
            nb = [(a, c) for a, c in nb if 0 <= a < h and 0 <= c < w]
            m.insert((i, i), float(len(nb)))
            for a, c in nb:
                m.insert((i, a * w + c), -1.0)
    p = torch.from_numpy(rng(4).standard_normal((h, w))).cuda()
    b = torch.empty(h * w, dtype=torch.float64, device="cuda")
    m.mul_vec(b, p.view(-1))
    g = pg.Grid2d((h, w))
    out = g.new_simplex_2(torch.float64)
    g.laplacian(out, pg.Simplex2(g, p), 1.0)
    np.testing.assert_allclose(b.cpu().numpy().reshape(h, w), out.data.cpu().numpy(), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_density_image_bit_exact(pg, oracle, dtype, tmp_path):
    from panopaea_gb300 import io

    f = torch.from_numpy(rng(5).standard_normal((40, 33)) * 2).to(dtype)
    f[3, 4] = float("nan")
    img = io.density_image(f.cuda(), -2.0, 2.0)
    want = oracle.transfer_rgb8(f.numpy(), -2.0, 2.0)
    assert np.array_equal(img.cpu().numpy(), want)
    path = str(tmp_path / "density.png")
    io.write_png(path, img)
    assert np.array_equal(io.read_png(path), want)


def test_reference_loop_snapshot(pg, oracle, tmp_path):
    """Density snapshot of the reference loop after 10 steps
    (examples/dec_fluid.rs:143-164) equals the oracle's, pixel for pixel."""
    from panopaea_gb300 import io

    dims = (64, 64)
    g = pg.Grid2d(dims)
    vel, rho, p = g.new_simplex_1(torch.float64), g.new_simplex_2(torch.float64), g.new_simplex_2(torch.float64)
    cfg = pg.StepConfig(source_lo=(0, 5, 27), source_hi=(1, 20, 37))
    vo = np.zeros(oracle.num_faces(dims))
    ro = np.zeros(dims)
    po = np.zeros(dims)
    prm = oracle.step_params(source=((0, 5, 27), (1, 20, 37)))
    for _ in range(10):
        pg.step(g, cfg, vel, rho, p)
        oracle.step(vo, ro, po, dims, prm)
    img = io.density_image(rho.data)
    want = oracle.transfer_rgb8(ro, -2.0, 2.0)
    diff = np.abs(img.cpu().numpy().astype(int) - want.astype(int))
    assert diff.max() <= 1  # the PCG's rounding may move a pixel across a level
