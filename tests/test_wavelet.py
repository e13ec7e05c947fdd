"""Wavelet transforms (panopaea/src/math/wavelet): the device transforms
bit-exact against the oracle's restatement for every function, filter and
mode; and, on the CPU, the properties the restated algorithm has (the Haar
transforms invert exactly; the spline filters invert away from the
borders, where the reference's mirror sampling and wrapped scatter are not
a perfect-reconstruction boundary rule; the border variants reconstruct
their input's leading samples for every filter), and the border variants'
index arithmetic run on the host against the oracle."""

import os

import numpy as np
import pytest

from conftest import rng

WAVELETS = [0, 1, 2, 3, 4]


def test_haar_inverts_exactly(oracle):
    x = rng(51).standard_normal(128)
    assert np.abs(oracle.wavelet_ifwt_1d(0, oracle.wavelet_fwt_1d(0, x, 4), 4) - x).max() < 1e-13
    X = rng(52).standard_normal((32, 64))
    for mode_f, mode_i in ((0, 0), (0, 2)):
        Y = oracle.wavelet_fwt_2d(mode_f, 0, 0, X, 3)
        assert np.abs(oracle.wavelet_ifwt_2d(mode_i, 0, 0, Y, 3) - X).max() < 1e-13


@pytest.mark.parametrize("wavelet", [1, 2, 3, 4])
def test_splines_invert_in_the_interior(oracle, wavelet):
    X = rng(53 + wavelet).standard_normal((64, 64))
    Z = oracle.wavelet_ifwt_2d(0, wavelet, wavelet, oracle.wavelet_fwt_2d(0, wavelet, wavelet, X, 2), 2)
    assert np.abs(Z - X)[12:-12, 12:-12].max() < 1e-12


def test_haar_energy_and_mean(oracle):
    """Orthonormal Haar: energy kept; the coarse band carries the mean."""
    x = rng(57).standard_normal(64)
    y = oracle.wavelet_fwt_1d(0, x, 6)
    assert np.vdot(y, y) == pytest.approx(np.vdot(x, x), rel=1e-12)
    assert y[0] == pytest.approx(x.sum() / 8.0, rel=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("wavelet", WAVELETS)
@pytest.mark.parametrize("n,levels", [(16, 1), (64, 3), (1024, 5)])
def test_gpu_1d_bit_exact(pg, oracle, wavelet, n, levels):
    import torch

    from panopaea_gb300 import wavelet as WV

    if (n >> (levels - 1)) < (2, 6, 6, 10, 4)[wavelet]:
        pytest.skip("last level shorter than the filter")
    x = rng(n + 7 * wavelet).standard_normal(n)
    t = torch.from_numpy(x.copy()).cuda()
    WV.fwt_1d(t, levels, wavelet)
    y = oracle.wavelet_fwt_1d(wavelet, x, levels)
    assert np.array_equal(t.cpu().numpy(), y)
    WV.ifwt_1d(t, levels, wavelet)
    assert np.array_equal(t.cpu().numpy(), oracle.wavelet_ifwt_1d(wavelet, y, levels))


@pytest.mark.gpu
@pytest.mark.parametrize("wx,wy", [(0, 0), (1, 1), (2, 3), (4, 2), (3, 3)])
@pytest.mark.parametrize("shape,levels", [((32, 64), 2), ((64, 48), 3), ((128, 256), 4)])
def test_gpu_2d_bit_exact(pg, oracle, wx, wy, shape, levels):
    import torch

    from panopaea_gb300 import wavelet as WV

    taps = (2, 6, 6, 10, 4)
    if (shape[1] >> (levels - 1)) < taps[wx] or (shape[0] >> (levels - 1)) < taps[wy]:
        pytest.skip("last level shorter than the filter")
    X = rng(shape[0] + 3 * wx + wy).standard_normal(shape)
    for fmode, imode in ((0, 0), (1, 2)):
        t = torch.from_numpy(X.copy()).cuda()
        WV.fwt_2d(t, levels, wx, wy, mode=fmode)
        Y = oracle.wavelet_fwt_2d(fmode, wx, wy, X, levels)
        assert np.array_equal(t.cpu().numpy(), Y), fmode
        WV.ifwt_2d(t, levels, wx, wy, mode=imode)
        assert np.array_equal(t.cpu().numpy(), oracle.wavelet_ifwt_2d(imode, wx, wy, Y, levels)), imode


@pytest.mark.gpu
@pytest.mark.parametrize("shape,levels", [((16, 16), 1), ((64, 32), 3), ((256, 128), 5)])
def test_gpu_div_coeff_bit_exact(pg, oracle, shape, levels):
    import torch

    from panopaea_gb300 import wavelet as WV

    r = rng(shape[0] * levels)
    vx, vy = r.standard_normal(shape), r.standard_normal(shape)
    d, n = WV.div_coeff_2d(levels, torch.from_numpy(vx).cuda(), torch.from_numpy(vy).cuda())
    do, no = oracle.wavelet_div_coeff_2d(levels, vx, vy)
    assert np.array_equal(d.cpu().numpy(), do) and np.array_equal(n.cpu().numpy(), no)
    a, b = WV.inv_div_coeff_2d(levels, d, n)
    ao, bo = oracle.wavelet_inv_div_coeff_2d(levels, do, no)
    assert np.array_equal(a.cpu().numpy(), ao) and np.array_equal(b.cpu().numpy(), bo)


@pytest.mark.gpu
def test_gpu_wavelet_rejects_bad_sizes(pg):
    import torch

    from panopaea_gb300 import wavelet as WV

    with pytest.raises(pg.PgError):
        WV.fwt_1d(torch.zeros(24, dtype=torch.float64, device="cuda"), 4)  # 24 not a multiple of 16
    with pytest.raises(pg.PgError):
        WV.fwt_1d(torch.zeros(16, dtype=torch.float64, device="cuda"), 2, WV.BIOR24)  # 8 < 10 taps
    with pytest.raises(TypeError):
        WV.fwt_1d(torch.zeros(16, dtype=torch.float32, device="cuda"), 1)


# ---------------------------------------------------------------------------
# Border variants (mod.rs:454-681)

def test_border_oracle_reconstructs_leading_samples(oracle):
    """Zero padding plus B-wide band borders make the border transforms
    perfect-reconstruction for every filter: the inverse returns the input's
    leading samples (all of them for even sizes) to rounding.  A property of
    the restated algorithm that pins the oracle's band and wrap arithmetic."""
    r = rng(91)
    for wavelet in WAVELETS:
        for n, levels in ((64, 3), (100, 4), (17, 2), (2, 1)):
            x = r.standard_normal(n)
            y = oracle.wavelet_ifwt_1d_border(wavelet, oracle.wavelet_fwt_1d_border(wavelet, x, levels), n)
            m = min(n, y.size)
            assert m >= n - levels and np.abs(y[:m] - x[:m]).max() < 1e-13, (wavelet, n, levels)
    for wx, wy in ((0, 0), (1, 2), (3, 4), (4, 3)):
        for shape, levels in (((32, 48), 3), ((17, 24), 2)):
            X = r.standard_normal(shape)
            Y = oracle.wavelet_ifwt_2d_border(wx, wy, oracle.wavelet_fwt_2d_border(wx, wy, X, levels), *shape)
            a, b = min(shape[0], Y.shape[0]), min(shape[1], Y.shape[1])
            assert np.abs(Y[:a, :b] - X[:a, :b]).max() < 1e-13, (wx, wy, shape, levels)


def test_border_sizes_match_the_oracle_layout(oracle):
    """The library's host-only size functions against the oracle's band
    arithmetic (s // 2 + 2 B per level), for the packed transform and the
    inverse's length / shape."""
    from panopaea_gb300 import wavelet as WV

    for wavelet in WAVELETS:
        for n in (2, 3, 16, 17, 100, 4097):
            for levels in range(0, 7):
                b = oracle.wavelet_border_bands(n, levels, wavelet)
                packed, temp, m = WV.border_sizes_1d(n, levels, wavelet)
                assert packed == ((b[-1] if levels else n) + sum(b))
                assert temp >= 0
                if m >= 0:
                    x = rng(n).standard_normal(n)
                    y = oracle.wavelet_ifwt_1d_border(wavelet, oracle.wavelet_fwt_1d_border(wavelet, x, levels), n)
                    assert y.size == m
    for wx, wy in ((0, 0), (1, 2), (3, 4)):
        for h, w in ((2, 2), (16, 16), (17, 40)):
            for levels in range(0, 5):
                packed, temp, shape = WV.border_sizes_2d(h, w, levels, wx, wy)
                br, bc = oracle.wavelet_border_bands(h, levels, wy), oracle.wavelet_border_bands(w, levels, wx)
                cr, cc = (br[-1], bc[-1]) if levels else (h, w)
                assert packed == cr * cc + sum(3 * r * c for r, c in zip(br, bc))
                if shape[0] >= 0:
                    assert shape == oracle.wavelet_border_inverse_shape(wx, wy, h, w, levels)
    import panopaea_gb300 as pg

    with pytest.raises(pg.PgError):
        WV.border_sizes_1d(1, 1)
    with pytest.raises(pg.PgError):
        WV.border_sizes_2d(8, 8, 1, 7)


def test_border_index_arithmetic_on_the_host(oracle, tmp_path):
    """The per-sample functions and level plans of pg_wavelet_border.cuh
    (what the device kernels run) executed on the CPU by a host-only program
    on exactly sized arrays (AddressSanitizer and UBSan where available),
    bit for bit against the oracle over every wavelet, 1D sizes 2..72 and
    larger, 2D sizes 2..40 and 96 x 130, 0..8 levels."""
    import shutil
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    olib = oracle.lib()._name
    exe = str(tmp_path / "wavelet_border_check")
    base = [cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-ffp-contract=off",
            "-I" + os.path.join(root, "panopaea_gb300", "csrc"), "-I" + os.path.join(root, "include"),
            os.path.join(root, "tests", "cpp", "wavelet_border_check.cpp"), olib,
            "-Wl,-rpath," + os.path.dirname(olib), "-o", exe]
    p = subprocess.run(base[:1] + ["-fsanitize=address,undefined", "-fno-sanitize-recover=all"] + base[1:],
                       capture_output=True, text=True)
    if p.returncode != 0:  # no sanitizer runtime: the bit-exact comparison still runs
        p = subprocess.run(base, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    assert "warning" not in p.stderr, p.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and " 0 wrong" in r.stdout, r.stdout[-3000:] + r.stderr[-3000:]


@pytest.mark.gpu
@pytest.mark.parametrize("wavelet", WAVELETS)
def test_gpu_1d_border_bit_exact(pg, oracle, wavelet):
    import torch

    from panopaea_gb300 import wavelet as WV

    for n, levels in ((2, 1), (17, 2), (64, 3), (1000, 5), (4097, 8), (65536, 6), (40, 0)):
        x = rng(n + 11 * wavelet).standard_normal(n)
        coarse, details = WV.fwt_1d_border(torch.from_numpy(x).cuda(), levels, wavelet)
        oc, od = oracle.wavelet_fwt_1d_border(wavelet, x, levels)
        assert np.array_equal(coarse.cpu().numpy(), oc), (n, levels)
        assert len(details) == len(od) and all(np.array_equal(a.cpu().numpy(), b) for a, b in zip(details, od))
        y = WV.ifwt_1d_border((coarse, details), wavelet)
        assert np.array_equal(y.cpu().numpy(), oracle.wavelet_ifwt_1d_border(wavelet, (oc, od), n)), (n, levels)


@pytest.mark.gpu
@pytest.mark.parametrize("wx,wy", [(0, 0), (1, 1), (2, 3), (4, 2), (3, 3), (0, 4)])
def test_gpu_2d_border_bit_exact(pg, oracle, wx, wy):
    import torch

    from panopaea_gb300 import wavelet as WV

    for shape, levels in (((2, 3), 1), ((17, 24), 2), ((64, 48), 3), ((257, 300), 4), ((16, 16), 0)):
        X = rng(shape[0] + 5 * wx + wy).standard_normal(shape)
        t = WV.fwt_2d_border(torch.from_numpy(X).cuda(), levels, wx, wy)
        o = oracle.wavelet_fwt_2d_border(wx, wy, X, levels)
        assert np.array_equal(t[0].cpu().numpy(), o[0]), (shape, levels)
        for da, db in zip(t[1], o[1]):
            assert all(np.array_equal(a.cpu().numpy(), b) for a, b in zip(da, db)), (shape, levels)
        Y = WV.ifwt_2d_border(t, wx, wy)
        assert np.array_equal(Y.cpu().numpy(), oracle.wavelet_ifwt_2d_border(wx, wy, o, *shape)), (shape, levels)
        V = rng(shape[1] + 7).standard_normal(shape)
        tv = WV.fwt_2d_border(torch.from_numpy(V).cuda(), levels, wx, wy)
        ov = oracle.wavelet_fwt_2d_border(wx, wy, V, levels)
        (dc, dd), (nc, nd) = WV.div_coeff_2d_border(t, tv, wx, wy)
        (odc, odd), (onc, ond) = oracle.wavelet_div_coeff_2d_border(wx, wy, o, ov, *shape)
        assert np.array_equal(dc.cpu().numpy(), odc) and np.array_equal(nc.cpu().numpy(), onc)
        for a3, b3, c3, e3 in zip(dd, odd, nd, ond):
            assert all(np.array_equal(a.cpu().numpy(), b) for a, b in zip(a3, b3))
            assert all(np.array_equal(a.cpu().numpy(), b) for a, b in zip(c3, e3))


@pytest.mark.gpu
def test_gpu_border_rejects_bad_arguments(pg):
    import torch

    from panopaea_gb300 import wavelet as WV

    with pytest.raises(pg.PgError):
        WV.fwt_1d_border(torch.zeros(1, dtype=torch.float64, device="cuda"), 1)  # n < 2
    with pytest.raises(pg.PgError):  # the inverse's sizes go below zero: forward only
        WV.ifwt_1d_border(WV.fwt_1d_border(torch.zeros(2, dtype=torch.float64, device="cuda"), 6))
    with pytest.raises(pg.PgError):
        WV.ifwt_2d_border(WV.fwt_2d_border(torch.zeros((2, 2), dtype=torch.float64, device="cuda"), 4))
    with pytest.raises(ValueError):
        c, d = WV.fwt_1d_border(torch.zeros(16, dtype=torch.float64, device="cuda"), 2)
        WV.ifwt_1d_border((c, d[:1] + [d[1][:-1]]))
