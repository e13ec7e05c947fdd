"""Wavelet transforms (panopaea/src/math/wavelet): the device transforms
bit-exact against the oracle's restatement for every function, filter and
mode; and, on the CPU, the properties the restated algorithm has (the Haar
transforms invert exactly; the spline filters invert away from the
borders, where the reference's mirror sampling and wrapped scatter are not
a perfect-reconstruction boundary rule)."""

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
