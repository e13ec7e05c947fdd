"""The network oracle (oracle/unet_oracle.cpp) on the CPU: its backward pass
against central finite differences in the exact (double, unrounded) mode,
the bf16 rounding rule, and the invariances the network definition implies."""

import numpy as np
import pytest

from conftest import rng

CIN = [16, 16, 16, 32, 32, 64, 96, 32, 48, 16]
COUT = [16, 16, 32, 32, 64, 64, 32, 32, 16, 16]


def he_params(oracle, seed, dtype=np.float64):
    """He-normal weights (fan-in 27 * real input channels), zero rows for
    the padded input channels of layer 0, head ~ N(0, 0.3^2)."""
    r = rng(seed)
    params = np.zeros(oracle.unet_num_params())
    o = 0
    for k in range(10):
        n = 27 * CIN[k] * COUT[k]
        fan = 27 * (2 if k == 0 else CIN[k])
        wk = (r.standard_normal(n) * np.sqrt(2.0 / fan)).reshape(27, CIN[k], COUT[k])
        if k == 0:
            wk[:, 2:, :] = 0
        params[o:o + n] = wk.ravel()
        o += n
    params[o:] = 0.3 * r.standard_normal(16)
    return params.astype(dtype)


def test_param_count(oracle):
    assert oracle.unet_num_params() == 27 * sum(a * b for a, b in zip(CIN, COUT)) + 16


def _face_mask(oracle, dims, box):
    cs = np.zeros(dims, np.uint8)
    cs[box] = 1
    return cs, oracle.cell_mask_to_faces(cs)


@pytest.mark.parametrize("loss_kind", [0, 1])
def test_backward_matches_finite_differences(oracle, loss_kind):
    """Exact mode, 8^3 with a solid block, both losses (MSE, energy norm):
    analytic gradients of 12 random weights (every layer and the head)
    within 1e-4 relative of central differences (step 1e-6)."""
    dims = (8, 8, 8)
    r = rng(31)
    params = he_params(oracle, 32)
    cs, fs = _face_mask(oracle, dims, np.s_[2:4, 2:5, 1:4])
    b = r.standard_normal(dims)
    b[cs > 0] = 0
    pt = r.standard_normal(dims)

    def run(pp, grad=False):
        return oracle.unet_run(pp, 1.3, 0.5, dims, b, fs, pt, want_grad=grad, loss_kind=loss_kind)

    _, loss, g = run(params, True)
    assert loss > 0
    offs = np.cumsum([0] + [27 * a * c for a, c in zip(CIN, COUT)])
    picks = []
    for k in range(10):
        lo, hi = offs[k], offs[k + 1]
        nz = np.flatnonzero(g[lo:hi]) + lo
        picks += list(r.choice(nz, 1, replace=False))
    picks += [offs[10] + 3, offs[10] + 11]
    for j in picks:
        e = 1e-6
        pp = params.copy()
        pp[j] += e
        lp = run(pp)[1]
        pp[j] -= 2 * e
        lm = run(pp)[1]
        fd = (lp - lm) / (2 * e)
        assert abs(fd - g[j]) <= 1e-4 * abs(g[j]) + 1e-12, (j, g[j], fd)


def test_energy_loss_is_blind_to_constants(oracle):
    """The energy-norm loss of a target shifted by a constant is unchanged
    (the constant is in the Laplacian's null space); the MSE loss is not."""
    dims = (8, 8, 8)
    r = rng(37)
    params = he_params(oracle, 38)
    b = r.standard_normal(dims)
    pt = r.standard_normal(dims)
    l1 = oracle.unet_run(params, 1.0, 1.0, dims, b, None, pt, loss_kind=1)[1]
    l2 = oracle.unet_run(params, 1.0, 1.0, dims, b, None, pt + 3.0, loss_kind=1)[1]
    assert l2 == pytest.approx(l1, rel=1e-9)
    m1 = oracle.unet_run(params, 1.0, 1.0, dims, b, None, pt, loss_kind=0)[1]
    m2 = oracle.unet_run(params, 1.0, 1.0, dims, b, None, pt + 3.0, loss_kind=0)[1]
    assert m2 > 2 * m1


def test_bf16_mode_tracks_exact_mode(oracle):
    """The bf16-storage mode (the GPU's) stays within a few percent of the
    exact mode: outputs, loss and the gradient as a whole."""
    dims = (8, 16, 8)
    r = rng(33)
    params = he_params(oracle, 34)
    b = r.standard_normal(dims)
    pt = r.standard_normal(dims)
    p64, l64, g64 = oracle.unet_run(params, 2.0, 1.0, dims, b, None, pt, want_grad=True)
    p32, l32, g32 = oracle.unet_run(params.astype(np.float32), 2.0, 1.0, dims, b.astype(np.float32), None,
                                    pt.astype(np.float32), want_grad=True)
    assert np.linalg.norm(p32 - p64) <= 0.03 * np.linalg.norm(p64)
    assert abs(l32 - l64) <= 0.01 * l64
    assert np.linalg.norm(g32 - g64) <= 0.1 * np.linalg.norm(g64)


def test_bf16_rounding_rule(oracle):
    """Round to nearest even on the upper 16 bits; NaN stays NaN."""
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -2.5e-3, 3.0e38, np.inf], np.float32)
    got = oracle.bf16_round(x)
    u = x.view(np.uint32).astype(np.uint64)
    want = (((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)).view(np.float32)
    want[-1] = np.inf
    assert np.array_equal(got, want)
    assert np.isnan(oracle.bf16_round(np.array([np.nan], np.float32)))[0]


def test_guess_scales_with_dt_and_vanishes_on_solids(oracle):
    dims = (8, 8, 8)
    r = rng(35)
    params = he_params(oracle, 36)
    b = r.standard_normal(dims)
    cs, fs = _face_mask(oracle, dims, np.s_[0:1, :, :])
    p1 = oracle.unet_run(params, 1.0, 1.0, dims, b, fs)[0]
    p2 = oracle.unet_run(params, 1.0, 0.25, dims, b, fs)[0]
    np.testing.assert_allclose(p2, 4 * p1, rtol=1e-12)
    assert np.all(p1[0] == 0) and np.any(p1[1:] != 0)
