"""Wavelet and divergence-free wavelet transforms on the device
(panopaea/src/math/wavelet: mod.rs:1-451, haar.rs, spline.rs).

Arrays are float64 CUDA tensors, transformed in place (1D: length n; 2D:
(h, w)); every transformed length must be a multiple of 2**levels.  The
reference describes the module as early, mostly abandoned tests: its
boundary rules (mirror sampling, wrapped scatter) are kept as written, so
only the Haar transform inverts exactly at the borders.
"""

import ctypes as C

import torch

from . import _native as N

HAAR, BIOR13, BIOR22, BIOR24, BIOR31 = 0, 1, 2, 3, 4
ISOTROPIC, ANISOTROPIC, SEPARATE = 0, 1, 2


def _p(t):
    if t.dtype != torch.float64 or not t.is_cuda or not t.is_contiguous():
        raise TypeError("wavelet transforms take contiguous float64 CUDA tensors")
    return C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def fwt_1d(data, levels, wavelet=HAAR):
    """fwt_1d (mod.rs:114-129): |coarse n|detail n|detail n-1|..., in place."""
    temp = torch.empty_like(data)
    N.check(N.load().pg_wavelet_fwt_1d(int(wavelet), _p(data), data.numel(), int(levels), _p(temp), _stream()))
    return data


def ifwt_1d(data, levels, wavelet=HAAR):
    """ifwt_1d (mod.rs:131-143), in place."""
    temp = torch.empty_like(data)
    N.check(N.load().pg_wavelet_ifwt_1d(int(wavelet), _p(data), data.numel(), int(levels), _p(temp), _stream()))
    return data


def fwt_2d(data, levels, wavelet_x=HAAR, wavelet_y=None, mode=ISOTROPIC):
    """fwt_2d_isotropic / fwt_2d_separate_isotropic (mode ISOTROPIC) and
    fwt_2d_anisotropic (mode ANISOTROPIC), in place."""
    wy = wavelet_x if wavelet_y is None else wavelet_y
    h, w = data.shape
    temp = torch.empty_like(data)
    N.check(N.load().pg_wavelet_fwt_2d(int(mode), int(wavelet_x), int(wy), _p(data), h, w, int(levels), _p(temp),
                                       _stream()))
    return data


def ifwt_2d(data, levels, wavelet_x=HAAR, wavelet_y=None, mode=ISOTROPIC):
    """ifwt_2d_isotropic (mode ISOTROPIC: y, then x) or
    ifwt_2d_separate_isotropic (mode SEPARATE: x, then y), in place."""
    wy = wavelet_x if wavelet_y is None else wavelet_y
    h, w = data.shape
    temp = torch.empty_like(data)
    N.check(N.load().pg_wavelet_ifwt_2d(int(mode), int(wavelet_x), int(wy), _p(data), h, w, int(levels), _p(temp),
                                        _stream()))
    return data


def div_coeff_2d(levels, vx, vy):
    """div_coeff_2d (mod.rs:296-376): returns (div, n)."""
    div, n = torch.zeros_like(vx), torch.zeros_like(vx)
    h, w = vx.shape
    N.check(N.load().pg_wavelet_div_coeff_2d(int(levels), _p(vx), _p(vy), _p(div), _p(n), h, w, _stream()))
    return div, n


def inv_div_coeff_2d(levels, div, n):
    """inv_div_coeff_2d (mod.rs:378-451): returns (vx, vy)."""
    vx, vy = torch.zeros_like(div), torch.zeros_like(div)
    h, w = div.shape
    N.check(N.load().pg_wavelet_inv_div_coeff_2d(int(levels), _p(div), _p(n), _p(vx), _p(vy), h, w, _stream()))
    return vx, vy
