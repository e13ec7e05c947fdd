"""Wavelet and divergence-free wavelet transforms on the device
(panopaea/src/math/wavelet: mod.rs:1-681, haar.rs, spline.rs).

Arrays are float64 CUDA tensors.  The mirror-sampled transforms
(mod.rs:1-451) work in place (1D: length n; 2D: (h, w)); every transformed
length must be a multiple of 2**levels.  The reference describes the module
as early, mostly abandoned tests: its boundary rules (mirror sampling,
wrapped scatter) are kept as written, so only the Haar transform inverts
exactly at the borders.  The border variants (mod.rs:454-681) zero-sample
and return new (coarse, details) tensors whose bands grow by the border
width; they reconstruct the input's leading samples for every filter.
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


# ---------------------------------------------------------------------------
# Border variants (mod.rs:454-681): zero sampling, bands of s // 2 + 2 * B
# samples (B = the filter length).  A transform is (coarse, details) as the
# reference returns it -- 1D: details a list of bands, finest first; 2D: a
# list of [lyhx, hylx, hyhx] -- whose tensors are views of one packed
# float64 CUDA tensor (the coarse band, then the detail bands in that order).

TAPS = (2, 6, 6, 10, 4)  # filter length = border width per wavelet


def _i64():
    return C.c_int64(0)


def border_sizes_1d(n, levels, wavelet=HAAR):
    """(packed, temp, inverse_n): elements of the packed transform, of the
    scratch array, and the inverse's length (-1: the inverse's size
    arithmetic goes below zero at some level, as for tiny n with many
    levels; only the forward transform runs).  Host only."""
    p, t, m = _i64(), _i64(), _i64()
    N.check(N.load().pg_wavelet_border_sizes_1d(int(wavelet), int(n), int(levels), C.byref(p), C.byref(t), C.byref(m)))
    return p.value, t.value, m.value


def border_sizes_2d(h, w, levels, wavelet_x=HAAR, wavelet_y=None):
    """(packed, temp, (inverse_h, inverse_w)); host only."""
    wy = wavelet_x if wavelet_y is None else wavelet_y
    p, t, a, b = _i64(), _i64(), _i64(), _i64()
    N.check(N.load().pg_wavelet_border_sizes_2d(int(wavelet_x), int(wy), int(h), int(w), int(levels), C.byref(p),
                                                C.byref(t), C.byref(a), C.byref(b)))
    return p.value, t.value, (a.value, b.value)


def _bands(s, levels, wavelet):
    out = []
    for _ in range(levels):
        s = s // 2 + 2 * TAPS[wavelet]
        out.append(s)
    return out


def _scratch(n, like):
    return torch.empty(max(int(n), 1), dtype=torch.float64, device=like.device)


def fwt_1d_border(data, levels, wavelet=HAAR):
    """fwt_1d_border (mod.rs:454-472): returns (coarse, details)."""
    n = data.numel()
    packed_n, temp_n, _ = border_sizes_1d(n, levels, wavelet)
    packed = torch.empty(packed_n, dtype=torch.float64, device=data.device)
    temp = _scratch(temp_n, data)
    N.check(N.load().pg_wavelet_fwt_1d_border(int(wavelet), _p(data), n, int(levels), _p(packed), _p(temp),
                                              _stream()))
    b = _bands(n, levels, wavelet)
    nc = b[-1] if levels else n
    coarse, details, off = packed[:nc], [], nc
    for k in b:
        details.append(packed[off:off + k])
        off += k
    return coarse, details


def _even_n(first_band, wavelet):
    # a forward input length with these bands (n and n + 1 give the same)
    return 2 * (first_band - 2 * TAPS[wavelet])


def ifwt_1d_border(transform, wavelet=HAAR):
    """ifwt_1d_border (mod.rs:474-486) of a (coarse, details) pair of the
    shape fwt_1d_border returns."""
    coarse, details = transform
    levels = len(details)
    n = _even_n(details[0].numel(), wavelet) if levels else coarse.numel()
    b = _bands(n, levels, wavelet)
    if [d.numel() for d in details] != b or (levels and coarse.numel() != b[-1]):
        raise ValueError("ifwt_1d_border: band lengths do not form a border transform")
    packed = torch.cat([coarse.reshape(-1)] + [d.reshape(-1) for d in details]).contiguous()
    _, temp_n, m = border_sizes_1d(n, levels, wavelet)
    out = torch.empty(max(m, 0), dtype=torch.float64, device=coarse.device)
    # m < 0: the library rejects the call (the inverse's sizes underflow)
    N.check(N.load().pg_wavelet_ifwt_1d_border(int(wavelet), _p(packed), n, levels,
                                               _p(out) if m > 0 else None, _p(_scratch(temp_n, coarse)), _stream()))
    return out


def fwt_2d_border(data, levels, wavelet_x=HAAR, wavelet_y=None):
    """fwt_2d_separate_isotropic_border (mod.rs:551-597): returns (coarse,
    [[lyhx, hylx, hyhx] per level, finest first])."""
    wy = wavelet_x if wavelet_y is None else wavelet_y
    h, w = data.shape
    packed_n, temp_n, _ = border_sizes_2d(h, w, levels, wavelet_x, wy)
    packed = torch.empty(packed_n, dtype=torch.float64, device=data.device)
    N.check(N.load().pg_wavelet_fwt_2d_border(int(wavelet_x), int(wy), _p(data), h, w, int(levels), _p(packed),
                                              _p(_scratch(temp_n, data)), _stream()))
    return _unpack_2d(packed, h, w, levels, wavelet_x, wy)


def _unpack_2d(packed, h, w, levels, wx, wy):
    br, bc = _bands(h, levels, wy), _bands(w, levels, wx)
    cr, cc = (br[-1], bc[-1]) if levels else (h, w)
    coarse, details, off = packed[:cr * cc].view(cr, cc), [], cr * cc
    for r, c in zip(br, bc):
        band = []
        for _ in range(3):
            band.append(packed[off:off + r * c].view(r, c))
            off += r * c
        details.append(band)
    return coarse, details


def _pack_2d(transform, wx, wy):
    coarse, details = transform
    levels = len(details)
    if levels:
        r0, c0 = details[0][0].shape
        h, w = _even_n(r0, wy), _even_n(c0, wx)
    else:
        h, w = coarse.shape
    br, bc = _bands(h, levels, wy), _bands(w, levels, wx)
    shapes = [tuple(a.shape) for d in details for a in d]
    if shapes != [(r, c) for r, c in zip(br, bc) for _ in range(3)] or \
            (levels and tuple(coarse.shape) != (br[-1], bc[-1])):
        raise ValueError("border transform: band shapes do not form a border transform")
    packed = torch.cat([coarse.reshape(-1)] + [a.reshape(-1) for d in details for a in d]).contiguous()
    return packed, h, w, levels


def ifwt_2d_border(transform, wavelet_x=HAAR, wavelet_y=None):
    """ifwt_2d_separate_isotropic_border (mod.rs:599-641): y, then x."""
    wy = wavelet_x if wavelet_y is None else wavelet_y
    packed, h, w, levels = _pack_2d(transform, wavelet_x, wy)
    _, temp_n, (ih, iw) = border_sizes_2d(h, w, levels, wavelet_x, wy)
    # ih < 0: the library rejects the call (the inverse's sizes underflow)
    out = torch.empty((max(ih, 0), max(iw, 0)), dtype=torch.float64, device=packed.device)
    N.check(N.load().pg_wavelet_ifwt_2d_border(int(wavelet_x), int(wy), _p(packed), h, w, levels,
                                               _p(out) if out.numel() else None, _p(_scratch(temp_n, packed)),
                                               _stream()))
    return out


def div_coeff_2d_border(tvx, tvy, wavelet_x=HAAR, wavelet_y=None):
    """div_coeff_2d_border (mod.rs:645-681) of two 2D border transforms:
    returns the (div, n) transforms."""
    wy = wavelet_x if wavelet_y is None else wavelet_y
    a, h, w, levels = _pack_2d(tvx, wavelet_x, wy)
    b, h2, w2, levels2 = _pack_2d(tvy, wavelet_x, wy)
    if (h, w, levels) != (h2, w2, levels2):
        raise ValueError("div_coeff_2d_border: the two transforms differ in shape")
    d, n = torch.empty_like(a), torch.empty_like(a)
    N.check(N.load().pg_wavelet_div_coeff_2d_border(int(wavelet_x), int(wy), _p(a), _p(b), h, w, levels, _p(d),
                                                    _p(n), _stream()))
    return _unpack_2d(d, h, w, levels, wavelet_x, wy), _unpack_2d(n, h, w, levels, wavelet_x, wy)
