"""numpy front-end of the C++ oracle (test infrastructure only).

Only the test-suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline use this module, always as the results to compare against or the
timed CPU baseline;
the product (``panopaea_gb300``) never imports it.

Arrays follow the reference layouts: 2D cells (h, w), faces
[vy (h+1)w | vx h(w+1)]; 3D cells (d, h, w), faces [vz | vy | vx].
"""

import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None


class StepParams(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("buoyancy", C.c_double),
        ("source_enabled", C.c_int),
        ("source_lo", C.c_long * 3),
        ("source_hi", C.c_long * 3),
        ("source_density", C.c_double),
        ("source_vy", C.c_double),
        ("source_field", C.c_void_p),
        ("walls_after_advect", C.c_int),
        ("zero_solid_after_project", C.c_int),
        ("precond", C.c_int),
        ("rel_stop", C.c_int),
        ("threshold", C.c_double),
        ("rel_tol", C.c_double),
        ("max_iter", C.c_long),
        ("advect_scheme", C.c_int),
        ("density_bf16", C.c_int),
    ]


class StepStats(C.Structure):
    _fields_ = [("iterations", C.c_long), ("residual", C.c_double), ("bmax", C.c_double), ("converged", C.c_int),
                ("t_total", C.c_double), ("t_solve", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_oracle.build())
        _lib.pgo_num_faces.restype = C.c_long
        for s in ("f32", "f64"):
            getattr(_lib, "pgo_pcg_" + s).restype = C.c_long
            getattr(_lib, "pgo_norm_max_" + s).restype = C.c_double
    return _lib


def set_threads(n, all_loops=False):
    lib().pgo_set_threads(int(n), int(bool(all_loops)))


def set_dot64(on):
    """Accumulate dot products in double (the library's choice) or in T
    (the reference's ndarray dot, the default)."""
    lib().pgo_set_dot64(int(bool(on)))


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _sfx(a):
    return {np.dtype(np.float32): "f32", np.dtype(np.float64): "f64"}[a.dtype]


def _shape(dims):
    if len(dims) == 2:
        return 2, 1, dims[0], dims[1]
    return 3, dims[0], dims[1], dims[2]


def num_faces(dims):
    nd, d, h, w = _shape(dims)
    return int(lib().pgo_num_faces(nd, C.c_long(d), C.c_long(h), C.c_long(w)))


def _c(a):
    assert a.flags["C_CONTIGUOUS"]
    return a


def hodge_1_dual(dual, dims):
    out = np.empty_like(dual)
    getattr(lib(), "pgo_hodge_1_dual_" + _sfx(dual))(_p(out), _p(_c(dual)), C.c_long(dims[0]), C.c_long(dims[1]))
    return out


def hodge_1_primal(primal, dims):
    out = np.empty_like(primal)
    getattr(lib(), "pgo_hodge_1_primal_" + _sfx(primal))(_p(out), _p(_c(primal)), C.c_long(dims[0]),
                                                         C.c_long(dims[1]))
    return out


def derivative_1_primal(edges, dims):
    h, w = dims
    out = np.empty((h, w), edges.dtype)
    getattr(lib(), "pgo_derivative_1_primal_" + _sfx(edges))(_p(out), _p(_c(edges)), C.c_long(h), C.c_long(w))
    return out


def derivative_0_dual(faces, dims, edges=None):
    """grid.rs:318-334; `edges` supplies the untouched boundary values."""
    nd, d, h, w = _shape(dims)
    out = np.zeros(num_faces(dims), faces.dtype) if edges is None else edges.copy()
    getattr(lib(), "pgo_derivative_0_dual_" + _sfx(faces))(_p(out), _p(_c(faces)), nd, C.c_long(d), C.c_long(h),
                                                           C.c_long(w))
    return out


def mask_faces(edges, solid):
    out = edges.copy()
    getattr(lib(), "pgo_mask_faces_" + _sfx(edges))(_p(out), _p(_c(solid)), C.c_long(out.size))
    return out


def laplacian(p, dt, dims, face_solid=None):
    nd, d, h, w = _shape(dims)
    out = np.empty_like(p)
    getattr(lib(), "pgo_laplacian_" + _sfx(p))(_p(out), _p(_c(p)), C.c_double(dt), _p(face_solid), nd, C.c_long(d),
                                               C.c_long(h), C.c_long(w))
    return out


def divergence_rhs(vel, dims, face_solid=None):
    nd, d, h, w = _shape(dims)
    out = np.empty(tuple(dims), vel.dtype)
    getattr(lib(), "pgo_divergence_rhs_" + _sfx(vel))(_p(out), _p(_c(vel)), _p(face_solid), nd, C.c_long(d),
                                                      C.c_long(h), C.c_long(w))
    return out


def advect(src, dt, vel, dims):
    nd, d, h, w = _shape(dims)
    out = np.empty_like(src)
    getattr(lib(), "pgo_advect_" + _sfx(src))(_p(out), _p(_c(src)), C.c_double(dt), _p(_c(vel)), nd, C.c_long(d),
                                              C.c_long(h), C.c_long(w))
    return out


def advect_mac(src, dt, vel, dims):
    nd, d, h, w = _shape(dims)
    out = np.empty_like(src)
    getattr(lib(), "pgo_advect_mac_" + _sfx(src))(_p(out), _p(_c(src)), C.c_double(dt), _p(_c(vel)), nd,
                                                  C.c_long(d), C.c_long(h), C.c_long(w))
    return out


def project(vel, p, dt, dims, face_solid=None, zero_solid=False):
    nd, d, h, w = _shape(dims)
    out = vel.copy()
    getattr(lib(), "pgo_project_" + _sfx(vel))(_p(out), _p(_c(p)), C.c_double(dt), _p(face_solid),
                                               int(bool(zero_solid)), nd, C.c_long(d), C.c_long(h), C.c_long(w))
    return out


def walls(vel, dims):
    nd, d, h, w = _shape(dims)
    out = vel.copy()
    getattr(lib(), "pgo_walls_" + _sfx(vel))(_p(out), nd, C.c_long(d), C.c_long(h), C.c_long(w))
    return out


def pcg(b, dt, dims, max_iter, threshold, precond=0, face_solid=None):
    """pcg.rs:14-82; returns (x, r, aux, search, iterations, residual, converged)."""
    nd, d, h, w = _shape(dims)
    x, r, aux, s = (np.zeros_like(b) for _ in range(4))
    res = C.c_double()
    conv = C.c_int()
    it = getattr(lib(), "pgo_pcg_" + _sfx(b))(int(precond), _p(x), _p(_c(b)), C.c_long(max_iter),
                                              C.c_double(threshold), _p(r), _p(aux), _p(s), C.c_double(dt),
                                              _p(face_solid), nd, C.c_long(d), C.c_long(h), C.c_long(w),
                                              C.byref(res), C.byref(conv))
    return x, r, aux, s, int(it), res.value, bool(conv.value)


def norm_max(a):
    return getattr(lib(), "pgo_norm_max_" + _sfx(a))(_p(_c(a)), C.c_long(a.size))


def open_face_count(dims, face_solid=None, dtype=np.float64):
    nd, d, h, w = _shape(dims)
    out = np.empty(tuple(dims), dtype)
    getattr(lib(), "pgo_open_face_count_" + _sfx(out))(_p(out), _p(face_solid), nd, C.c_long(d), C.c_long(h),
                                                       C.c_long(w))
    return out


def step(vel, density, pressure, dims, params, face_solid=None):
    """One step of examples/dec_fluid.rs:46-141 in place; returns StepStats."""
    nd, d, h, w = _shape(dims)
    st = StepStats()
    getattr(lib(), "pgo_step_" + _sfx(vel))(_p(_c(vel)), _p(_c(density)), _p(_c(pressure)), _p(face_solid),
                                            C.byref(params), C.byref(st), nd, C.c_long(d), C.c_long(h),
                                            C.c_long(w))
    return st


def step_params(dt=0.05, buoyancy=0.0, source=None, source_density=1.0, source_vy=20.0, source_field=None,
                walls_after_advect=False, zero_solid_after_project=False, precond=0, rel_stop=False,
                threshold=0.1, rel_tol=1e-6, max_iter=100, advect_scheme=0, density_bf16=False):
    """StepParams; `source` = ((z0, y0, x0), (z1, y1, x1)) or None."""
    p = StepParams()
    p.dt = dt
    p.buoyancy = buoyancy
    p.source_enabled = int(source is not None)
    if source is not None:
        for i in range(3):
            p.source_lo[i] = source[0][i]
            p.source_hi[i] = source[1][i]
    p.source_density = source_density
    p.source_vy = source_vy
    p.source_field = source_field.ctypes.data if source_field is not None else None
    p.walls_after_advect = int(walls_after_advect)
    p.zero_solid_after_project = int(zero_solid_after_project)
    p.precond = precond
    p.rel_stop = int(rel_stop)
    p.threshold = threshold
    p.rel_tol = rel_tol
    p.max_iter = max_iter
    p.advect_scheme = advect_scheme
    p.density_bf16 = int(bool(density_bf16))
    return p


def advect2(src, dt, vel, dims, scheme):
    """Second-order limited advection of a cell scalar (1 MacCormack, 2 BFECC)."""
    nd, d, h, w = _shape(dims)
    out = np.empty_like(src)
    getattr(lib(), "pgo_advect2_" + _sfx(src))(_p(out), _p(_c(src)), C.c_double(dt), _p(_c(vel)), int(scheme), nd,
                                               C.c_long(d), C.c_long(h), C.c_long(w))
    return out


def advect_bf16(src_bits, dt, vel, dims):
    """advect of a bfloat16 cell field given as uint16 bit patterns with a
    float32 velocity; returns uint16 bit patterns."""
    nd, d, h, w = _shape(dims)
    src_bits = np.ascontiguousarray(src_bits, np.uint16)
    vel = np.ascontiguousarray(vel, np.float32)
    out = np.empty_like(src_bits)
    lib().pgo_advect_bf16(_p(out), _p(src_bits), C.c_double(dt), _p(vel), nd, C.c_long(d), C.c_long(h), C.c_long(w))
    return out


def bf16_bits(a):
    """float32 array -> uint16 bfloat16 bit patterns (round to nearest even)."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def bits_to_f32(b):
    return (np.ascontiguousarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


def reference_face_mask(dims, box=((70, 80), (50, 70))):
    """The obstacle of examples/dec_fluid.rs:71-78 as a face mask: vy[y, x]
    and vx[y, x] are solid for y in box[0], x in box[1] (same index box in
    both face arrays)."""
    h, w = dims
    m = np.zeros(num_faces(dims), np.uint8)
    vy = m[:(h + 1) * w].reshape(h + 1, w)
    vx = m[(h + 1) * w:].reshape(h, w + 1)
    (y0, y1), (x0, x1) = box
    vy[y0:y1, x0:x1] = 1
    vx[y0:y1, x0:x1] = 1
    return m


def cell_mask_to_faces(cell_solid):
    """Face is solid iff an adjacent cell is solid (the library's rule)."""
    cs = np.asarray(cell_solid, bool)
    if cs.ndim == 2:
        h, w = cs.shape
        vy = np.zeros((h + 1, w), bool)
        vy[:-1] |= cs
        vy[1:] |= cs
        vx = np.zeros((h, w + 1), bool)
        vx[:, :-1] |= cs
        vx[:, 1:] |= cs
        return np.concatenate([vy.ravel(), vx.ravel()]).astype(np.uint8)
    d, h, w = cs.shape
    vz = np.zeros((d + 1, h, w), bool)
    vz[:-1] |= cs
    vz[1:] |= cs
    vy = np.zeros((d, h + 1, w), bool)
    vy[:, :-1] |= cs
    vy[:, 1:] |= cs
    vx = np.zeros((d, h, w + 1), bool)
    vx[:, :, :-1] |= cs
    vx[:, :, 1:] |= cs
    return np.concatenate([vz.ravel(), vy.ravel(), vx.ravel()]).astype(np.uint8)


HAVE_LIB = os.path.exists(build_oracle.LIB)


def csr_mul_vec(row_indices, col_indices, data, x):
    """panopaea/src/sparse.rs:119-128 on the CPU."""
    rows = len(row_indices) - 1
    b = np.empty(rows, data.dtype)
    rp = np.ascontiguousarray(row_indices, np.int64)
    ci = np.ascontiguousarray(col_indices, np.int64)
    getattr(lib(), "pgo_csr_mul_vec_" + _sfx(data))(C.c_long(rows), _p(rp), _p(ci), _p(_c(data)), _p(_c(x)), _p(b))
    return b


def diag_mul_vec(a, x):
    b = np.empty_like(x)
    getattr(lib(), "pgo_diag_mul_vec_" + _sfx(x))(C.c_long(x.size), _p(_c(a)), _p(_c(x)), _p(b))
    return b


def transfer_rgb8(field, lower, upper):
    """imgproc.rs:2-5 + png.rs row flip: (h, w, 3) uint8 image rows."""
    h, w = field.shape
    out = np.empty((h, w, 3), np.uint8)
    getattr(lib(), "pgo_transfer_rgb8_" + _sfx(field))(C.c_long(h), C.c_long(w), _p(_c(field)), C.c_double(lower),
                                                       C.c_double(upper), _p(out))
    return out


# ---------------------------------------------------------------------------
# The learned pressure-guess network (oracle/unet_oracle.cpp).

def unet_num_params():
    lib().pgo_unet_num_params.restype = C.c_long
    return int(lib().pgo_unet_num_params())


def unet_run(params, out_scale, dt, dims, b, face_solid=None, p_true=None, want_grad=False, loss_kind=1):
    """Forward pass (guess p), and with `p_true` the loss (0 MSE, 1 energy
    norm) and, if asked, the gradient of every parameter.  float32 arrays run
    the bf16-storage mode of the GPU kernels, float64 arrays the exact mode.
    Returns (p, loss, grad)."""
    d, h, w = dims
    dt_ = np.float32 if params.dtype == np.float32 else np.float64
    params = np.ascontiguousarray(params, dt_)
    b = np.ascontiguousarray(b, dt_)
    if face_solid is not None:
        face_solid = np.ascontiguousarray(face_solid, np.uint8)
    nopen = open_face_count(dims, face_solid, np.float64).astype(np.uint8)
    p = np.empty(dims, dt_)
    grad = np.empty(params.size, dt_) if (want_grad and p_true is not None) else None
    loss = C.c_double(0.0)
    if p_true is not None:
        p_true = np.ascontiguousarray(p_true, dt_)
    fn = getattr(lib(), "pgo_unet_run_" + _sfx(params))
    fn.restype = None
    fn(_p(params), C.c_double(out_scale), C.c_double(dt), C.c_long(d), C.c_long(h), C.c_long(w), _p(b), _p(nopen),
       _p(face_solid), int(loss_kind), _p(p_true), _p(p), _p(grad), C.byref(loss))
    return p, (loss.value if p_true is not None else None), grad


def bf16_round(x):
    fn = lib().pgo_bf16_round
    fn.restype = C.c_float
    fn.argtypes = [C.c_float]
    return np.array([fn(float(v)) for v in np.ravel(x)], np.float32).reshape(np.shape(x))


# ---------------------------------------------------------------------------
# Wavelet transforms (oracle/wavelet_oracle.cpp); float64 arrays, returned new.

def _wcall(name, *args):
    fn = getattr(lib(), name)
    fn.restype = None
    fn(*args)


def wavelet_fwt_1d(wavelet, data, levels):
    out = np.array(data, np.float64)
    _wcall("wvo_fwt_1d", int(wavelet), _p(out), C.c_long(out.size), int(levels))
    return out


def wavelet_ifwt_1d(wavelet, data, levels):
    out = np.array(data, np.float64)
    _wcall("wvo_ifwt_1d", int(wavelet), _p(out), C.c_long(out.size), int(levels))
    return out


def wavelet_fwt_2d(mode, wx, wy, data, levels):
    out = np.array(data, np.float64)
    h, w = out.shape
    _wcall("wvo_fwt_2d", int(mode), int(wx), int(wy), _p(out), C.c_long(h), C.c_long(w), int(levels))
    return out


def wavelet_ifwt_2d(mode, wx, wy, data, levels):
    out = np.array(data, np.float64)
    h, w = out.shape
    _wcall("wvo_ifwt_2d", int(mode), int(wx), int(wy), _p(out), C.c_long(h), C.c_long(w), int(levels))
    return out


def wavelet_div_coeff_2d(levels, vx, vy):
    vx = np.ascontiguousarray(vx, np.float64)
    vy = np.ascontiguousarray(vy, np.float64)
    dv, nn = np.zeros_like(vx), np.zeros_like(vx)
    h, w = vx.shape
    _wcall("wvo_div_coeff_2d", int(levels), _p(vx), _p(vy), _p(dv), _p(nn), C.c_long(h), C.c_long(w))
    return dv, nn


def wavelet_inv_div_coeff_2d(levels, dv, nn):
    dv = np.ascontiguousarray(dv, np.float64)
    nn = np.ascontiguousarray(nn, np.float64)
    vx, vy = np.zeros_like(dv), np.zeros_like(dv)
    h, w = dv.shape
    _wcall("wvo_inv_div_coeff_2d", int(levels), _p(dv), _p(nn), _p(vx), _p(vy), C.c_long(h), C.c_long(w))
    return vx, vy


# Border variants (mod.rs:454-681).  A transform is (coarse, details): 1D
# details a list of arrays (finest first), 2D a list of [lyhx, hylx, hyhx].
WAVELET_TAPS = (2, 6, 6, 10, 4)  # filter length = border width of each wavelet


def wavelet_border_bands(s, levels, wavelet):
    """Band lengths s_{k+1} = s_k // 2 + 2 * border width, finest first."""
    out = []
    for _ in range(levels):
        s = s // 2 + 2 * WAVELET_TAPS[wavelet]
        out.append(s)
    return out


def wavelet_fwt_1d_border(wavelet, data, levels):
    x = np.ascontiguousarray(data, np.float64)
    b = wavelet_border_bands(x.size, levels, wavelet)
    packed = np.zeros((b[-1] if levels else x.size) + sum(b))
    _wcall("wvo_fwt_1d_border", int(wavelet), _p(x), C.c_long(x.size), int(levels), _p(packed))
    coarse, off, details = packed[:packed.size - sum(b)], packed.size - sum(b), []
    for n in b:
        details.append(packed[off:off + n])
        off += n
    return coarse, details


def wavelet_ifwt_1d_border(wavelet, transform, n):
    """ifwt_1d_border of the fwt_1d_border of a length-n input."""
    coarse, details = transform
    packed = np.ascontiguousarray(np.concatenate([coarse] + list(details)), np.float64)
    out = np.zeros(packed.size + n)
    fn = lib().wvo_ifwt_1d_border
    fn.restype = C.c_long
    m = fn(int(wavelet), _p(packed), C.c_long(n), int(len(details)), _p(out))
    return out[:m]


def wavelet_fwt_2d_border(wx, wy, data, levels):
    x = np.ascontiguousarray(data, np.float64)
    h, w = x.shape
    br, bc = wavelet_border_bands(h, levels, wy), wavelet_border_bands(w, levels, wx)
    cshape = (br[-1], bc[-1]) if levels else (h, w)
    total = cshape[0] * cshape[1] + sum(3 * r * c for r, c in zip(br, bc))
    packed = np.zeros(total)
    _wcall("wvo_fwt_2d_border", int(wx), int(wy), _p(x), C.c_long(h), C.c_long(w), int(levels), _p(packed))
    return _unpack2(packed, cshape, br, bc)


def _unpack2(packed, cshape, br, bc):
    off = cshape[0] * cshape[1]
    coarse, details = packed[:off].reshape(cshape), []
    for r, c in zip(br, bc):
        band = []
        for _ in range(3):
            band.append(packed[off:off + r * c].reshape(r, c))
            off += r * c
        details.append(band)
    return coarse, details


def _pack2(transform):
    coarse, details = transform
    return np.ascontiguousarray(np.concatenate([np.ravel(coarse)] + [np.ravel(a) for d in details for a in d]),
                                np.float64)


def wavelet_border_inverse_shape(wx, wy, h, w, levels):
    """Shape of ifwt_2d_separate_isotropic_border of the forward transform
    of an (h, w) input: per level 2 * coarse - 4 * border width."""
    br, bc = wavelet_border_bands(h, levels, wy), wavelet_border_bands(w, levels, wx)
    r, c = (br[-1], bc[-1]) if levels else (h, w)
    for _ in range(levels):
        r, c = 2 * r - 4 * WAVELET_TAPS[wy], 2 * c - 4 * WAVELET_TAPS[wx]
    return r, c


def wavelet_ifwt_2d_border(wx, wy, transform, h, w):
    """ifwt_2d_separate_isotropic_border of the forward transform of an (h, w) input."""
    levels = len(transform[1])
    packed = _pack2(transform)
    shape = wavelet_border_inverse_shape(wx, wy, h, w, levels)
    out = np.zeros(shape)
    fn = lib().wvo_ifwt_2d_border
    fn.restype = C.c_long
    m = fn(int(wx), int(wy), _p(packed), C.c_long(h), C.c_long(w), int(levels), _p(out))
    assert m == out.size
    return out


def wavelet_div_coeff_2d_border(wx, wy, tvx, tvy, h, w):
    """div_coeff_2d_border of two forward transforms of (h, w) inputs:
    returns the (div, n) transforms."""
    levels = len(tvx[1])
    a, b = _pack2(tvx), _pack2(tvy)
    d, n = np.zeros_like(a), np.zeros_like(a)
    _wcall("wvo_div_coeff_2d_border", int(wx), int(wy), _p(a), _p(b), C.c_long(h), C.c_long(w), int(levels), _p(d),
           _p(n))
    br, bc = wavelet_border_bands(h, levels, wy), wavelet_border_bands(w, levels, wx)
    cshape = np.shape(tvx[0])
    return _unpack2(d, cshape, br, bc), _unpack2(n, cshape, br, bc)
