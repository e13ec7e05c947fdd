"""Headless field I/O: the density snapshots of examples/dec_fluid.rs:143-164
without a window or an image library.

* :func:`density_image` -- imgproc::transfer (panopaea_utils/src/imgproc.rs:
  2-5) of a 2D cell field into an (h, w, 3) uint8 image on the device, rows
  flipped as png::export writes them (png.rs:12: +y up);
* :func:`write_png` -- an 8-bit RGB PNG written with zlib (png.rs:6-18
  saves the same image through the `image` crate);
* :func:`save_field` / :func:`load_field` -- raw little-endian dumps of a
  device field with a small header, for fixtures and restarts.
"""

import ctypes as C
import struct
import zlib

import numpy as np
import torch

from . import _native as N

_MAGIC = b"PGFIELD1"


def density_image(field, lower=-2.0, upper=2.0):
    """(h, w) CUDA tensor -> (h, w, 3) uint8 CUDA tensor (transfer in f64)."""
    if field.dim() != 2:
        raise ValueError("density_image takes a 2D cell field (slice 3D fields first)")
    h, w = field.shape
    f = field.contiguous()
    out = torch.empty((h, w, 3), dtype=torch.uint8, device=f.device)
    sfx = {torch.float32: "f32", torch.float64: "f64"}[f.dtype]
    lib = N.load()
    N.check(getattr(lib, "pg_transfer_rgb8_" + sfx)(h, w, C.c_void_p(f.data_ptr()), C.c_double(lower),
                                                    C.c_double(upper), C.c_void_p(out.data_ptr()),
                                                    C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out


def _chunk(tag, data):
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def png_bytes(rgb):
    """(h, w, 3) uint8 array -> PNG file bytes (8-bit RGB, no filtering)."""
    rgb = np.ascontiguousarray(np.asarray(rgb, np.uint8))
    h, w, _ = rgb.shape
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))
    return (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)) +
            _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b""))


def write_png(path, rgb):
    if isinstance(rgb, torch.Tensor):
        rgb = rgb.cpu().numpy()
    with open(path, "wb") as f:
        f.write(png_bytes(rgb))


def read_png(path):
    """Reads back what write_png writes (8-bit RGB, filter type 0)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = [raw[y * (3 * w + 1) + 1:(y + 1) * (3 * w + 1)] for y in range(h)]
    return np.frombuffer(b"".join(rows), np.uint8).reshape(h, w, 3)


def save_field(path, tensor, kind, dims):
    """kind: 'cells' or 'faces'; dims: (h, w) or (d, h, w)."""
    t = tensor.detach().contiguous().cpu()
    code = {torch.float32: 0, torch.float64: 1}[t.dtype]
    d = tuple(dims) if len(dims) == 3 else (1,) + tuple(dims)
    hdr = _MAGIC + struct.pack("<iiiqqqq", {"faces": 1, "cells": 2}[kind], code, len(dims), d[0], d[1], d[2],
                               t.numel())
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(t.numpy().tobytes())


def load_field(path, device="cuda"):
    """-> (tensor, kind, dims)."""
    with open(path, "rb") as f:
        blob = f.read()
    if blob[:8] != _MAGIC:
        raise ValueError("not a panopaea field dump")
    kind, code, nd, d, h, w, n = struct.unpack("<iiiqqqq", blob[8:52])
    dt = np.float32 if code == 0 else np.float64
    arr = np.frombuffer(blob[52:], dt, count=n).copy()
    dims = (h, w) if nd == 2 else (d, h, w)
    return torch.from_numpy(arr).to(device), {1: "faces", 2: "cells"}[kind], dims
