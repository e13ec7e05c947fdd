"""SparseMatrix / DiagonalMatrix of panopaea/src/sparse.rs with device products.

`SparseMatrix` keeps the reference's CSR construction semantics on the host
(`new((rows, cols))`, `insert((i, j), v)` keeps each row's columns sorted and
overwrites an existing entry, sparse.rs:49-86); `mul_vec(b, x)` runs on the
device (``pg_csr_mul_vec_*``), one thread per row folding the row in storage
order as sparse.rs:119-128 does.  `DiagonalMatrix.mul_vec` is b = x * a
(sparse.rs:20-25); `a * b` multiplies two diagonals (sparse.rs:143-154).
"""

import bisect
import ctypes as C

import numpy as np
import torch

from . import _native as N


def _sfx(t):
    return {torch.float32: "f32", torch.float64: "f64"}[t.dtype]


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class SparseMatrix:
    def __init__(self, dim, dtype=torch.float32):
        self._dim = (int(dim[0]), int(dim[1]))
        self.dtype = dtype
        self.data = []
        self.col_indices = []
        self.row_indices = [0] * (self._dim[0] + 1)
        self._dev = None

    def dim(self):
        return self._dim

    def insert(self, index, elem):
        i, j = int(index[0]), int(index[1])
        if not (0 <= i < self._dim[0] and 0 <= j < self._dim[1]):
            raise IndexError("Element index out of bounds")
        start, end = self.row_indices[i], self.row_indices[i + 1]
        pos = bisect.bisect_left(self.col_indices, j, start, end)
        if pos < end and self.col_indices[pos] == j:
            self.data[pos] = elem  # overwrite existing element
        else:
            self.data.insert(pos, elem)
            self.col_indices.insert(pos, j)
            for k in range(i + 1, len(self.row_indices)):
                self.row_indices[k] += 1
        self._dev = None

    def _device(self):
        if self._dev is None:
            self._dev = (
                torch.tensor(self.row_indices, dtype=torch.int64, device="cuda"),
                torch.tensor(self.col_indices or [0], dtype=torch.int64, device="cuda"),
                torch.tensor(self.data or [0.0], dtype=self.dtype, device="cuda"),
            )
        return self._dev

    def mul_vec(self, b, x):
        """b = A x on the device (b, x: 1-D CUDA tensors of this dtype)."""
        rp, ci, d = self._device()
        lib = N.load()
        N.check(getattr(lib, "pg_csr_mul_vec_" + _sfx(d))(self._dim[0], C.c_void_p(rp.data_ptr()),
                                                           C.c_void_p(ci.data_ptr()), C.c_void_p(d.data_ptr()),
                                                           C.c_void_p(x.data_ptr()), C.c_void_p(b.data_ptr()),
                                                           _stream()))
        return b

    def to_csr_numpy(self):
        return (np.array(self.row_indices, np.int64), np.array(self.col_indices, np.int64),
                np.array(self.data, np.float64 if self.dtype == torch.float64 else np.float32))


class DiagonalMatrix:
    def __init__(self, dim, dtype=torch.float32, data=None):
        self.dim = int(dim)
        self.data = torch.zeros(self.dim, dtype=dtype, device="cuda") if data is None else data

    def __getitem__(self, i):
        return self.data[i]

    def __setitem__(self, i, v):
        self.data[i] = v

    def mul_vec(self, b, x):
        lib = N.load()
        N.check(getattr(lib, "pg_diag_mul_vec_" + _sfx(self.data))(self.dim, C.c_void_p(self.data.data_ptr()),
                                                                    C.c_void_p(x.data_ptr()),
                                                                    C.c_void_p(b.data_ptr()), _stream()))
        return b

    def __mul__(self, rhs):
        out = DiagonalMatrix(self.dim, self.data.dtype, torch.empty_like(self.data))
        return self._mul_into(out, rhs)

    def _mul_into(self, out, rhs):
        # sparse.rs:143-154: self[i] = self[i] * rhs[i], elementwise
        lib = N.load()
        N.check(getattr(lib, "pg_diag_mul_vec_" + _sfx(self.data))(self.dim, C.c_void_p(rhs.data.data_ptr()),
                                                                    C.c_void_p(self.data.data_ptr()),
                                                                    C.c_void_p(out.data.data_ptr()), _stream()))
        return out
