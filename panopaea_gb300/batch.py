"""Batches of independent 2D grids on one GPU (``pg_batch_*``), and the
partition of a batch across ranks.

Every grid keeps the reference's layouts (dec/grid.rs:36-100); the batch
packs them back to back.  One call of :meth:`Batch2d.step` advances every
grid by one step of examples/dec_fluid.rs:46-141, each grid with its own CG
scalars and stop rule, every stage one launch over all grids.
"""

import ctypes as C

import numpy as np
import torch

from . import _native as N


class Batch2d:
    def __init__(self, dims):
        self._lib = N.load()
        self.dims = [(int(h), int(w)) for h, w in dims]
        n = len(self.dims)
        hs = (C.c_int64 * n)(*[d[0] for d in self.dims])
        ws = (C.c_int64 * n)(*[d[1] for d in self.dims])
        self._h = C.c_void_p()
        N.check(self._lib.pg_batch_create_2d(n, hs, ws, C.byref(self._h)))
        co = (C.c_int64 * (n + 1))()
        fo = (C.c_int64 * (n + 1))()
        N.check(self._lib.pg_batch_layout(self._h, co, fo))
        self.cell_offsets = np.array(co[:], np.int64)
        self.face_offsets = np.array(fo[:], np.int64)
        self.ncells = int(self.cell_offsets[-1])
        self.nfaces = int(self.face_offsets[-1])

    def __len__(self):
        return len(self.dims)

    def close(self):
        if self._h:
            self._lib.pg_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _bind(self):
        N.check(self._lib.pg_batch_set_stream(self._h, C.c_void_p(torch.cuda.current_stream().cuda_stream)))

    # packed fields -----------------------------------------------------------
    def new_faces(self):
        return torch.zeros(self.nfaces, dtype=torch.float32, device="cuda")

    def new_cells(self):
        return torch.zeros(self.ncells, dtype=torch.float32, device="cuda")

    def cells_of(self, packed, i):
        h, w = self.dims[i]
        a = int(self.cell_offsets[i])
        return packed[a:a + h * w].view(h, w)

    def faces_of(self, packed, i):
        return packed[int(self.face_offsets[i]):int(self.face_offsets[i + 1])]

    def pack_cells(self, arrays):
        return np.concatenate([np.asarray(a, np.float32).ravel() for a in arrays])

    def pack_faces(self, arrays):
        return np.concatenate([np.asarray(a, np.float32).ravel() for a in arrays])

    # geometry and tuning -----------------------------------------------------
    def set_solid_cells(self, masks):
        """masks: list of (h, w) arrays (1 = solid), or None to clear."""
        if masks is None:
            return N.check(self._lib.pg_batch_set_solid_cells(self._h, None))
        m = np.ascontiguousarray(np.concatenate([np.asarray(a, np.uint8).ravel() for a in masks]))
        assert m.size == self.ncells
        return N.check(self._lib.pg_batch_set_solid_cells(self._h, C.c_void_p(m.ctypes.data)))

    def tile(self):
        tx, ty, fu = C.c_int32(), C.c_int32(), C.c_int32()
        N.check(self._lib.pg_batch_tile(self._h, C.byref(tx), C.byref(ty), C.byref(fu)))
        return tx.value, ty.value, bool(fu.value)

    def set_tile(self, tx, ty, fused=True):
        N.check(self._lib.pg_batch_set_tile(self._h, int(tx), int(ty), int(bool(fused))))

    def autotune(self, cache_path=None):
        self._bind()
        N.check(self._lib.pg_batch_autotune(self._h, cache_path.encode() if cache_path else None))
        return self.tile()

    # the step ------------------------------------------------------------------
    def step(self, config, vel, density, pressure, source_field=None):
        """One step of every grid; returns the per-grid solve statistics."""
        self._bind()
        prm = config.to_c()
        prm.source_enabled = 0
        prm.source_field = source_field.data_ptr() if source_field is not None else None
        stats = (N.PcgStats * len(self))()
        rc = self._lib.pg_batch_step_f32(self._h, C.byref(prm), C.c_void_p(vel.data_ptr()),
                                         C.c_void_p(density.data_ptr()), C.c_void_p(pressure.data_ptr()), stats)
        N.check(rc, allow=(N.PG_OK, N.PG_NOT_CONVERGED))
        return [s.as_dict() for s in stats]


def partition_by_cost(dims, nranks, cost=None):
    """Split a batch across ranks: largest-first greedy assignment to the
    least-loaded rank by `cost` (default: cells, the per-iteration work).
    Returns one sorted index list per rank; every grid appears exactly once
    and the step needs no data exchange between ranks."""
    costs = [(h * w if cost is None else cost(h, w)) for h, w in dims]
    order = sorted(range(len(dims)), key=lambda i: (-costs[i], i))
    load = [0] * nranks
    parts = [[] for _ in range(nranks)]
    for i in order:
        r = min(range(nranks), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]
