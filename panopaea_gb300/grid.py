"""Device-backed mirror of the reference's grid, field and DEC operator API.

The reference (msiglreith/panopaea) names these in Rust:

* ``Grid2d::new((h, w))`` / ``Grid2d::dim()`` -- domain/grid.rs:2-15;
  ``Grid3d`` -- domain/grid.rs:17-20 (declared only; defined here);
* ``Simplex1`` (face field, one buffer [vy (h+1)w | vx h(w+1)], ``split``)
  and ``Simplex2`` (cell field) -- dec/grid.rs:36-100;
* ``Manifold2d`` methods ``new_simplex_1/2``, ``hodge_1_dual``,
  ``hodge_1_primal``, ``hodge_2_primal``, ``derivative_0_dual``,
  ``derivative_1_primal`` -- dec/manifold.rs:29-83.

Here the storage is a CUDA tensor (torch provides only device memory and the
stream) and every operator is one call into ``libpanopaea_gpu.so``.
Arguments keep the reference's order: destination first.
"""

import ctypes as C

import torch

from . import _native as N


def _sfx(t):
    if t.dtype == torch.float32:
        return "f32"
    if t.dtype == torch.float64:
        return "f64"
    raise TypeError("fields must be float32 or float64, got %s" % t.dtype)


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class _Field:
    def view_linear(self):
        """math/linear_view.rs:5-9: the flat 1-D view."""
        return self.data.view(-1)

    def view_linear_mut(self):
        return self.data.view(-1)

    @property
    def dtype(self):
        return self.data.dtype

    def fill(self, v):
        self.data.fill_(v)
        return self

    def assign(self, other):
        self.data.copy_(other.data)
        return self

    def cpu(self):
        return self.data.detach().cpu()


class Simplex1(_Field):
    """Face field (dec/grid.rs:36-73).  `data` is 1-D of num_elem_1 values."""

    def __init__(self, grid, data):
        if data.numel() != grid.num_elem_1():
            raise ValueError("Simplex1 needs %d values, got %d" % (grid.num_elem_1(), data.numel()))
        self.grid = grid
        self.data = data.reshape(-1)

    def dim(self):
        return self.grid.dim()

    def split(self):
        """(vertical, horizontal) views, dec/grid.rs:47-53; 3D: (vz, vy, vx)."""
        g = self.grid
        if g.ndim == 2:
            h, w = g.dim()
            n0 = (h + 1) * w
            return self.data[:n0].view(h + 1, w), self.data[n0:].view(h, w + 1)
        d, h, w = g.dim()
        nz, ny = (d + 1) * h * w, d * (h + 1) * w
        return (self.data[:nz].view(d + 1, h, w), self.data[nz:nz + ny].view(d, h + 1, w),
                self.data[nz + ny:].view(d, h, w + 1))

    split_mut = split


class Simplex2(_Field):
    """Cell field (dec/grid.rs:76-100): (h, w), or (d, h, w) in 3D."""

    def __init__(self, grid, data):
        shape = grid.dim()
        if tuple(data.shape) != tuple(shape):
            data = data.reshape(shape)
        self.grid = grid
        self.data = data

    def dim(self):
        return self.grid.dim()


class _GridBase:
    ndim = 0

    def __init__(self):
        self._lib = N.load()
        self._h = C.c_void_p()
        self.device = torch.device("cuda", torch.cuda.current_device())

    def _bind_stream(self):
        N.check(self._lib.pg_grid_set_stream(self._h, C.c_void_p(torch.cuda.current_stream().cuda_stream)))

    def _call(self, name, *args, allow=(N.PG_OK,)):
        self._bind_stream()
        return N.check(getattr(self._lib, name)(self._h, *args), allow)

    def close(self):
        if self._h:
            self._lib.pg_grid_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # --- sizes (dec/grid.rs:346-356) ---------------------------------------
    def num_elem_1(self):
        return int(self._lib.pg_grid_num_elem_1(self._h))

    def num_elem_2(self):
        return int(self._lib.pg_grid_num_elem_2(self._h))

    # --- storage (dec/grid.rs:358-371) ---------------------------------------
    def new_simplex_1(self, dtype=torch.float32):
        return Simplex1(self, torch.zeros(self.num_elem_1(), dtype=dtype, device=self.device))

    def new_simplex_2(self, dtype=torch.float32):
        return Simplex2(self, torch.zeros(self.dim(), dtype=dtype, device=self.device))

    # --- solid masks (examples/dec_fluid.rs:71-78 as data) -------------------
    def set_solid_faces(self, face_solid):
        """1 = solid, in the face layout; None clears."""
        if face_solid is None:
            return self._call("pg_grid_set_solid_faces", None)
        m = torch.as_tensor(face_solid).to(torch.uint8).reshape(-1).contiguous().cpu()
        if m.numel() != self.num_elem_1():
            raise ValueError("face mask needs %d entries" % self.num_elem_1())
        return self._call("pg_grid_set_solid_faces", C.c_void_p(m.data_ptr()))

    def set_solid_cells(self, cell_solid):
        if cell_solid is None:
            return self._call("pg_grid_set_solid_cells", None)
        m = torch.as_tensor(cell_solid).to(torch.uint8).reshape(-1).contiguous().cpu()
        if m.numel() != self.num_elem_2():
            raise ValueError("cell mask needs %d entries" % self.num_elem_2())
        return self._call("pg_grid_set_solid_cells", C.c_void_p(m.data_ptr()))

    # --- Manifold2d operators (dec/manifold.rs:50-80) ------------------------
    def hodge_1_dual(self, primal, dual):
        self._call("pg_hodge_1_dual_" + _sfx(primal.data), _ptr(primal.data), _ptr(dual.data))

    def hodge_1_primal(self, dual, primal):
        self._call("pg_hodge_1_primal_" + _sfx(dual.data), _ptr(dual.data), _ptr(primal.data))

    def hodge_2_primal(self, dual, primal):
        self._call("pg_hodge_2_primal_" + _sfx(dual.data), _ptr(dual.data), _ptr(primal.data))

    def derivative_1_primal(self, faces, edges):
        self._call("pg_derivative_1_primal_" + _sfx(faces.data), _ptr(faces.data), _ptr(edges.data))

    def derivative_0_dual(self, edges, faces):
        self._call("pg_derivative_0_dual_" + _sfx(edges.data), _ptr(edges.data), _ptr(faces.data))

    def mask_solid_faces(self, edges):
        self._call("pg_mask_solid_faces_" + _sfx(edges.data), _ptr(edges.data))

    # --- fused operators -----------------------------------------------------
    def laplacian(self, out, p, dt):
        """The PCG operator closure of examples/dec_fluid.rs:100-119."""
        self._call("pg_laplacian_" + _sfx(out.data), _ptr(out.data), _ptr(p.data), C.c_double(dt))

    def divergence_rhs(self, b, vel):
        """-div of examples/dec_fluid.rs:68-83."""
        self._call("pg_divergence_rhs_" + _sfx(b.data), _ptr(b.data), _ptr(vel.data))

    def project(self, vel, pressure, dt, zero_solid=False):
        """examples/dec_fluid.rs:123-141."""
        self._call("pg_project_" + _sfx(vel.data), _ptr(vel.data), _ptr(pressure.data), C.c_double(dt),
                   int(bool(zero_solid)))

    def walls(self, vel):
        self._call("pg_walls_" + _sfx(vel.data), _ptr(vel.data))

    def synchronize(self):
        self._call("pg_grid_synchronize")


class Grid2d(_GridBase):
    """domain/grid.rs:2-15; dim = (h, w) = (y, x)."""

    ndim = 2

    def __init__(self, dim):
        super().__init__()
        h, w = dim
        N.check(self._lib.pg_grid_create_2d(int(h), int(w), C.byref(self._h)))
        self._dim = (int(h), int(w))

    def dim(self):
        return self._dim


class Grid3d(_GridBase):
    """domain/grid.rs:17-20 (struct only in the reference); dim = (d, h, w)."""

    ndim = 3

    def __init__(self, dim):
        super().__init__()
        d, h, w = dim
        N.check(self._lib.pg_grid_create_3d(int(d), int(h), int(w), C.byref(self._h)))
        self._dim = (int(d), int(h), int(w))

    def dim(self):
        return self._dim
