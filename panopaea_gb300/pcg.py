"""``precond_conjugate_gradient`` with the reference's signature (pcg.rs:14-82).

The reference takes the operator as a closure ``FnMut(&mut L, &L)``.  A
closure cannot run on the device through a C ABI, so the operator must be a
:class:`LaplacianOperator` -- the masked Laplacian closure of
examples/dec_fluid.rs:100-119 (``dt * d1 *1^-1 M d0dual *2``), which the
library evaluates in a fused kernel.  Any other callable raises TypeError.

The preconditioner argument mirrors ``trait Preconditioner`` (pcg.rs:4-6):
``()`` / ``None`` / :data:`IDENTITY` is the reference's identity impl
(pcg.rs:8-12); :data:`JACOBI` is an extension.
"""

import ctypes as C

from . import _native as N
from .grid import _ptr, _sfx


class Preconditioner:
    def __init__(self, kind, name):
        self.kind = kind
        self.name = name

    def __repr__(self):
        return "Preconditioner(%s)" % self.name


IDENTITY = Preconditioner(N.PG_PRECOND_NONE, "()")
JACOBI = Preconditioner(N.PG_PRECOND_JACOBI, "jacobi")


class LaplacianOperator:
    """The operator closure of examples/dec_fluid.rs:100-119 for `grid` and `dt`."""

    def __init__(self, grid, timestep):
        self.grid = grid
        self.timestep = float(timestep)

    def __call__(self, out, p):
        self.grid.laplacian(out, p, self.timestep)


def _kind(preconditioner):
    if preconditioner is None or preconditioner == ():
        return N.PG_PRECOND_NONE
    if isinstance(preconditioner, Preconditioner):
        return preconditioner.kind
    raise TypeError("unsupported preconditioner %r" % (preconditioner,))


def precond_conjugate_gradient(preconditioner, x, b, max_iterations, threshold, residual, auxiliary, search, a):
    """pcg.rs:14-82 on the device.  Returns the solve statistics (a dict).

    Stop rule and recurrence are the reference's: x = 0; return at once if
    ||b||inf < threshold; stop when ||r||inf < threshold or after
    max_iterations operator applications.  Dot products accumulate in FP64.
    """
    if not isinstance(a, LaplacianOperator):
        raise TypeError("the operator must be a LaplacianOperator: host closures cannot run on the device")
    g = a.grid
    st = N.PcgStats()
    g._call("pg_pcg_" + _sfx(x.data), _kind(preconditioner), _ptr(x.data), _ptr(b.data), int(max_iterations),
            C.c_double(threshold), _ptr(residual.data), _ptr(auxiliary.data), _ptr(search.data),
            C.c_double(a.timestep), C.byref(st), allow=(N.PG_OK, N.PG_NOT_CONVERGED))
    return st.as_dict()
