"""The fluid step of examples/dec_fluid.rs on the device.

* :func:`advect` -- examples/dec_fluid.rs:173-211 (bilinear; trilinear in 3D);
* :func:`advect_mac` -- examples/dec_fluid.rs:213-291;
* :func:`step` -- one iteration of the loop at examples/dec_fluid.rs:46-141
  (inflow, advection, -div, PCG, projection, walls), with the extension
  switches of :class:`StepConfig` (buoyancy, wall-consistent RHS, relative
  stop rule, Jacobi/MG preconditioners, FP64 residual refinement).
"""

import ctypes as C
from dataclasses import dataclass, field

import torch

from . import _native as N
from .grid import _ptr, _sfx


def advect(dst, src, timestep, vel):
    """examples/dec_fluid.rs:173-211: dst = src sampled at x - dt * u(x)."""
    g = src.grid
    g._call("pg_advect_" + _sfx(dst.data), _ptr(dst.data), _ptr(src.data), C.c_double(timestep), _ptr(vel.data))


MACCORMACK, BFECC = 1, 2


def advect2(dst, src, timestep, vel, scheme=MACCORMACK):
    """Second-order limited advection of a cell scalar (extension)."""
    g = src.grid
    g._call("pg_advect2_" + _sfx(dst.data), _ptr(dst.data), _ptr(src.data), C.c_double(timestep), _ptr(vel.data),
            int(scheme))


def advect_mac(dst, src, timestep, vel):
    """examples/dec_fluid.rs:213-291: MAC face advection."""
    g = src.grid
    g._call("pg_advect_mac_" + _sfx(dst.data), _ptr(dst.data), _ptr(src.data), C.c_double(timestep),
            _ptr(vel.data))


@dataclass
class SolverConfig:
    precond: int = N.PG_PRECOND_NONE
    rel_stop: bool = False
    threshold: float = 0.1          # dec_fluid.rs:44
    rel_tol: float = 1e-6
    max_iter: int = 100             # dec_fluid.rs:95
    refine: int = 0
    check_every: int = 0
    inner_rel_tol: float = 0.0
    mg_levels: int = 0
    mg_smooth: int = 0
    fp64_native: bool = False
    initial_guess: bool = False      # refine > 0: x holds a starting guess

    def to_c(self):
        p = N.SolverParams()
        p.precond = int(self.precond)
        p.rel_stop = int(bool(self.rel_stop))
        p.threshold = float(self.threshold)
        p.rel_tol = float(self.rel_tol)
        p.max_iter = int(self.max_iter)
        p.refine = int(self.refine)
        p.check_every = int(self.check_every)
        p.inner_rel_tol = float(self.inner_rel_tol)
        p.mg_levels = int(self.mg_levels)
        p.mg_smooth = int(self.mg_smooth)
        p.fp64_native = int(bool(self.fp64_native))
        p.initial_guess = int(bool(self.initial_guess))
        return p


@dataclass
class StepConfig:
    """Defaults are the reference's dec_fluid.rs configuration (128x128 inflow box)."""

    dt: float = 0.05                 # dec_fluid.rs:43
    buoyancy: float = 0.0
    source_enabled: bool = True      # dec_fluid.rs:48-57
    source_lo: tuple = (0, 5, 54)    # (z, y, x)
    source_hi: tuple = (1, 20, 64)
    source_density: float = 1.0
    source_vy: float = 20.0
    source_field: object = None      # optional device cell field (Simplex2)
    walls_after_advect: bool = False
    zero_solid_after_project: bool = False
    advect_scheme: int = 0           # 0 reference, 1 MacCormack, 2 BFECC (density)
    solver: SolverConfig = field(default_factory=SolverConfig)

    def to_c(self):
        p = N.StepParams()
        p.dt = float(self.dt)
        p.buoyancy = float(self.buoyancy)
        p.source_enabled = int(bool(self.source_enabled))
        p.walls_after_advect = int(bool(self.walls_after_advect))
        for i in range(3):
            p.source_lo[i] = int(self.source_lo[i])
            p.source_hi[i] = int(self.source_hi[i])
        p.source_density = float(self.source_density)
        p.source_vy = float(self.source_vy)
        p.source_field = self.source_field.data.data_ptr() if self.source_field is not None else None
        p.zero_solid_after_project = int(bool(self.zero_solid_after_project))
        p.advect_scheme = int(self.advect_scheme)
        p.solver = self.solver.to_c()
        return p


def solve_pressure(grid, x, b, timestep, solver):
    """Pressure solve A x = b (library-owned work vectors); returns stats."""
    st = N.PcgStats()
    prm = solver.to_c()
    grid._call("pg_solve_pressure_f32", C.byref(prm), _ptr(x.data), _ptr(b.data), C.c_double(timestep),
               C.byref(st), allow=(N.PG_OK, N.PG_NOT_CONVERGED))
    return st.as_dict()


def step(grid, config, vel, density, pressure):
    """One fluid step in place; returns the pressure-solve statistics.  A
    bfloat16 density field selects the BF16-stored density step (FP32
    velocity and pressure)."""
    st = N.PcgStats()
    prm = config.to_c()
    name = "pg_step_bf16rho_f32" if density.data.dtype == torch.bfloat16 else "pg_step_" + _sfx(vel.data)
    grid._call(name, C.byref(prm), _ptr(vel.data), _ptr(density.data), _ptr(pressure.data),
               C.byref(st), allow=(N.PG_OK, N.PG_NOT_CONVERGED))
    return st.as_dict()


def advect_bf16(dst, src, timestep, vel):
    """advect of a bfloat16 cell field with an FP32 velocity."""
    g = src.grid
    g._call("pg_advect_bf16", _ptr(dst.data), _ptr(src.data), C.c_double(timestep), _ptr(vel.data))
