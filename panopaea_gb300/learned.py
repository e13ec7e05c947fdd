"""Learned initial guess for the pressure solve (extension; the reference has
no learned component).

:class:`PressureNet` wraps the device network of ``pg_unet_*`` (a 3-level
3D conv U-Net, 16 base channels, BF16 weights/activations with FP32
accumulation; forward, backward and Adam all run in the library).  It maps
(b, the grid's solid mask) to a guess of the solution of A p = b, which
:func:`solve_with_guess` hands to the FP64-refined PCG as its starting
point: the CG still runs to the same tolerance, so the network only changes
how many iterations that takes, never the answer's accuracy.

:func:`training_pair` produces one (divergence, mask) -> pressure sample:
1-6 axis-aligned solid boxes (sides 8-48 cells, scaled down on small
grids), a seeded filtered-noise velocity (i.i.d. N(0, 1) faces, 3 passes of
a 3^3 box filter, max |u| = 2, walls), b = -div u, and p from the pressure
solver run to relative residual 1e-6.
"""

import ctypes as C

import numpy as np
import torch
import torch.nn.functional as F

from . import _native as N
from .fluid import SolverConfig, solve_pressure
from .grid import Simplex1, Simplex2, _ptr

CIN = (16, 16, 16, 32, 32, 64, 96, 32, 48, 16)
COUT = (16, 16, 32, 32, 64, 64, 32, 32, 16, 16)


def num_params():
    return int(N.load().pg_unet_num_params())


def he_init(seed=0):
    """He-normal conv weights (fan-in = 27 x real input channels; the 14
    padding input channels of layer 0 get zero rows), output layer
    N(0, 0.3^2).  float32, the library's parameter layout."""
    r = np.random.default_rng(seed)
    out = np.zeros(num_params(), np.float32)
    o = 0
    for k in range(10):
        n = 27 * CIN[k] * COUT[k]
        fan = 27 * (2 if k == 0 else CIN[k])
        wk = (r.standard_normal(n) * np.sqrt(2.0 / fan)).reshape(27, CIN[k], COUT[k])
        if k == 0:
            wk[:, 2:, :] = 0
        out[o:o + n] = wk.ravel()
        o += n
    out[o:] = 0.3 * r.standard_normal(16)
    return out


class PressureNet:
    """The device network for grids of shape `dims` (d, h, w), every side a
    multiple of 4 and >= 16."""

    def __init__(self, dims, params=None, out_scale=1.0, seed=0):
        self._lib = N.load()
        self._h = C.c_void_p()
        d, h, w = (int(v) for v in dims)
        N.check(self._lib.pg_unet_create(d, h, w, C.byref(self._h)))
        self.dims = (d, h, w)
        self.set_params(he_init(seed) if params is None else params, out_scale)

    def close(self):
        if self._h:
            self._lib.pg_unet_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _bind_stream(self):
        N.check(self._lib.pg_unet_set_stream(self._h, C.c_void_p(torch.cuda.current_stream().cuda_stream)))

    def set_params(self, params, out_scale):
        p = np.ascontiguousarray(params, np.float32)
        if p.size != num_params():
            raise ValueError("expected %d parameters, got %d" % (num_params(), p.size))
        self._bind_stream()
        N.check(self._lib.pg_unet_set_params(self._h, C.c_void_p(p.ctypes.data), float(out_scale)))
        self.out_scale = float(out_scale)

    def get_params(self):
        p = np.empty(num_params(), np.float32)
        s = C.c_double()
        self._bind_stream()
        N.check(self._lib.pg_unet_get_params(self._h, C.c_void_p(p.ctypes.data), C.byref(s)))
        return p, s.value

    def get_grads(self):
        g = np.empty(num_params(), np.float32)
        self._bind_stream()
        N.check(self._lib.pg_unet_get_grads(self._h, C.c_void_p(g.ctypes.data)))
        return g

    def zero_grads(self):
        self._bind_stream()
        N.check(self._lib.pg_unet_zero_grads(self._h))

    def accumulate(self, grid, b, p_true, dt, want_loss=True):
        """Forward + backward of one sample; adds to the gradients.  Returns
        the loss (synchronises) or None."""
        self._bind_stream()
        loss = C.c_double()
        N.check(self._lib.pg_unet_accumulate_f32(self._h, grid.handle, _ptr(b.data), _ptr(p_true.data), float(dt),
                                                 C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, grad_scale=1.0):
        a = N.AdamParams(float(lr), float(beta1), float(beta2), float(eps), float(grad_scale))
        self._bind_stream()
        N.check(self._lib.pg_unet_adam_step(self._h, C.byref(a)))

    def set_loss(self, kind):
        """0 = mean squared error, 1 = energy norm (default)."""
        self._bind_stream()
        N.check(self._lib.pg_unet_set_loss(self._h, int(kind)))

    def forward(self, grid, b, dt, p):
        """p = the network's raw output for b."""
        self._bind_stream()
        N.check(self._lib.pg_unet_forward_f32(self._h, grid.handle, _ptr(b.data), float(dt), _ptr(p.data)))

    def guess(self, grid, b, dt, x, corrections=0):
        """x = the network's guess for A x = b, scaled by the step that
        minimises the error's energy norm (+ `corrections` further rounds on
        the residual)."""
        self._bind_stream()
        grid._bind_stream()
        N.check(self._lib.pg_unet_guess_f32(self._h, grid.handle, _ptr(b.data), float(dt), int(corrections),
                                            _ptr(x.data)))

    def save(self, path):
        p, s = self.get_params()
        np.savez(path, params=p, out_scale=np.float64(s), dims=np.array(self.dims))

    @classmethod
    def load(cls, path, dims=None):
        z = np.load(path)
        return cls(dims or tuple(int(v) for v in z["dims"]), params=z["params"], out_scale=float(z["out_scale"]))


def solve_with_guess(net, grid, x, b, dt, solver, corrections=0):
    """Pressure solve started from the network's guess (refined PCG; the
    tolerance is the solver's own)."""
    if solver.refine <= 0:
        raise ValueError("solve_with_guess needs solver.refine > 0")
    net.guess(grid, b, dt, x, corrections)
    cfg = SolverConfig(**{**solver.__dict__, "initial_guess": True})
    return solve_pressure(grid, x, b, dt, cfg)


def solve_learned_pcg(net, grid, x, b, dt, solver):
    """Pressure solve A x = b with the network inside the CG: for a residual
    r the preconditioner is z = a q + D^-1 (r - a A q), q = net(r), a the
    energy-optimal step along q (a flexible CG, Polak-Ribiere beta, since z
    depends on r non-linearly).  The solver's tolerance, refinement and
    initial_guess apply (its precond does not); returns the statistics."""
    net._bind_stream()
    grid._bind_stream()
    st = N.PcgStats()
    prm = solver.to_c()
    grid._call("pg_solve_pressure_learned_f32", C.byref(prm), net._h, _ptr(x.data), _ptr(b.data), C.c_double(dt),
               C.byref(st), allow=(N.PG_OK, N.PG_NOT_CONVERGED))
    return st.as_dict()


# ---------------------------------------------------------------------------
# Training data.

def box_obstacles(dims, rng, nmin=1, nmax=6, smin=8, smax=48):
    """1-6 axis-aligned solid boxes with sides smin..smax cells (scaled by
    min(dims) / 128 on smaller grids), uint8 cell mask."""
    scale = min(1.0, min(dims) / 128.0)
    lo, hi = max(2, int(round(smin * scale))), max(3, int(round(smax * scale)))
    m = np.zeros(dims, np.uint8)
    for _ in range(int(rng.integers(nmin, nmax + 1))):
        sz = [int(rng.integers(lo, hi + 1)) for _ in range(3)]
        o = [int(rng.integers(1, max(2, n - s - 1))) for n, s in zip(dims, sz)]
        m[o[0]:o[0] + sz[0], o[1]:o[1] + sz[1], o[2]:o[2] + sz[2]] = 1
    return m


def _box3_dev(a, passes):
    """`passes` passes of a 3x3x3 box filter with edge replication (the
    separable filter with edge padding per axis)."""
    a = a[None, None]
    for _ in range(passes):
        a = F.avg_pool3d(F.pad(a, (1, 1, 1, 1, 1, 1), mode="replicate"), 3, stride=1)
    return a[0, 0]


def noise_velocity(dims, seed, umax=2.0, passes=3):
    """Filtered-noise face velocity on the device, walls zeroed, max |u| = umax."""
    gen = torch.Generator(device="cuda")
    gen.manual_seed(int(seed))
    d, h, w = dims
    shapes = [(d + 1, h, w), (d, h + 1, w), (d, h, w + 1)]
    parts = []
    for ax, s in enumerate(shapes):
        p = _box3_dev(torch.randn(s, generator=gen, device="cuda"), passes)
        idx0 = tuple(0 if i == ax else slice(None) for i in range(3))
        idx1 = tuple(-1 if i == ax else slice(None) for i in range(3))
        p[idx0] = 0
        p[idx1] = 0
        parts.append(p)
    m = max(float(p.abs().max()) for p in parts)
    return torch.cat([p.reshape(-1) for p in parts]) * (umax / m)


def training_pair(grid, seed, dt=1.0, solver=None, umax=2.0, solve=True):
    """Set the grid's mask to a seeded box configuration and return
    (b, p, mask, stats): b = -div u of a seeded filtered-noise velocity, p
    its pressure to relative 1e-6 (by default plain CG in FP64 refinement;
    p and stats are None with solve=False)."""
    rng = np.random.default_rng(seed)
    dims = grid.dim()
    mask = box_obstacles(dims, rng)
    grid.set_solid_cells(mask)
    vel = Simplex1(grid, noise_velocity(dims, int(rng.integers(1 << 62)), umax))
    b = grid.new_simplex_2()
    grid.divergence_rhs(b, vel)
    del vel
    if not solve:
        return b, None, mask, None
    p = grid.new_simplex_2()
    solver = solver or SolverConfig(rel_stop=True, rel_tol=1e-6, max_iter=20000, refine=8)
    st = solve_pressure(grid, p, b, dt, solver)
    return b, p, mask, st


def estimate_out_scale(pairs, dt):
    """rms(p) * dt / rms(b) over (b, p) pairs: the output scale that makes
    the network's normalised target O(1)."""
    num = den = 0.0
    for b, p in ((t[0], t[1]) for t in pairs):
        num += float((p.data.double() ** 2).mean())
        den += float((b.data.double() ** 2).mean())
    return float(np.sqrt(num / max(den, 1e-300))) * dt


def train(net, grid, pairs, dt, epochs=1, batch=4, lr=1e-3, lr_end=None, log=None):
    """Adam over (b, p, mask) triples, `batch` samples per step, learning
    rate cosine-decayed from `lr` to `lr_end` (default lr / 20).  Returns
    the mean loss of each epoch."""
    lr_end = lr / 20 if lr_end is None else lr_end
    steps = epochs * ((len(pairs) + batch - 1) // batch)
    hist, step = [], 0
    for ep in range(epochs):
        tot, cnt, inb = 0.0, 0, 0
        for i, (b, p, mask) in enumerate(pairs):
            grid.set_solid_cells(mask)
            tot += net.accumulate(grid, b, p, dt)
            cnt += 1
            inb += 1
            if inb == batch or i == len(pairs) - 1:
                t = step / max(1, steps - 1)
                net.adam_step(lr=lr_end + 0.5 * (lr - lr_end) * (1 + np.cos(np.pi * t)), grad_scale=1.0 / inb)
                step += 1
                inb = 0
        hist.append(tot / max(cnt, 1))
        if log:
            log("epoch %d loss %.4g" % (ep, hist[-1]))
    return hist


def train_streaming(net, grid, seeds, dt, solver=None, batch=8, lr=1e-3, lr_end=None, log=None):
    """One pass over freshly generated pairs (generated, trained on, then
    dropped: nothing is stored), `batch` samples per Adam step, cosine
    learning-rate decay.  Returns (losses, seconds generating, seconds
    training)."""
    import time

    lr_end = lr / 20 if lr_end is None else lr_end
    seeds = list(seeds)
    steps = (len(seeds) + batch - 1) // batch
    losses, t_gen, t_train, step, inb = [], 0.0, 0.0, 0, 0
    for i, sd in enumerate(seeds):
        t0 = time.perf_counter()
        b, p, mask, _ = training_pair(grid, sd, dt, solver)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        losses.append(net.accumulate(grid, b, p, dt))
        inb += 1
        if inb == batch or i == len(seeds) - 1:
            t = step / max(1, steps - 1)
            net.adam_step(lr=lr_end + 0.5 * (lr - lr_end) * (1 + np.cos(np.pi * t)), grad_scale=1.0 / inb)
            step += 1
            inb = 0
        torch.cuda.synchronize()
        t_gen += t1 - t0
        t_train += time.perf_counter() - t1
        if log and (i + 1) % 500 == 0:
            log("pair %d loss %.4g" % (i + 1, float(np.mean(losses[-500:]))))
    return losses, t_gen, t_train


__all__ = ["PressureNet", "he_init", "num_params", "solve_with_guess", "training_pair", "box_obstacles",
           "noise_velocity", "estimate_out_scale", "train", "train_streaming", "Simplex2"]
