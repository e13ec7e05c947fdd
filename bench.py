#!/usr/bin/env python
"""Throughput of the grid-fluid step on GB300, in Mcell-steps/s.

Default workload: the 3D precision study -- a 256^3 MAC grid, f32 fields,
filtered-noise velocity (max |u| = 2 cells/step, dt = 1), solid walls; a
step is trilinear advection of velocity and density, the 7-point pressure
projection to relative residual 1e-6, and the gradient subtraction.  Each
step continues the simulation from the previous one.

Two solver forms run on the same workload:
  chosen -- multigrid-preconditioned CG (falls back to Jacobi-PCG when the
            library has no MG) inside FP64 residual refinement;
  plain  -- the reference's unpreconditioned CG in FP32 storage.
`value` is the chosen form; the plain form is reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

K defaults to 50 (0.24 s of timed work at 256^3, so the clock samples --
nvidia-smi polled every 50 ms from before the timed region -- fall inside
it), W to 3.

Multi-GPU (torchrun, one rank per GPU): every rank advances its own replica
grid (the step has no data-path exchange), `value` = all cells x steps over
the max time over ranks ("scaling": "weak").

--impl reference times the reference's CPU algorithm (the oracle restatement,
the reference's threading: derivative_0_dual / derivative_1_primal parallel,
everything else serial) on the host cores: whole steps, each run to
convergence and timed, as many as fit in --ref-budget seconds (at least
one); the same steps with every loop parallel are reported beside them.
The CPU baseline of the GPU line is one such whole step with every loop
parallel.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s at rel. residual 1e-6 on 1 GB300; chosen form vs plain FP32 PCG"
UNIT = "Mcell-steps/s"

# Algorithmic bytes per cell for one launch of each kernel kind (f32 fields,
# uint8 face-open flags), 3D / 2D: the unique bytes each launch must move.
BYTES_PER_CELL = {
    "cg_spmv": (17, 17),        # r, p_old, flags in; p_new, Ap out
    "cg_update": (24, 24),      # x, p, r, Ap in; x, r out (Jacobi: +1 flags)
    "cg_init": (13, 13),        # b in; x, r out; flags (Jacobi)
    "advect": (20, 16),         # rho + 3 (2) faces in, rho out
    "advect_mac": (24, 16),     # 3 (2) faces in (self-advection), 3 (2) out
    "rhs": (17, 13),            # faces + flags in, b out
    "project": (29, 21),        # p, faces, flags in; faces out
    "residual64": (17, 17),     # b, x64, flags in; r out
    "refine_update": (20, 20),  # x64, d in; x64 out
    # fine-level multigrid kernels, per fine cell:
    "mg_smooth": (6.5, 6.5),    # half-sweep: f, flags of its colour, e of the other in; e of its colour out
    # fused red-black pair (3D): e, f, flags in, e out = 13; the first pre-smoothing pair reads no e (9), the
    # first post-smoothing one also the coarse correction (13.5): 12.125 averaged over a 2-sweep V-cycle
    "mg_pair": (12.125, 12.125),
    "mg_restrict": (9.5, 9.5),  # e, f, flags in; coarse f (1/8 or 1/4 of the cells) out
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 50: a timed region long enough for the clock samples to fall in; "
                         "5 bounded CPU samples for --impl reference)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="precision_3d_256")
    ap.add_argument("--dims", default=None, help="override, e.g. 128,128,128")
    ap.add_argument("--plain-steps", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-PCG comparison (profiling runs)")
    ap.add_argument("--ref-budget", type=float, default=150.0,
                    help="--impl reference: seconds of timed full CPU steps (at least one step is timed)")
    ap.add_argument("--no-precision", action="store_true", help="skip the FP64 / BF16 precision study")
    ap.add_argument("--pairs", type=int, default=10000, help="learned_3d_128: training pairs (streamed)")
    ap.add_argument("--held", type=int, default=256, help="learned_3d_128: held-out grids")
    ap.add_argument("--held-fcg", type=int, default=32,
                    help="learned_3d_128: held-out grids solved by the flexible CG with the network inside (the "
                         "first ones; a network forward per iteration)")
    ap.add_argument("--gen", default="mg", choices=["mg", "plain"], help="learned_3d_128: solver of the pairs")
    ap.add_argument("--batch-count", type=int, default=512, help="batch_512: number of grids")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 5 if args.impl == "reference" else 50
    return args


# ---------------------------------------------------------------------------
# distributed plumbing (replicas; only the barrier and the max over ranks)

def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, ws, rank, local, backend):
        import torch

        self.ws, self.rank, self.local = ws, rank, local
        self.torch = torch
        self.pg = None
        if ws > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            if self.torch.cuda.is_available():
                self.pg.barrier(device_ids=[self.local])
            else:
                self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        dev = "cuda" if self.torch.cuda.is_available() else "cpu"
        t = self.torch.tensor([float(v)], dtype=self.torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks during the timed region

class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # the timed region starts once the sampler is producing samples
            t_end = time.time() + 3.0
            while time.time() < t_end and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.06)  # the sample in flight at the end of the region
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        with open(self.path) as f:
            lines = f.read().splitlines()
        os.unlink(self.path)
        return self.summarize(lines)

    @staticmethod
    def summarize(lines):
        """nvidia-smi CSV rows (the query Q, no header, no units) -> the
        `clocks` object: median SM clock over the loaded samples (power at
        least half the peak seen), the maximum clock, and every throttle
        reason that was active in any sample."""
        rows = []
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append(dict(sm=float(f[1]), smax=float(f[2]), power=float(f[3]), hw=f[5], hwt=f[6], swt=f[7],
                                 pcap=f[8]))
            except ValueError:
                continue
        if not rows:
            return None
        pmax = max(r["power"] for r in rows)
        load = [r for r in rows if r["power"] >= 0.5 * pmax] or rows
        reasons = set()
        for r in rows:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                              ("pcap", "sw_power_cap")):
                if r[key].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in load), "sm_max_mhz": max(r["smax"] for r in rows),
                "power_w_max": pmax, "samples": len(rows), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------

def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kind, workload):
    """Per-launch DRAM bytes of `kind` from the committed ncu summary, if any
    (lines `traffic <kind> <workload> <bytes_per_launch>`)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for ln in open(path):
        f = ln.split()
        if len(f) >= 4 and f[0] == "traffic" and f[1] == kind and f[2] == workload:
            return float(f[3])
    return None


def solver_cfgs(pg, spec, have_mg):
    """(chosen, comparison): MG-PCG in FP64 refinement, and the plain FP32
    PCG of the reference (or Jacobi-PCG in refinement, where the workload
    names that comparison)."""
    rel_tol = spec["rel_tol"]
    chosen = pg.SolverConfig(precond=2 if have_mg else 1, rel_stop=True, rel_tol=rel_tol, max_iter=20000, refine=4)
    if spec.get("compare") == "jacobi":
        other = pg.SolverConfig(precond=1, rel_stop=True, rel_tol=rel_tol, max_iter=200000, refine=4)
    else:
        other = pg.SolverConfig(precond=0, rel_stop=True, rel_tol=rel_tol, max_iter=200000)
    return chosen, other


def e2e_pipelined(torch, pg, dist, grid, cfg, fresh, vel0, rho0, steps, ws, cells):
    """Steps of independent frames through the public API with host buffers:
    every step copies its frame's velocity and density in from pinned host
    memory and its result back out, inside the timed region.  The copies run
    on a second stream over two device buffer sets, so the copy-in of the
    next frame and the copy-out of the previous one overlap the current
    step (which runs on the grid's stream, its scratch shared by both sets).
    The first copy-in and the last copy-out are not overlapped."""
    hin_v = torch.from_numpy(vel0.copy()).pin_memory()
    hin_r = torch.from_numpy(rho0.copy()).pin_memory()
    hout = [(torch.empty_like(hin_v).pin_memory(), torch.empty_like(hin_r).pin_memory()) for _ in range(2)]
    sets = [fresh(), fresh()]
    comp = torch.cuda.current_stream()
    cs = torch.cuda.Stream()
    h2d_done = [torch.cuda.Event() for _ in range(2)]
    c_done = [torch.cuda.Event() for _ in range(2)]

    def h2d(k):
        v, r, _ = sets[k % 2]
        with torch.cuda.stream(cs):
            v.data.copy_(hin_v, non_blocking=True)
            r.data.copy_(hin_r, non_blocking=True)
            h2d_done[k % 2].record(cs)

    def d2h(k):
        v, r, _ = sets[k % 2]
        with torch.cuda.stream(cs):
            cs.wait_event(c_done[k % 2])
            hout[k % 2][0].copy_(v.data, non_blocking=True)
            hout[k % 2][1].copy_(r.data, non_blocking=True)

    dist.barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(comp)
    cs.wait_event(t0)
    h2d(0)
    for k in range(steps):
        if k + 1 < steps:
            h2d(k + 1)  # behind the copy-out of frame k - 1, which used the same set
        comp.wait_event(h2d_done[k % 2])
        pg.step(grid, cfg, *sets[k % 2])
        c_done[k % 2].record(comp)
        d2h(k)
    last = torch.cuda.Event()
    last.record(cs)
    comp.wait_event(last)
    t1.record(comp)
    torch.cuda.synchronize()
    dist.barrier()
    ms_e = dist.max(t0.elapsed_time(t1))
    nb = (vel0.size + rho0.size) * 4
    return {"value": ws * cells * steps / (ms_e / 1e3) / 1e6, "unit": UNIT, "h2d_bytes_per_step": nb,
            "d2h_bytes_per_step": nb, "ms_per_step": ms_e / steps,
            "frames": "independent frames from pinned host memory; copies overlap the neighbouring steps on a "
                      "second stream (two device buffer sets)"}


def step_cfg(pg, spec, solver, source_field=None):
    return pg.StepConfig(dt=spec["dt"], buoyancy=spec["buoyancy"], source_enabled=False, walls_after_advect=True,
                         zero_solid_after_project=True, source_field=source_field, solver=solver)


def have_mg(pg, grid):
    """Probe the MG preconditioner on a tiny problem."""
    import torch

    g = pg.Grid3d((8, 8, 8)) if grid.ndim == 3 else pg.Grid2d((8, 8))
    b = g.new_simplex_2()
    b.data.view(-1)[0], b.data.view(-1)[-1] = 1.0, -1.0
    x = g.new_simplex_2()
    try:
        st = pg.solve_pressure(g, x, b, 1.0, pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=100))
        torch.cuda.synchronize()
        return st["status"] == 0
    except Exception:
        return False


# ---------------------------------------------------------------------------
# CPU: the reference algorithm on the host cores (oracle restatement)

def _threads():
    return os.cpu_count() or 1


def cpu_full_step(O, dims, spec, vel0, rho0, all_loops, src=None, fs=None):
    """One full step of the reference algorithm on the host, from the given
    state: inflow, advection, RHS, the reference's CG (identity
    preconditioner, f32 storage and f32 dot sums, pcg.rs:14-82) run to
    convergence at the workload's relative tolerance, projection.  Nothing is
    truncated or extrapolated.  Returns the wall time and the CG's iteration
    count."""
    O.set_threads(_threads(), all_loops=all_loops)
    vel = vel0.astype(np.float32).copy()
    rho = rho0.astype(np.float32).copy()
    p = np.zeros(rho.shape, np.float32)
    prm = O.step_params(dt=spec["dt"], buoyancy=spec["buoyancy"], source_field=src, walls_after_advect=True,
                        zero_solid_after_project=True, precond=0, rel_stop=True, rel_tol=spec["rel_tol"],
                        max_iter=10_000_000)
    t0 = time.perf_counter()
    st = O.step(vel, rho, p, dims, prm, fs)
    t1 = time.perf_counter()
    return {"s": t1 - t0, "iterations": int(st.iterations), "converged": bool(st.converged)}


def cpu_timed_steps(O, dims, spec, vel0, rho0, all_loops, max_steps, budget_s):
    """Full reference steps from the same initial state, timed one by one:
    at least one, then more while the next (estimated as the last) still
    fits in budget_s and max_steps is not reached."""
    runs = []
    while len(runs) < max(1, max_steps):
        if runs and sum(r["s"] for r in runs) + runs[-1]["s"] > budget_s:
            break
        runs.append(cpu_full_step(O, dims, spec, vel0, rho0, all_loops))
    cells = int(np.prod(dims))
    med = statistics.median(r["s"] for r in runs)
    return {"value": cells / med / 1e6, "ms_per_step": 1e3 * med, "steps": len(runs),
            "iterations": [r["iterations"] for r in runs], "converged": all(r["converged"] for r in runs),
            "seconds": [r["s"] for r in runs]}


THREADING = {False: "reference (derivative_0_dual / derivative_1_primal parallel as rayon runs them, the rest "
                    "serial as written)",
             True: "every loop parallel, reductions in per-thread slices (a parallelised port, faster than the "
                   "reference as written)"}


def cpu_warmup(O, spec, nd, warmup):
    """Untimed warm-up of the host path: `warmup` full steps of a 64^3 (64^2)
    grid, which bring the library and OpenMP's thread pool up."""
    small = (64,) * nd
    from panopaea_gb300 import workloads as W

    v, r = W.filtered_noise_velocity(small), (W.filtered_noise_density(small) if nd == 3 else
                                               W.gaussian_blob_2d(small))
    for _ in range(warmup):
        cpu_full_step(O, small, spec, v, r, False)


def oracle_fp64_step(O, dims, spec, vel0, rho0):
    """The all-FP64 oracle step (FP64 fields, Jacobi-PCG to relative 1e-10,
    every loop parallel) from the initial state: the reference result of the
    precision study."""
    O.set_threads(_threads(), all_loops=True)
    v = vel0.astype(np.float64)
    r = rho0.astype(np.float64)
    p = np.zeros(r.shape)
    prm = O.step_params(dt=spec["dt"], buoyancy=spec["buoyancy"], walls_after_advect=True,
                        zero_solid_after_project=True, precond=1, rel_stop=True, rel_tol=1e-10, max_iter=10_000_000)
    t0 = time.perf_counter()
    st = O.step(v, r, p, dims, prm)
    return v, r, {"form": "CPU oracle: FP64 fields, FP64 Jacobi-PCG to relative 1e-10, every loop parallel",
                  "s": time.perf_counter() - t0, "iterations": int(st.iterations), "threads": _threads()}


def cpu_leg(O, dims, spec, vel0, rho0, prec_fields):
    """Rank 0, N = 1: the CPU baseline -- one full step of the reference
    algorithm with every loop parallel on the host cores, measured (a
    bounded sample of the workload: one step) -- and, for the precision
    study, the oracle's all-FP64 step from the same initial state, against
    which the GPU forms' fields are compared."""
    cpu_warmup(O, spec, len(dims), 1)
    b = cpu_timed_steps(O, dims, spec, vel0, rho0, True, 1, 0.0)
    cpu = {"value": b["value"], "unit": UNIT, "cores": _threads(), "kind": "port",
           "sample": "one full %s step from the initial state (inflow, advection, RHS, the reference's "
                     "unpreconditioned CG in f32 to relative %g: %d iterations, projection), measured, nothing "
                     "extrapolated; threading: %s" % ("x".join(map(str, dims)), spec["rel_tol"],
                                                       b["iterations"][0], THREADING[True]),
           "ms_per_step": b["ms_per_step"], "iterations": b["iterations"][0], "extrapolated": False}
    oracle64 = None
    if prec_fields is not None:
        v64, r64, info = oracle_fp64_step(O, dims, spec, vel0, rho0)

        def rel(a, b_):
            a, b_ = a.ravel(), b_.ravel()
            return float(np.abs(a - b_).max() / max(np.abs(b_).max(), 1e-300))

        oracle64 = dict(info)
        for k, (gv, gr) in prec_fields.items():
            oracle64[k] = {"velocity_rel_linf": rel(gv, v64), "density_rel_linf": rel(gr, r64)}
    return cpu, oracle64


def reference_arm(args, spec, dims):
    """The reference's CPU algorithm (the oracle restatement) on the host
    cores, full steps measured one by one from the workload's initial state.
    `value` uses the reference's own threading; the same steps with every
    loop parallel are reported beside it.  Warm-up: `--warmup` untimed full
    steps of a 64^3 grid; the timed steps run until --ref-budget seconds
    would be exceeded (at least one)."""
    ws, rank, local = dist_setup()
    if rank != 0:
        return
    from oracle import pyoracle as O
    from panopaea_gb300 import workloads as W

    vel0, rho0 = W.initial_state(args.workload, dims)
    cpu_warmup(O, spec, len(dims), args.warmup)
    ref = cpu_timed_steps(O, dims, spec, vel0, rho0, False, args.steps, args.ref_budget)
    par = cpu_timed_steps(O, dims, spec, vel0, rho0, True, args.steps, args.ref_budget / 2)
    value = ref["value"]
    sample = ("%d full %s step(s) from the initial state, each timed whole: inflow, advection, RHS, the "
              "reference's unpreconditioned CG in f32 (f32 dot sums) to relative %g (%s iterations), "
              "projection; nothing extrapolated; warm-up %d untimed 64^3 steps" %
              (ref["steps"], "x".join(map(str, dims)), spec["rel_tol"], ref["iterations"], args.warmup))
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": ref["steps"], "requested_steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ref["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "dims": list(dims), "form": "reference CG (identity preconditioner)",
                   "threading": THREADING[False]},
        "iterations_per_step": ref["iterations"], "seconds_per_step": ref["seconds"],
        "all_loops_parallel": {"value": par["value"], "unit": UNIT, "ms_per_step": par["ms_per_step"],
                               "steps": par["steps"], "iterations_per_step": par["iterations"],
                               "threading": THREADING[True]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": _threads(), "kind": "port", "sample": sample,
                         "extrapolated": False},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------

def precision_study(torch, pg, grid, spec, vel0, rho0, chosen, src):
    """One step from the initial state three ways: the chosen FP32 form, the
    same with the density stored in BF16, and an all-FP64 step (FP64 fields,
    FP64 Jacobi-PCG to relative 1e-10).  Relative L-inf differences of
    velocity and density against FP64, and each form's device time."""
    def one(vel_t, rho_t, cfg):
        gv, gr = pg.Simplex1(grid, vel_t.clone()), pg.Simplex2(grid, rho_t.clone())
        gp = pg.Simplex2(grid, torch.zeros(rho_t.shape, dtype=vel_t.dtype, device="cuda"))
        pg.step(grid, cfg, gv, gr, gp)  # warm-up (workspaces, graphs), then the same state again
        gv.data.copy_(vel_t)
        gr.data.copy_(rho_t)
        gp.data.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        st = pg.step(grid, cfg, gv, gr, gp)
        e1.record()
        torch.cuda.synchronize()
        return gv.data.double(), gr.data.double(), st, e0.elapsed_time(e1)

    def rel(a, b):
        return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))

    cfg32 = step_cfg(pg, spec, chosen, src)
    v32, r32, s32, t32 = one(torch.from_numpy(vel0).cuda(), torch.from_numpy(rho0).reshape(grid.dim()).cuda(), cfg32)
    vb, rb, sb, tb = one(torch.from_numpy(vel0).cuda(), torch.from_numpy(rho0).reshape(grid.dim()).cuda().to(torch.bfloat16), cfg32)
    s64 = pg.SolverConfig(precond=1, rel_stop=True, rel_tol=1e-10, max_iter=200000)
    cfg64 = step_cfg(pg, spec, s64, None)
    v64, r64, st64, t64 = one(torch.from_numpy(vel0).double().cuda(), torch.from_numpy(rho0).reshape(grid.dim()).double().cuda(), cfg64)
    study = {
        "step": "one step from the initial state",
        "fp64_gpu": {"form": "this library's FP64 entry points: FP64 fields, FP64 Jacobi-PCG to relative 1e-10",
                     "ms": t64, "iterations": st64["iterations"]},
        "fp32_refined": {"velocity_rel_linf_vs_fp64_gpu": rel(v32, v64), "density_rel_linf_vs_fp64_gpu": rel(r32, r64),
                         "ms": t32, "iterations": s32["iterations"],
                         "true_residual_rel": s32["true_residual_max"] / s32["b_max"] if s32["b_max"] else 0.0},
        "bf16_density": {"velocity_rel_linf_vs_fp64_gpu": rel(vb, v64), "density_rel_linf_vs_fp64_gpu": rel(rb, r64),
                         "density_rel_linf_vs_fp32": rel(rb, r32), "ms": tb, "iterations": sb["iterations"]},
    }
    # host copies for the comparison with the CPU oracle's FP64 step
    fields = {k: (v.cpu().numpy(), r.cpu().numpy().ravel()) for k, (v, r) in
              {"fp32_refined": (v32, r32), "bf16_density": (vb, rb), "fp64_gpu": (v64, r64)}.items()}
    return study, fields


def timed_steps(torch, pg, dist, grid, cfg, gv, gr, gp, k):
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(k):
        stats.append(pg.step(grid, cfg, gv, gr, gp))
    e1.record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    return e0.elapsed_time(e1), stats


def ours(args, spec, dims):
    import torch

    import panopaea_gb300 as pg
    from panopaea_gb300 import _native as N
    from panopaea_gb300 import workloads as W

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = Dist(ws, rank, local, "nccl")
    lib = pg.load()
    cells = int(np.prod(dims))
    vel0, rho0 = W.initial_state(args.workload, dims)
    grid = pg.Grid3d(dims) if len(dims) == 3 else pg.Grid2d(dims)
    src = None
    if args.workload.startswith("sphere_3d"):
        mask, src_h = W.sphere_plume(dims, spec["sphere_r"], spec["disk_r"])
        grid.set_solid_cells(mask)
        src = pg.Simplex2(grid, torch.from_numpy(src_h).cuda())
        del mask, src_h
    mg = have_mg(pg, grid)
    chosen, plain = solver_cfgs(pg, spec, mg)
    cfg_c, cfg_p = step_cfg(pg, spec, chosen, src), step_cfg(pg, spec, plain, src)
    compare_key = "jacobi_pcg" if spec.get("compare") == "jacobi" else "plain_fp32_pcg"

    def fresh():
        return (pg.Simplex1(grid, torch.from_numpy(vel0).cuda()), pg.Simplex2(grid, torch.from_numpy(rho0).cuda()),
                grid.new_simplex_2())

    # --- chosen form: warm-up, then the timed region (profiled) ------------
    gv, gr, gp = fresh()
    for _ in range(args.warmup):
        pg.step(grid, cfg_c, gv, gr, gp)
    torch.cuda.synchronize()
    # Headline: unprofiled, the solver loops run as device-side CUDA graphs.
    clocks = Clocks(local)
    clocks.start()
    launches0 = lib.pg_kernel_launches()
    ms, stats = timed_steps(torch, pg, dist, grid, cfg_c, gv, gr, gp, args.steps)
    launches = lib.pg_kernel_launches() - launches0
    clk = clocks.stop()
    ms_max = dist.max(ms)
    value = ws * cells * args.steps / (ms_max / 1e3) / 1e6
    its = [s["iterations"] for s in stats]
    # --- e2e through the public API with host buffers, right after the
    # headline (before the profiled pass and the comparison runs) ---------
    e2e = None
    if not args.no_e2e:
        e2e = e2e_pipelined(torch, pg, dist, grid, cfg_c, fresh, vel0, rho0, args.steps, ws, cells)
    # Kernel breakdown: the same number of further steps with a CUDA-event
    # pair around every launch (stream-launched loops, so each kernel is
    # timed on the stream it runs on).  The host-polled CG loop of this mode
    # launches iterations past its stop test, which exit at entry: per-kind
    # figures count only the launches that did work.
    import ctypes as C

    lib.pg_profile_reset()
    lib.pg_profile_enable(1)
    ms_prof, _ = timed_steps(torch, pg, dist, grid, cfg_c, gv, gr, gp, args.steps)
    lib.pg_profile_enable(0)
    kinds = {}
    for k in range(lib.pg_profile_num_kinds()):
        t = C.c_double()
        n = C.c_int64()
        lib.pg_profile_read_active(k, C.byref(t), C.byref(n))
        if n.value:
            kinds[lib.pg_profile_kind_name(k).decode()] = (t.value, n.value)
    # --- one V-cycle and its coarse levels, replayed as CUDA graphs --------
    vcyc = None
    if mg:
        full_ms, coarse_ms = C.c_double(), C.c_double()
        if lib.pg_debug_mg_vcycle_ms(grid.handle, C.c_double(spec["dt"]), 2, 50, C.byref(full_ms),
                                     C.byref(coarse_ms)) == N.PG_OK:
            per_step = float(np.mean(its))  # one V-cycle per CG iteration
            vcyc = {"full_ms": full_ms.value, "coarse_ms": coarse_ms.value, "vcycles_per_step": per_step,
                    "coarse_ms_per_step": coarse_ms.value * per_step,
                    "how": "each captured once into a CUDA graph and replayed 50 times between two events"}
    # --- plain FP32 PCG on the same workload -------------------------------
    plain_out = None
    if not args.no_plain:
        gv2, gr2, gp2 = fresh()
        st_first = pg.step(grid, cfg_p, gv2, gr2, gp2)  # warm-up, from the initial state
        kp = args.plain_steps or max(1, min(args.steps, 3))
        ms_p, st_p = timed_steps(torch, pg, dist, grid, cfg_p, gv2, gr2, gp2, kp)
        ms_p = dist.max(ms_p)
        value_plain = ws * cells * kp / (ms_p / 1e3) / 1e6
        plain_out = {"value": value_plain, "unit": UNIT, "ms_per_step": ms_p / kp,
                     "iterations_per_step": [s["iterations"] for s in st_p], "speedup_of_chosen": value / value_plain,
                     "iterations_first_step": st_first["iterations"],
                     "sums": "FP64-class dot products (the CPU reference sums in f32 and needs more iterations "
                             "from the same state: see cpu_baseline.iterations)"}
        del gv2, gr2, gp2
    # --- precision study (256^3): FP32 storage + refinement and BF16-stored
    # density against an all-FP64 step on the same initial state -----------
    precision, prec_fields = None, None
    if not args.no_precision and spec.get("cpu") and len(dims) == 3:
        precision, prec_fields = precision_study(torch, pg, grid, spec, vel0, rho0, chosen, src)
    # --- roofline of the dominant kernel ------------------------------------
    peak, peak_src = peaks()
    # Dominant kernel among those with a per-cell byte count (fine-grid
    # kernels); coarse multigrid levels are latency-bound and reported in
    # kernels_ms only.
    accounted = [k for k in kinds if k in BYTES_PER_CELL]
    dom = max(accounted, key=lambda k: kinds[k][0]) if accounted else None
    roof = None
    if dom:
        tot, n = kinds[dom]
        bpc = BYTES_PER_CELL[dom][0 if len(dims) == 3 else 1]
        per_launch_ms = tot / n
        achieved = bpc * cells / (per_launch_ms / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_src, "traffic": ncu_traffic(dom, args.workload),
                "algorithmic_bytes_per_launch": bpc * cells, "avg_launch_ms": per_launch_ms, "launches": n,
                "share_of_profiled": tot / ms_prof,
                "dominant_overall": max(kinds, key=lambda k: kinds[k][0])}
    # --- CPU baseline (rank 0, N = 1) ---------------------------------------
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu and spec.get("cpu"):
        from oracle import pyoracle as O

        cpu, oracle64 = cpu_leg(O, dims, spec, vel0, rho0, prec_fields)
        if precision is not None and oracle64 is not None:
            precision["fp64_oracle"] = oracle64
    del prec_fields
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "dims": list(dims), "cells": cells, "dt": spec["dt"],
                       "rel_tol": spec["rel_tol"],
                       "form": ("MG-preconditioned CG" if mg else "Jacobi-PCG") + " in FP64 residual refinement",
                       "parallelism": "replicas x%d" % ws,
                       "l2": "inputs larger than L2 (%.0f MB of fields per step)" % ((vel0.size + rho0.size * 3) * 4 / 1e6)},
            "iterations_per_step": its,
            "true_residual_rel": [s["true_residual_max"] / s["b_max"] if s["b_max"] else 0.0 for s in stats],
            compare_key: plain_out,
            "precision_study": precision,
            "roofline": roof,
            "profiled_ms_per_step": ms_prof / args.steps,
            "kernels_ms": {k: {"ms": v[0], "launches": v[1]} for k, v in sorted(kinds.items(), key=lambda kv: -kv[1][0])},
            "mg_vcycle_graph": vcyc,
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": int(launches),
        }
        print(json.dumps(out), flush=True)
    dist.close()


# ---------------------------------------------------------------------------
# Learned initial guess (128^3 grids with solid boxes)

def unet_forward_flops(dims):
    """Multiply-adds x 2 of the network's convolutions for one forward pass
    on grids of `dims` (layer 0 counted with its 2 real input channels)."""
    from panopaea_gb300 import learned

    v = [int(np.prod([n >> lvl for n in dims])) for lvl in range(3)]
    level = (0, 0, 1, 1, 2, 2, 1, 1, 0, 0)
    fl = 0
    for k in range(10):
        cin = 2 if k == 0 else learned.CIN[k]
        fl += 2 * 27 * cin * learned.COUT[k] * v[level[k]]
    return fl + 2 * 16 * v[0]


def bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def bench_learned(args):
    """128^3 grids, 1-6 solid boxes, filtered-noise divergence.  The network
    is trained on --pairs freshly generated (b, p) pairs (streamed), then
    --held held-out grids are solved to relative 1e-6 (FP64-class
    refinement) by plain CG and by MG-PCG, each from x = 0 and from the
    learned guess, by Jacobi-PCG, and by the flexible CG with the network
    inside as a preconditioner correction.  A step = one pressure solve;
    value = the learned-guess + plain CG form; every form is reported."""
    import ctypes as C

    import torch

    import panopaea_gb300 as pg
    from panopaea_gb300 import learned

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = Dist(ws, rank, local, "nccl")
    lib = pg.load()
    dims = tuple(int(v) for v in args.dims.split(",")) if args.dims else (128, 128, 128)
    cells = int(np.prod(dims))
    g = pg.Grid3d(dims)
    dt = 1.0
    gen_solver = pg.SolverConfig(precond=2 if args.gen == "mg" else 0, rel_stop=True, rel_tol=1e-6,
                                 max_iter=100000, refine=8)
    first = [learned.training_pair(g, 1_000_000 + i, dt, gen_solver)[:2] for i in range(16)]
    scale = learned.estimate_out_scale(first, dt)
    del first
    net = learned.PressureNet(dims, out_scale=scale, seed=1)
    losses, t_gen, t_train = learned.train_streaming(net, g, range(2_000_000 + 10_000 * rank,
                                                                   2_000_000 + 10_000 * rank + args.pairs),
                                                     dt, gen_solver, batch=8, lr=1e-3)
    forms = {
        "plain_cg": (pg.SolverConfig(precond=0, rel_stop=True, rel_tol=1e-6, max_iter=100000, refine=8), None),
        "learned_guess_plain_cg": (pg.SolverConfig(precond=0, rel_stop=True, rel_tol=1e-6, max_iter=100000,
                                                   refine=8), 1),
        "mg_pcg": (pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=20000, refine=4), None),
        "learned_guess_mg_pcg": (pg.SolverConfig(precond=2, rel_stop=True, rel_tol=1e-6, max_iter=20000,
                                                 refine=4), 0),
        # the network inside the CG: flexible CG with z = a net(r) + D^-1 (r - a A net(r))
        "learned_precond_fcg": (pg.SolverConfig(rel_stop=True, rel_tol=1e-6, max_iter=100000, refine=8), "pc"),
        "jacobi_pcg": (pg.SolverConfig(precond=1, rel_stop=True, rel_tol=1e-6, max_iter=100000, refine=8), None),
    }

    def run_form(solver, corr, b):
        if corr is None:
            return pg.solve_pressure(g, x, b, dt, solver)
        if corr == "pc":
            return learned.solve_learned_pcg(net, g, x, b, dt, solver)
        return learned.solve_with_guess(net, g, x, b, dt, solver, corr)
    res = {k: {"ms": [], "iterations": [], "true_residual_rel": []} for k in forms}
    held = [learned.training_pair(g, 9_000_000 + i, dt, solve=False)[::2] for i in range(args.held)]
    stream = torch.cuda.current_stream()
    x = g.new_simplex_2()
    # warm-up (graphs, workspaces)
    g.set_solid_cells(held[0][1])
    for name, (solver, corr) in forms.items():
        for _ in range(2):
            run_form(solver, corr, held[0][0])
    clocks = Clocks(local)
    clocks.start()
    launches0 = lib.pg_kernel_launches()
    dist.barrier()
    setup_ms = []
    for gi, (b, mask) in enumerate(held):
        g.set_solid_cells(mask)
        # untimed: the multigrid hierarchy of the new mask (its build is reported as setup_ms)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        pg.solve_pressure(g, x, b, dt, forms["mg_pcg"][0])
        e1.record(stream)
        torch.cuda.synchronize()
        setup_ms.append(e0.elapsed_time(e1))
        for name, (solver, corr) in forms.items():
            if corr == "pc" and gi >= args.held_fcg:  # a network forward per iteration: a subset of the grids
                continue
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            st = run_form(solver, corr, b)
            e1.record(stream)
            torch.cuda.synchronize()
            res[name]["ms"].append(e0.elapsed_time(e1))
            res[name]["iterations"].append(st["iterations"])
            res[name]["true_residual_rel"].append(st["true_residual_max"] / st["b_max"] if st["b_max"] else 0.0)
    dist.barrier()
    launches = lib.pg_kernel_launches() - launches0
    clk = clocks.stop()
    out_forms = {}
    for name, r in res.items():
        ms = dist.max(float(np.mean(r["ms"])))
        out_forms[name] = {"value": ws * cells / (ms / 1e3) / 1e6, "unit": UNIT, "ms_per_solve": ms,
                           "mean_iterations": float(np.mean(r["iterations"])),
                           "max_true_residual_rel": float(np.max(r["true_residual_rel"])), "grids": len(r["ms"])}
    # e2e: b from pinned host memory, guess + plain CG, x back to the host
    hb = held[0][0].data.cpu().pin_memory()
    hx = torch.empty_like(hb).pin_memory()
    g.set_solid_cells(held[0][1])
    b = g.new_simplex_2()
    solver, corr = forms["learned_guess_plain_cg"]
    dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ne = min(4, args.held)
    e0.record(stream)
    for _ in range(ne):
        b.data.copy_(hb, non_blocking=True)
        learned.solve_with_guess(net, g, x, b, dt, solver, corr)
        hx.copy_(x.data, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_e = dist.max(e0.elapsed_time(e1) / ne)
    # roofline: the network's convolutions in one guess (tensor-core bound)
    lib.pg_profile_reset()
    lib.pg_profile_enable(1)
    net.guess(g, b, dt, x, 0)
    torch.cuda.synchronize()
    lib.pg_profile_enable(0)
    kinds = {}
    for k in range(lib.pg_profile_num_kinds()):
        t, n = C.c_double(), C.c_int64()
        lib.pg_profile_read(k, C.byref(t), C.byref(n))  # every launch of a guess does work
        if n.value:
            kinds[lib.pg_profile_kind_name(k).decode()] = (t.value, n.value)
    peak, src = bf16_peak()
    conv_ms, conv_n = kinds.get("unet_conv", (float("nan"), 0))
    flops = unet_forward_flops(dims)
    achieved = flops / (conv_ms / 1e3) / 1e12
    if rank == 0:
        v = out_forms["learned_guess_plain_cg"]["value"]
        out = {
            "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.held, "warmup": 2,
            "ms_per_step": out_forms["learned_guess_plain_cg"]["ms_per_solve"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 fields, bf16 network", "data": "synthetic",
            "config": {"workload": "learned_3d_128", "dims": list(dims), "cells": cells, "rel_tol": 1e-6,
                       "step": "one pressure solve", "train_pairs": args.pairs, "held_out_grids": args.held,
                       "pair_solver": "MG-PCG in FP64 refinement to 1e-6" if args.gen == "mg"
                       else "plain CG in FP64 refinement to 1e-6",
                       "form": "learned guess + 1 learned correction, then plain CG in FP64 refinement",
                       "parallelism": "replicas x%d" % ws, "l2": "fields of 8 MB per grid: L2-resident"},
            "forms": out_forms,
            "mg_setup_and_first_solve_ms": float(np.mean(setup_ms)),
            "speedup_vs_plain_cg": out_forms["plain_cg"]["ms_per_solve"] / out_forms["learned_guess_plain_cg"]["ms_per_solve"],
            "iterations_saved_vs_plain_cg": 1.0 - out_forms["learned_guess_plain_cg"]["mean_iterations"] /
            out_forms["plain_cg"]["mean_iterations"],
            "training": {"pairs": args.pairs, "loss_first_100": float(np.mean(losses[:100])),
                         "loss_last_100": float(np.mean(losses[-100:])), "seconds_generating": t_gen,
                         "seconds_training": t_train, "ms_per_training_sample": 1e3 * t_train / max(1, args.pairs),
                         "loss": "energy norm"},
            "roofline": {"bound": "tensor", "kernel": "unet_conv", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak, "peak_source": src, "traffic": None,
                         "algorithmic_flops_per_guess": flops, "conv_ms_per_guess": conv_ms, "launches": conv_n},
            "kernels_ms_one_guess": {k: {"ms": t, "launches": n} for k, (t, n) in kinds.items()},
            "cpu_baseline": None,
            "e2e": {"value": ws * cells / (ms_e / 1e3) / 1e6, "unit": UNIT, "h2d_bytes_per_step": 4 * cells,
                    "d2h_bytes_per_step": 4 * cells, "ms_per_step": ms_e},
            "clocks": clk, "gpu_launches": int(launches),
        }
        print(json.dumps(out), flush=True)
    dist.close()


# ---------------------------------------------------------------------------
# Batching: 512 independent 2D grids

def bench_batch(args):
    """512 2D grids, sides from {64, 96, ..., 512}, 0-8 solid circles, a
    Gaussian source at a boundary-adjacent cell, dt 0.5, buoyancy 1; every
    stage one launch over all grids (the batch path), batched MG-PCG to
    relative 1e-6 per grid (batched Jacobi-PCG beside it); tile shape from
    the autotuner.  Grids are partitioned by cost across ranks (no data
    exchange)."""
    import torch

    import panopaea_gb300 as pg
    from panopaea_gb300 import workloads as W

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = Dist(ws, rank, local, "nccl")
    lib = pg.load()
    dims_all, masks_all, srcs_all = W.batch_grids(args.batch_count)
    part = pg.partition_by_cost(dims_all, ws)[rank]
    dims = [dims_all[i] for i in part]
    B = pg.Batch2d(dims)
    B.set_solid_cells([masks_all[i] for i in part])
    t0 = time.time()
    tile = B.autotune()
    t_tune = time.time() - t0
    v, rho, p = B.new_faces(), B.new_cells(), B.new_cells()
    src = torch.from_numpy(B.pack_cells([srcs_all[i] for i in part])).cuda()
    def cfg_for(precond):
        return pg.StepConfig(dt=0.5, buoyancy=1.0, source_enabled=False, walls_after_advect=True,
                             zero_solid_after_project=True,
                             solver=pg.SolverConfig(precond=precond, rel_stop=True, rel_tol=1e-6, max_iter=100000))

    cfg = cfg_for(2)
    for _ in range(args.warmup):
        B.step(cfg, v, rho, p, source_field=src)
    stream = torch.cuda.current_stream()
    clocks = Clocks(local)
    clocks.start()
    launches0 = lib.pg_kernel_launches()
    dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stats = [B.step(cfg, v, rho, p, source_field=src) for _ in range(args.steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    launches = lib.pg_kernel_launches() - launches0
    clk = clocks.stop()
    ms = dist.max(e0.elapsed_time(e1))
    total_cells = sum(h * w for h, w in dims_all)
    value = total_cells * args.steps / (ms / 1e3) / 1e6
    its = [max(s["iterations"] for s in st) for st in stats]
    # profiled pass (CUDA events per launch, host-polled loop)
    import ctypes as C

    lib.pg_profile_reset()
    lib.pg_profile_enable(1)
    torch.cuda.synchronize()
    e0.record(stream)
    B.step(cfg, v, rho, p, source_field=src)
    e1.record(stream)
    torch.cuda.synchronize()
    lib.pg_profile_enable(0)
    ms_prof = e0.elapsed_time(e1)
    kinds = {}
    for k in range(lib.pg_profile_num_kinds()):
        t, n = C.c_double(), C.c_int64()
        lib.pg_profile_read_active(k, C.byref(t), C.byref(n))
        if n.value:
            kinds[lib.pg_profile_kind_name(k).decode()] = (t.value, n.value)
    # comparison: batched Jacobi-PCG on the same state (one step)
    cmp = None
    if not args.no_plain:
        cj = cfg_for(1)
        B.step(cj, v, rho, p, source_field=src)
        torch.cuda.synchronize()
        e0.record(stream)
        st_j = B.step(cj, v, rho, p, source_field=src)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_j = dist.max(e0.elapsed_time(e1))
        cmp = {"value": total_cells / (ms_j / 1e3) / 1e6, "unit": UNIT, "ms_per_step": ms_j,
               "max_iterations": max(s["iterations"] for s in st_j), "speedup_of_chosen": (ms_j / (ms / args.steps))}
    peak, peak_src = peaks()
    roof = None
    if "mg_smooth" in kinds:
        tot, n = kinds["mg_smooth"]
        achieved = BYTES_PER_CELL["mg_smooth"][1] * sum(h * w for h, w in dims) / (tot / n / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": "mg_smooth", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_src, "traffic": None,
                "algorithmic_bytes_per_launch": BYTES_PER_CELL["mg_smooth"][1] * sum(h * w for h, w in dims),
                "avg_launch_ms": tot / n, "launches": n, "share_of_profiled": tot / ms_prof}
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch_512", "grids": len(dims_all), "cells": total_cells, "dt": 0.5,
                       "rel_tol": 1e-6, "form": "batched MG-PCG (one V-cycle per iteration over every grid's "
                                                "hierarchy), one launch per stage over all grids, device-side "
                                                "graph loop",
                       "tile": list(tile), "autotune_s": t_tune, "parallelism": "cost-partitioned x%d" % ws,
                       "l2": "fields of %.0f MB per step" % (total_cells * 4 * 6 / 1e6)},
            "max_iterations_per_step": its,
            "statuses": sorted(set(s["status"] for st in stats for s in st)),
            "batched_jacobi_pcg": cmp,
            "profiled_ms_per_step": ms_prof,
            "kernels_ms": {k: {"ms": t, "launches": n} for k, (t, n) in sorted(kinds.items(), key=lambda kv: -kv[1][0])},
            "cpu_baseline": None, "roofline": roof, "e2e": None, "clocks": clk, "gpu_launches": int(launches),
        }
        print(json.dumps(out), flush=True)
    dist.close()


def main():
    args = parse_args()
    from panopaea_gb300 import workloads as W

    if args.impl != "reference" and args.workload == "learned_3d_128":
        return bench_learned(args)
    if args.impl != "reference" and args.workload == "batch_512":
        return bench_batch(args)
    spec = W.WORKLOADS[args.workload]
    dims = tuple(int(v) for v in args.dims.split(",")) if args.dims else tuple(spec["dims"])
    if args.impl == "reference":
        reference_arm(args, spec, dims)
    else:
        ours(args, spec, dims)


if __name__ == "__main__":
    main()
