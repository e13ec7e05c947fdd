"""The C ABI library builds, loads and exports every symbol the header
declares; the Python structs match the header's layout.  No compute calls
(CPU only)."""

import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "panopaea_gpu.h")


def header_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(pg_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from panopaea_gb300 import _native

    _native.load()
    return _native


def test_header_declares_the_reference_surface():
    fns = header_functions()
    for name in ["pg_grid_create_2d", "pg_grid_create_3d", "pg_field_alloc", "pg_hodge_1_dual_f32",
                 "pg_hodge_2_primal_f32", "pg_derivative_0_dual_f32", "pg_derivative_1_primal_f32",
                 "pg_laplacian_f32", "pg_divergence_rhs_f32", "pg_advect_f32", "pg_advect_mac_f32",
                 "pg_project_f32", "pg_pcg_f32", "pg_pcg_f64", "pg_step_f32", "pg_step_f64",
                 "pg_solve_pressure_f32"]:
        assert name in fns


def test_library_exports_every_declared_symbol(lib):
    raw = C.CDLL(lib.lib_path())
    missing = [f for f in header_functions() if not hasattr(raw, f)]
    assert not missing, missing
    # and the Python binding covers every declared entry point
    assert set(header_functions()) <= set(lib.exported_symbols())


def test_library_has_sm103a_code_only():
    """The shared library carries a cubin for sm_103a (checked by the
    build flags: one -gencode, no PTX for other targets)."""
    from panopaea_gb300 import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def _c_layout():
    prog = r"""
#include <stddef.h>
#include <stdio.h>
#include "panopaea_gpu.h"
#define P(T, F) printf(#T "." #F " %zu\n", offsetof(T, F));
int main(void) {
  printf("pg_pcg_stats %zu\n", sizeof(pg_pcg_stats));
  printf("pg_solver_params %zu\n", sizeof(pg_solver_params));
  printf("pg_step_params %zu\n", sizeof(pg_step_params));
  P(pg_pcg_stats, status) P(pg_pcg_stats, true_residual_max)
  P(pg_solver_params, max_iter) P(pg_solver_params, inner_rel_tol) P(pg_solver_params, mg_smooth)
  P(pg_step_params, source_lo) P(pg_step_params, source_field) P(pg_step_params, solver)
  P(pg_step_params, zero_solid_after_project)
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(c, "w").write(prog)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    return {k: int(v) for k, v in (ln.split() for ln in out.strip().splitlines())}


def test_ctypes_structs_match_header(lib):
    lay = _c_layout()
    N = lib
    assert C.sizeof(N.PcgStats) == lay["pg_pcg_stats"]
    assert C.sizeof(N.SolverParams) == lay["pg_solver_params"]
    assert C.sizeof(N.StepParams) == lay["pg_step_params"]
    assert N.PcgStats.status.offset == lay["pg_pcg_stats.status"]
    assert N.PcgStats.true_residual_max.offset == lay["pg_pcg_stats.true_residual_max"]
    assert N.SolverParams.max_iter.offset == lay["pg_solver_params.max_iter"]
    assert N.SolverParams.inner_rel_tol.offset == lay["pg_solver_params.inner_rel_tol"]
    assert N.SolverParams.mg_smooth.offset == lay["pg_solver_params.mg_smooth"]
    assert N.StepParams.source_lo.offset == lay["pg_step_params.source_lo"]
    assert N.StepParams.source_field.offset == lay["pg_step_params.source_field"]
    assert N.StepParams.solver.offset == lay["pg_step_params.solver"]
    assert N.StepParams.zero_solid_after_project.offset == lay["pg_step_params.zero_solid_after_project"]


def test_status_strings(lib):
    L = lib.load()
    assert L.pg_status_string(0) == b"PG_OK"
    assert L.pg_status_string(4) == b"PG_BAD_ARG"
    assert L.pg_version() >= 1


def test_timeout_status_is_distinct(lib):
    """PG_TIMEOUT (a bounded device wait gave up; the solve's results are
    not to be trusted) has its own code, string and Python error, distinct
    from non-convergence, NaN and breakdown -- checked on the host, no GPU."""
    L = lib.load()
    codes = [lib.PG_OK, lib.PG_NOT_CONVERGED, lib.PG_NAN_DETECTED, lib.PG_TIMEOUT, lib.PG_BAD_ARG,
             lib.PG_CUDA_ERROR, lib.PG_NO_DEVICE, lib.PG_OUT_OF_MEMORY, lib.PG_BREAKDOWN]
    assert len(set(codes)) == len(codes)
    strings = [L.pg_status_string(c) for c in codes]
    assert len(set(strings)) == len(strings) and L.pg_status_string(lib.PG_TIMEOUT) == b"PG_TIMEOUT"
    with pytest.raises(lib.PgError) as ei:
        lib.check(lib.PG_TIMEOUT, allow=(lib.PG_OK, lib.PG_NOT_CONVERGED))
    assert ei.value.status == lib.PG_TIMEOUT and str(ei.value).startswith("PG_TIMEOUT")
    assert L.pg_debug_stage_wait_polls_default() > 0


def test_no_device_fails_loudly(lib):
    """Without a GPU the library refuses to run rather than computing on the host."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = lib.load()
    h = C.c_void_p()
    rc = L.pg_grid_create_2d(8, 8, C.byref(h))
    assert rc == lib.PG_NO_DEVICE and not h.value
    with pytest.raises(lib.PgError):
        lib.check(rc)


def test_bad_args_are_rejected(lib):
    L = lib.load()
    assert L.pg_grid_create_2d(0, 8, C.byref(C.c_void_p())) == lib.PG_BAD_ARG
    assert L.pg_grid_create_2d(8, 8, None) == lib.PG_BAD_ARG
    assert L.pg_laplacian_f32(None, None, None, C.c_double(1.0)) == lib.PG_BAD_ARG
    assert L.pg_pcg_f32(None, 0, None, None, 10, C.c_double(0.1), None, None, None, C.c_double(1.0), None) \
        == lib.PG_BAD_ARG


def test_coarsest_pseudo_inverse(lib):
    """The multigrid coarsest solve's pseudo-inverse (host code, no GPU): on
    a 4^3 cell Laplacian with random face weights, a solid cell and two
    disconnected components it matches numpy's pinv to 1e-10 relative."""
    import numpy as np

    L = lib.load()
    rng = np.random.default_rng(3)
    d = h = w = 4
    n = d * h * w
    a = np.zeros((n, n))

    def link(c, k, wt):
        a[c, c] += wt
        a[k, k] += wt
        a[c, k] -= wt
        a[k, c] -= wt

    for z in range(d):
        for y in range(h):
            for x in range(w):
                c = (z * h + y) * w + x
                for ok, k in ((x > 0, c - 1), (y > 0, c - w), (z > 0, c - h * w)):
                    if not ok:
                        continue
                    wt = float(rng.choice([0.0, 0.5, 1.0, 1.5, 2.0]))
                    if 21 in (c, k) or (z == 2) != (k // (h * w) == 2):  # a solid cell; z = 2 cut off
                        wt = 0.0
                    link(c, k, wt)
    m = np.ascontiguousarray(a.copy())
    assert L.pg_debug_sym_pinv(n, m.ctypes.data) == 0
    want = np.linalg.pinv(a, rcond=1e-10, hermitian=True)
    assert np.abs(m - want).max() <= 1e-10 * np.abs(want).max()
    with pytest.raises(Exception):
        lib.check(L.pg_debug_sym_pinv(0, m.ctypes.data))
