// pg_cg.cuh -- the CG engine shared by pg_pcg_* and the pressure solver.
#pragma once
#include "pg_internal.cuh"

namespace pg {

// Buffers of one CG run.  p[0], p[1] ping-pong: the SpMV of iteration k
// reads p[k & 1] and writes p[(k + 1) & 1], so the search direction of the
// latest iteration is p[iter & 1].
template <class T> struct CgBuffers {
    T* x;
    const T* b;
    T* r;
    T* ap;
    T* p[2];
};

struct CgConfig {
    int precond;        // PG_PRECOND_NONE or PG_PRECOND_JACOBI
    i64 max_iter;
    double threshold;   // absolute: stop when ||r||inf < threshold
    double rel_tol;     // > 0: threshold = rel_tol * ||b||inf (set on device)
    double dt;
    int check_every;    // 0 = auto
    int zero_x;         // 1: x = 0 first (pcg.rs:32)
};

// Runs CG on the grid's stream and synchronises at the end.  Returns a
// pg_status for launch/CUDA failures; the solve outcome is in *stats.
template <class T> int run_cg(pg_grid* g, const CgConfig& cfg, CgBuffers<T> buf, pg_pcg_stats* stats);

}  // namespace pg
