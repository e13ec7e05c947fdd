// pg_solve.cuh -- solver workspace and the multigrid-preconditioned CG.
#pragma once
#include "pg_cg.cuh"

namespace pg {

struct MgHierarchy;

// Per-grid buffers of the solver and the step, grown on demand.
struct Extras {
    enum Slot { kR, kAp, kP0, kP1, kX64, kD, kRin, kTemp, kVelTemp, kB, kZ, kAdv1, kAdv2, kSlots };
    void* buf_[kSlots] = {};
    size_t bytes_[kSlots] = {};
    void* small = nullptr;  // 256 B of device scalars
    MgHierarchy* mg = nullptr;
    int buffer(int slot, size_t bytes, void** out);
    ~Extras();
};

Extras* extras_of(pg_grid* g);
int ensure_small(pg_grid* g);
void release_mg(Extras* ex);

// CG preconditioned by one multigrid V-cycle per iteration.
template <class T>
int solve_mgpcg(pg_grid* g, const pg_solver_params* prm, const CgConfig& cfg, CgBuffers<T> buf, pg_pcg_stats* st);

template <class T>
int solve_pressure(pg_grid* g, const pg_solver_params* prm, T* x, const T* b, double dt, pg_pcg_stats* st);

// The float pressure solve (plain or in FP64-class refinement, as prm says)
// with z = M(r) from an outer preconditioner hook whose apply() also folds
// z.r and beta into the CG state (a flexible CG when M is not linear);
// prm->precond is not used.
int solve_pressure_hooked(pg_grid* g, const pg_solver_params* prm, float* x, const float* b, double dt, ZHook* hook,
                          pg_pcg_stats* st);

}  // namespace pg
