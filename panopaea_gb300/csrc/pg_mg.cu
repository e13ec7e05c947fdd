// pg_mg.cu -- geometric multigrid preconditioner (placeholder until the
// V-cycle lands).
#include "pg_solve.cuh"

namespace pg {

void release_mg(Extras* ex) { ex->mg = nullptr; }

template <class T>
int solve_mgpcg(pg_grid*, const pg_solver_params*, const CgConfig&, CgBuffers<T>, pg_pcg_stats*) {
    return bad_arg("PG_PRECOND_MG is not available in this build");
}

template int solve_mgpcg<float>(pg_grid*, const pg_solver_params*, const CgConfig&, CgBuffers<float>, pg_pcg_stats*);
template int solve_mgpcg<double>(pg_grid*, const pg_solver_params*, const CgConfig&, CgBuffers<double>,
                                 pg_pcg_stats*);

}  // namespace pg
