// The reference's own tests and example, written against the C++ host API
// (include/panopaea.hpp) the way the Rust originals are written against
// panopaea's API:
//   grid_2d_divergence   panopaea/src/dec/grid.rs:428-482
//   grid_2d_laplacian    panopaea/src/dec/grid.rs:484-515
//   the PCG of examples/dec_fluid.rs:87-121 on the example's grid
//   the step loop of examples/dec_fluid.rs:46-141 (a few steps)
// plus the error behaviour (the reference panics; this API throws).
// Exit status 0 iff every check passes.
#include <cmath>
#include <cstdio>
#include <vector>

#include "grid_rs_vectors.h"
#include "panopaea.hpp"

using namespace panopaea;

static int failures = 0;
#define CHECK(cond, ...)                          \
    do {                                          \
        if (!(cond)) {                            \
            std::printf("FAIL %s:%d: ", __FILE__, __LINE__); \
            std::printf(__VA_ARGS__);             \
            std::printf("\n");                    \
            ++failures;                           \
        }                                         \
    } while (0)

// grid.rs:428-482
static void grid_2d_divergence() {
    Grid2d grid({5, 5});
    auto velocities = grid.new_simplex_1<float>();
    std::vector<float> v(GOLDEN_DIV_VELOCITIES_Y, GOLDEN_DIV_VELOCITIES_Y + 30);
    v.insert(v.end(), GOLDEN_DIV_VELOCITIES_X, GOLDEN_DIV_VELOCITIES_X + 30);
    velocities.upload(v);
    auto velocities_primal = grid.new_simplex_1<float>();
    grid.hodge_1_dual(velocities_primal, velocities);
    auto div = grid.new_simplex_2<float>();
    grid.derivative_1_primal(div, velocities_primal);
    const auto d = div.download();
    for (int i = 0; i < 25; ++i)
        CHECK(std::fabs(d[i] - GOLDEN_DIV_REF[i]) < GOLDEN_DIV_EPS, "div[%d] = %g, want %g", i, d[i], GOLDEN_DIV_REF[i]);
}

// grid.rs:484-515
static void grid_2d_laplacian() {
    Grid2d grid({3, 3});
    auto faces_primal = grid.new_simplex_2<double>();
    faces_primal.upload(std::vector<double>(GOLDEN_LAP_FACES_PRIMAL, GOLDEN_LAP_FACES_PRIMAL + 9));
    auto faces_dual = grid.new_simplex_2<double>();
    grid.hodge_2_primal(faces_dual, faces_primal);
    auto edges_dual = grid.new_simplex_1<double>();
    grid.derivative_0_dual(edges_dual, faces_dual);
    auto edges_primal = grid.new_simplex_1<double>();
    grid.hodge_1_dual(edges_primal, edges_dual);
    auto laplacian = grid.new_simplex_2<double>();
    grid.derivative_1_primal(laplacian, edges_primal);
    const auto l = laplacian.download();
    for (int i = 0; i < 9; ++i)
        CHECK(std::fabs(l[i] - GOLDEN_LAP_REF[i]) < GOLDEN_LAP_EPS, "lap[%d] = %g, want %g", i, l[i], GOLDEN_LAP_REF[i]);
    // the fused closure is the same operator at dt = 1
    auto fused = grid.new_simplex_2<double>();
    grid.laplacian(fused, faces_primal, 1.0);
    const auto f = fused.download();
    for (int i = 0; i < 9; ++i) CHECK(f[i] == l[i], "fused lap[%d] = %g vs %g", i, f[i], l[i]);
}

// examples/dec_fluid.rs:87-121: pcg(&(), pressure, divergence, 100, threshold, ...)
static void pcg_on_the_example_grid() {
    const std::size_t h = 128, w = 128;
    Grid2d grid({h, w});
    std::vector<double> vel((h + 1) * w + h * (w + 1));
    unsigned s = 12345u;
    for (auto& x : vel) {
        s = s * 1664525u + 1013904223u;
        x = ((s >> 8) & 0xffff) / 32768.0 - 1.0;
    }
    auto velocities = grid.new_simplex_1<double>();
    velocities.upload(vel);
    grid.walls(velocities);  // closed domain, as the example's wall step leaves it
    auto b = grid.new_simplex_2<double>();
    grid.divergence_rhs(b, velocities);
    auto pressure = grid.new_simplex_2<double>();
    auto residual = grid.new_simplex_2<double>();
    auto auxiliary = grid.new_simplex_2<double>();
    auto search = grid.new_simplex_2<double>();
    const double dt = 0.05, threshold = 1e-6;
    const auto st = precond_conjugate_gradient(Preconditioner::Identity, pressure, b, 5000, threshold, residual, auxiliary,
                                               search, LaplacianOperator{grid, dt});
    CHECK(st.status == PG_OK, "pcg status %d", st.status);
    CHECK(st.residual_max < threshold, "pcg residual %g", st.residual_max);
    // the true residual agrees with the recursive one
    auto ax = grid.new_simplex_2<double>();
    grid.laplacian(ax, pressure, dt);
    const auto bb = b.download(), a = ax.download();
    double m = 0.0;
    for (std::size_t i = 0; i < bb.size(); ++i) m = std::fmax(m, std::fabs(bb[i] - a[i]));
    CHECK(m < 10 * threshold, "true residual %g", m);
    // max_iterations bounds the operator applications, as pcg.rs:48
    const auto st2 = precond_conjugate_gradient(Preconditioner::Identity, pressure, b, 3, 1e-12, residual, auxiliary,
                                                search, LaplacianOperator{grid, dt});
    CHECK(st2.iterations == 3 && st2.status == PG_NOT_CONVERGED, "bounded pcg: %lld its, status %d",
          (long long)st2.iterations, st2.status);
}

// examples/dec_fluid.rs:46-141 with its own constants
static void the_example_step_loop() {
    Grid2d grid({128, 128});
    std::vector<uint8_t> solid(grid.num_elem_1(), 0);
    const std::size_t w = 128, h = 128;
    for (std::size_t y = 70; y < 80; ++y)
        for (std::size_t x = 50; x < 70; ++x) {  // dec_fluid.rs:71-78: the same box in both face arrays
            solid[y * w + x] = 1;
            solid[(h + 1) * w + y * (w + 1) + x] = 1;
        }
    grid.set_solid_faces(solid);
    auto vel = grid.new_simplex_1<double>();
    auto density = grid.new_simplex_2<double>();
    auto pressure = grid.new_simplex_2<double>();
    const auto prm = reference_step_params();
    long long its = 0;
    for (int i = 0; i < 5; ++i) its += step(grid, prm, vel, density, pressure).iterations;
    const auto d = density.download(), v = vel.download();
    bool finite = true;
    double dmax = 0.0;
    for (double x : d) {
        finite = finite && std::isfinite(x);
        dmax = std::fmax(dmax, x);
    }
    for (double x : v) finite = finite && std::isfinite(x);
    CHECK(finite, "non-finite field after the example's steps");
    CHECK(std::fabs(dmax - 1.0) < 1e-9, "density max %g (the inflow sets 1.0)", dmax);
    CHECK(its > 0, "no CG iterations");
}

static void errors_are_exceptions() {
    bool thrown = false;
    try {
        Grid2d grid({1, 5});
        auto a = grid.new_simplex_2<float>(), b = grid.new_simplex_2<float>();
        auto v = grid.new_simplex_1<float>();
        advect(a, b, 0.1, v);  // the reference indexes the +1 neighbour: needs sides >= 2
    } catch (const Error& e) {
        thrown = e.status() == PG_BAD_ARG;
    }
    CHECK(thrown, "advect on a 1-wide grid must throw PG_BAD_ARG");
    thrown = false;
    try {
        Grid2d grid({4, 4});
        auto f = grid.new_simplex_2<float>();
        f.upload(std::vector<float>(7));  // wrong length
    } catch (const Error& e) {
        thrown = e.status() == PG_BAD_ARG;
    }
    CHECK(thrown, "upload of the wrong length must throw");
}

int main() {
    try {
        grid_2d_divergence();
        grid_2d_laplacian();
        pcg_on_the_example_grid();
        the_example_step_loop();
        errors_are_exceptions();
    } catch (const std::exception& e) {
        std::printf("FAIL uncaught: %s\n", e.what());
        return 2;
    }
    if (failures) {
        std::printf("%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("ALL OK\n");
    return 0;
}
