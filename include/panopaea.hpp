// panopaea.hpp -- C++ host API of libpanopaea_gpu, mirroring the names,
// argument order and meaning of the reference's Rust API for the grid-fluid
// path (msiglreith/panopaea):
//
//   Grid2d::new / dim                         domain/grid.rs:2-15
//   Grid3d (declared only in the reference)   domain/grid.rs:17-20
//   Simplex1 / Simplex2, split / split_mut    dec/grid.rs:36-100
//   Manifold2d: new_simplex_1/2, num_elem_1/2,
//     hodge_1_dual, hodge_1_primal, hodge_2_primal,
//     derivative_0_dual, derivative_1_primal  dec/manifold.rs:29-83, dec/grid.rs:202-356
//   pcg::Preconditioner, precond_conjugate_gradient   pcg.rs:4-82
//   advect, advect_mac                         examples/dec_fluid.rs:173-291
//
// Fields live in device memory (same flat layouts as the reference); the
// host reads and writes them with upload / download.  Where the reference
// panics (shape mismatches, debug_asserts) this API throws panopaea::Error
// carrying the library's status code and message.  Header-only, C++17,
// over the C ABI of panopaea_gpu.h (link with -lpanopaea_gpu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "panopaea_gpu.h"

namespace panopaea {

class Error : public std::runtime_error {
  public:
    Error(int status, const std::string& what)
        : std::runtime_error(std::string(pg_status_string(status)) + ": " + what), status_(status) {}
    int status() const { return status_; }

  private:
    int status_;
};

namespace detail {
inline int check(int status, const char* what, bool allow_not_converged = false) {
    if (status == PG_OK || (allow_not_converged && status == PG_NOT_CONVERGED)) return status;
    const char* msg = pg_last_error();
    throw Error(status, std::string(what) + (msg && *msg ? std::string(" (") + msg + ")" : std::string()));
}
template <class T> struct Tag;
template <> struct Tag<float> {
    static constexpr int dtype = PG_F32;
};
template <> struct Tag<double> {
    static constexpr int dtype = PG_F64;
};
}  // namespace detail

// A device field of one grid: `kind` PG_FACES (Simplex1) or PG_CELLS (Simplex2).
template <class T, int Kind> class Field {
  public:
    Field() = default;
    Field(const pg_grid* g, std::size_t n) : grid_(g), n_(n) {
        void* p = nullptr;
        detail::check(pg_field_alloc(g, Kind, detail::Tag<T>::dtype, &p), "new_simplex");
        ptr_ = static_cast<T*>(p);
    }
    Field(const Field&) = delete;
    Field& operator=(const Field&) = delete;
    Field(Field&& o) noexcept { *this = std::move(o); }
    Field& operator=(Field&& o) noexcept {
        if (this != &o) {
            release();
            grid_ = o.grid_;
            n_ = o.n_;
            ptr_ = o.ptr_;
            o.ptr_ = nullptr;
        }
        return *this;
    }
    ~Field() { release(); }

    T* data() { return ptr_; }
    const T* data() const { return ptr_; }
    std::size_t len() const { return n_; }
    const pg_grid* grid() const { return grid_; }

    void upload(const std::vector<T>& host) {
        if (host.size() != n_) throw Error(PG_BAD_ARG, "upload: size mismatch");
        detail::check(pg_copy_h2d(grid_, ptr_, host.data(), sizeof(T) * n_), "upload");
        detail::check(pg_grid_synchronize(const_cast<pg_grid*>(grid_)), "upload");
    }
    std::vector<T> download() const {
        std::vector<T> host(n_);
        detail::check(pg_copy_d2h(grid_, host.data(), ptr_, sizeof(T) * n_), "download");
        detail::check(pg_grid_synchronize(const_cast<pg_grid*>(grid_)), "download");
        return host;
    }

  private:
    void release() {
        if (ptr_) pg_field_free(ptr_);
        ptr_ = nullptr;
    }
    const pg_grid* grid_ = nullptr;
    std::size_t n_ = 0;
    T* ptr_ = nullptr;
};

// dec/grid.rs:36-73 (faces: [vy (h+1)w | vx h(w+1)]; 3D prepends vz)
template <class T> using Simplex1 = Field<T, PG_FACES>;
// dec/grid.rs:76-100 (cells, row-major)
template <class T> using Simplex2 = Field<T, PG_CELLS>;

// One part of a split Simplex1: a row-major (rows, cols) device view.
template <class T> struct FaceView {
    T* ptr;
    std::size_t rows, cols;
};

// Shared grid behaviour (Manifold2d, dec/manifold.rs:29-83).
class GridBase {
  public:
    GridBase(const GridBase&) = delete;
    GridBase& operator=(const GridBase&) = delete;
    ~GridBase() {
        if (g_) pg_grid_destroy(g_);
    }
    pg_grid* raw() const { return g_; }

    std::size_t num_elem_1() const { return (std::size_t)pg_grid_num_elem_1(g_); }
    std::size_t num_elem_2() const { return (std::size_t)pg_grid_num_elem_2(g_); }
    template <class T = double> Simplex1<T> new_simplex_1() const { return Simplex1<T>(g_, num_elem_1()); }
    template <class T = double> Simplex2<T> new_simplex_2() const { return Simplex2<T>(g_, num_elem_2()); }

    // examples/dec_fluid.rs:71-78 as data: 1 = solid face (face layout); empty clears
    void set_solid_faces(const std::vector<uint8_t>& face_solid) {
        if (!face_solid.empty() && face_solid.size() != num_elem_1()) throw Error(PG_BAD_ARG, "set_solid_faces");
        detail::check(pg_grid_set_solid_faces(g_, face_solid.empty() ? nullptr : face_solid.data()), "set_solid_faces");
    }
    // extension: a face is solid iff an adjacent cell is
    void set_solid_cells(const std::vector<uint8_t>& cell_solid) {
        if (!cell_solid.empty() && cell_solid.size() != num_elem_2()) throw Error(PG_BAD_ARG, "set_solid_cells");
        detail::check(pg_grid_set_solid_cells(g_, cell_solid.empty() ? nullptr : cell_solid.data()), "set_solid_cells");
    }
    void set_stream(void* cuda_stream) { detail::check(pg_grid_set_stream(g_, cuda_stream), "set_stream"); }
    void synchronize() const { detail::check(pg_grid_synchronize(g_), "synchronize"); }

    // grid.rs:223-238: primal.vy = -dual.vy, primal.vx = dual.vx
    void hodge_1_dual(Simplex1<float>& primal, const Simplex1<float>& dual) const {
        detail::check(pg_hodge_1_dual_f32(g_, primal.data(), dual.data()), "hodge_1_dual");
    }
    void hodge_1_dual(Simplex1<double>& primal, const Simplex1<double>& dual) const {
        detail::check(pg_hodge_1_dual_f64(g_, primal.data(), dual.data()), "hodge_1_dual");
    }
    // grid.rs:206-221: dual.vy = primal.vy, dual.vx = -primal.vx
    void hodge_1_primal(Simplex1<float>& dual, const Simplex1<float>& primal) const {
        detail::check(pg_hodge_1_primal_f32(g_, dual.data(), primal.data()), "hodge_1_primal");
    }
    void hodge_1_primal(Simplex1<double>& dual, const Simplex1<double>& primal) const {
        detail::check(pg_hodge_1_primal_f64(g_, dual.data(), primal.data()), "hodge_1_primal");
    }
    // grid.rs:253-255: copy
    void hodge_2_primal(Simplex2<float>& dual, const Simplex2<float>& primal) const {
        detail::check(pg_hodge_2_primal_f32(g_, dual.data(), primal.data()), "hodge_2_primal");
    }
    void hodge_2_primal(Simplex2<double>& dual, const Simplex2<double>& primal) const {
        detail::check(pg_hodge_2_primal_f64(g_, dual.data(), primal.data()), "hodge_2_primal");
    }
    // grid.rs:295-305: face = -bottom + top - left + right
    void derivative_1_primal(Simplex2<float>& faces, const Simplex1<float>& edges) const {
        detail::check(pg_derivative_1_primal_f32(g_, faces.data(), edges.data()), "derivative_1_primal");
    }
    void derivative_1_primal(Simplex2<double>& faces, const Simplex1<double>& edges) const {
        detail::check(pg_derivative_1_primal_f64(g_, faces.data(), edges.data()), "derivative_1_primal");
    }
    // grid.rs:318-334: interior faces only, boundary faces keep their value
    void derivative_0_dual(Simplex1<float>& edges, const Simplex2<float>& faces) const {
        detail::check(pg_derivative_0_dual_f32(g_, edges.data(), faces.data()), "derivative_0_dual");
    }
    void derivative_0_dual(Simplex1<double>& edges, const Simplex2<double>& faces) const {
        detail::check(pg_derivative_0_dual_f64(g_, edges.data(), faces.data()), "derivative_0_dual");
    }

    // The operator closure of examples/dec_fluid.rs:100-119, fused.
    void laplacian(Simplex2<float>& out, const Simplex2<float>& p, double timestep) const {
        detail::check(pg_laplacian_f32(g_, out.data(), p.data(), timestep), "laplacian");
    }
    void laplacian(Simplex2<double>& out, const Simplex2<double>& p, double timestep) const {
        detail::check(pg_laplacian_f64(g_, out.data(), p.data(), timestep), "laplacian");
    }
    // examples/dec_fluid.rs:68-83: b = -div(M u)
    void divergence_rhs(Simplex2<float>& b, const Simplex1<float>& vel) const {
        detail::check(pg_divergence_rhs_f32(g_, b.data(), vel.data()), "divergence_rhs");
    }
    void divergence_rhs(Simplex2<double>& b, const Simplex1<double>& vel) const {
        detail::check(pg_divergence_rhs_f64(g_, b.data(), vel.data()), "divergence_rhs");
    }
    // examples/dec_fluid.rs:128-141: zero the boundary faces
    void walls(Simplex1<float>& vel) const { detail::check(pg_walls_f32(g_, vel.data()), "walls"); }
    void walls(Simplex1<double>& vel) const { detail::check(pg_walls_f64(g_, vel.data()), "walls"); }
    // examples/dec_fluid.rs:123-141: vel += dt d0dual(p), then walls
    void project(Simplex1<float>& vel, const Simplex2<float>& p, double dt, bool zero_solid = false) const {
        detail::check(pg_project_f32(g_, vel.data(), p.data(), dt, zero_solid), "project");
    }
    void project(Simplex1<double>& vel, const Simplex2<double>& p, double dt, bool zero_solid = false) const {
        detail::check(pg_project_f64(g_, vel.data(), p.data(), dt, zero_solid), "project");
    }

  protected:
    GridBase() = default;
    pg_grid* g_ = nullptr;
};

// domain/grid.rs:2-15: dim = (h, w) = (y, x)
class Grid2d : public GridBase {
  public:
    explicit Grid2d(std::pair<std::size_t, std::size_t> dim) : dim_(dim) {
        detail::check(pg_grid_create_2d((int64_t)dim.first, (int64_t)dim.second, &g_), "Grid2d::new");
    }
    std::pair<std::size_t, std::size_t> dim() const { return dim_; }

    // dec/grid.rs:47-53: (vertical (h+1) x w, horizontal h x (w+1))
    template <class T> std::pair<FaceView<T>, FaceView<T>> split(Simplex1<T>& f) const {
        const std::size_t h = dim_.first, w = dim_.second;
        return {FaceView<T>{f.data(), h + 1, w}, FaceView<T>{f.data() + (h + 1) * w, h, w + 1}};
    }

  private:
    std::pair<std::size_t, std::size_t> dim_;
};

// domain/grid.rs:17-20 declares Grid3d; here it is defined: dim = (d, h, w)
class Grid3d : public GridBase {
  public:
    struct Dim {
        std::size_t d, h, w;
    };
    explicit Grid3d(Dim dim) : dim_(dim) {
        detail::check(pg_grid_create_3d((int64_t)dim.d, (int64_t)dim.h, (int64_t)dim.w, &g_), "Grid3d::new");
    }
    Dim dim() const { return dim_; }

  private:
    Dim dim_;
};

// pcg.rs:4-12: the preconditioner is chosen, not a closure across the ABI.
enum class Preconditioner { Identity = PG_PRECOND_NONE, Jacobi = PG_PRECOND_JACOBI, Multigrid = PG_PRECOND_MG };

// The operator argument `a` of pcg.rs:14-28 for examples/dec_fluid.rs:100-119.
struct LaplacianOperator {
    const GridBase& grid;
    double timestep;
};

using PcgStats = pg_pcg_stats;

// pcg.rs:14-82.  Returns the statistics (the reference returns ()); a run
// stopped by max_iterations is not an error, as in the reference.
inline PcgStats precond_conjugate_gradient(Preconditioner precond, Simplex2<float>& x, const Simplex2<float>& b,
                                           std::size_t max_iterations, float threshold, Simplex2<float>& residual,
                                           Simplex2<float>& auxiliary, Simplex2<float>& search,
                                           const LaplacianOperator& a) {
    PcgStats st{};
    detail::check(pg_pcg_f32(a.grid.raw(), (int)precond, x.data(), b.data(), (int64_t)max_iterations, threshold,
                             residual.data(), auxiliary.data(), search.data(), a.timestep, &st),
                  "precond_conjugate_gradient", true);
    return st;
}
inline PcgStats precond_conjugate_gradient(Preconditioner precond, Simplex2<double>& x, const Simplex2<double>& b,
                                           std::size_t max_iterations, double threshold, Simplex2<double>& residual,
                                           Simplex2<double>& auxiliary, Simplex2<double>& search,
                                           const LaplacianOperator& a) {
    PcgStats st{};
    detail::check(pg_pcg_f64(a.grid.raw(), (int)precond, x.data(), b.data(), (int64_t)max_iterations, threshold,
                             residual.data(), auxiliary.data(), search.data(), a.timestep, &st),
                  "precond_conjugate_gradient", true);
    return st;
}

// examples/dec_fluid.rs:173-211, the reference's signature (the grid is the
// fields' owner) and a form naming the grid
template <class T> inline void advect(Simplex2<T>& dst, const Simplex2<T>& src, double dt, const Simplex1<T>& vel);
template <class T> inline void advect_mac(Simplex1<T>& dst, const Simplex1<T>& src, double dt, const Simplex1<T>& vel);
inline void advect(const GridBase& g, Simplex2<float>& dst, const Simplex2<float>& src, double dt,
                   const Simplex1<float>& vel) {
    detail::check(pg_advect_f32(g.raw(), dst.data(), src.data(), dt, vel.data()), "advect");
}
inline void advect(const GridBase& g, Simplex2<double>& dst, const Simplex2<double>& src, double dt,
                   const Simplex1<double>& vel) {
    detail::check(pg_advect_f64(g.raw(), dst.data(), src.data(), dt, vel.data()), "advect");
}
// examples/dec_fluid.rs:213-291
inline void advect_mac(const GridBase& g, Simplex1<float>& dst, const Simplex1<float>& src, double dt,
                       const Simplex1<float>& vel) {
    detail::check(pg_advect_mac_f32(g.raw(), dst.data(), src.data(), dt, vel.data()), "advect_mac");
}
inline void advect_mac(const GridBase& g, Simplex1<double>& dst, const Simplex1<double>& src, double dt,
                       const Simplex1<double>& vel) {
    detail::check(pg_advect_mac_f64(g.raw(), dst.data(), src.data(), dt, vel.data()), "advect_mac");
}

template <> inline void advect<float>(Simplex2<float>& dst, const Simplex2<float>& src, double dt,
                                      const Simplex1<float>& vel) {
    detail::check(pg_advect_f32(src.grid(), dst.data(), src.data(), dt, vel.data()), "advect");
}
template <> inline void advect<double>(Simplex2<double>& dst, const Simplex2<double>& src, double dt,
                                       const Simplex1<double>& vel) {
    detail::check(pg_advect_f64(src.grid(), dst.data(), src.data(), dt, vel.data()), "advect");
}
template <> inline void advect_mac<float>(Simplex1<float>& dst, const Simplex1<float>& src, double dt,
                                          const Simplex1<float>& vel) {
    detail::check(pg_advect_mac_f32(src.grid(), dst.data(), src.data(), dt, vel.data()), "advect_mac");
}
template <> inline void advect_mac<double>(Simplex1<double>& dst, const Simplex1<double>& src, double dt,
                                           const Simplex1<double>& vel) {
    detail::check(pg_advect_mac_f64(src.grid(), dst.data(), src.data(), dt, vel.data()), "advect_mac");
}

// One whole step of examples/dec_fluid.rs:46-141 (extension switches in
// pg_step_params; defaults below are the example's configuration).
inline pg_step_params reference_step_params() {
    pg_step_params p{};
    p.dt = 0.05;                 // dec_fluid.rs:43
    p.source_enabled = 1;        // dec_fluid.rs:48-57
    p.source_lo[0] = 0;
    p.source_lo[1] = 5;
    p.source_lo[2] = 54;
    p.source_hi[0] = 1;
    p.source_hi[1] = 20;
    p.source_hi[2] = 64;
    p.source_density = 1.0;
    p.source_vy = 20.0;
    p.solver.precond = PG_PRECOND_NONE;
    p.solver.threshold = 0.1;    // dec_fluid.rs:44
    p.solver.max_iter = 100;     // dec_fluid.rs:95
    return p;
}
inline PcgStats step(const GridBase& g, const pg_step_params& prm, Simplex1<float>& vel, Simplex2<float>& density,
                     Simplex2<float>& pressure) {
    PcgStats st{};
    detail::check(pg_step_f32(g.raw(), &prm, vel.data(), density.data(), pressure.data(), &st), "step", true);
    return st;
}
inline PcgStats step(const GridBase& g, const pg_step_params& prm, Simplex1<double>& vel, Simplex2<double>& density,
                     Simplex2<double>& pressure) {
    PcgStats st{};
    detail::check(pg_step_f64(g.raw(), &prm, vel.data(), density.data(), pressure.data(), &st), "step", true);
    return st;
}

}  // namespace panopaea
