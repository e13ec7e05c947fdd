/*
 * panopaea_gpu.h -- C ABI of the GB300 (sm_103a) grid-fluid library.
 *
 * The reference (msiglreith/panopaea, Rust) exposes this path as generic
 * traits and functions: Grid2d / Simplex1 / Simplex2 storage, the
 * Manifold2d operators, pcg::precond_conjugate_gradient, and the advect /
 * advect_mac / projection code of examples/dec_fluid.rs.  Every entry point
 * below names the reference item it replaces (path:line inside the
 * reference project).  A closure cannot cross a C ABI, so the PCG operator
 * closure of examples/dec_fluid.rs:100-119 is built in (the masked
 * Laplacian, scaled by dt) and the preconditioner is an enum.
 *
 * Conventions
 *   - Field pointers are DEVICE pointers.  Layouts are the reference's:
 *       cell field (Simplex2, grid.rs:76-100): row-major (y, x), h*w values;
 *         3D: (z, y, x), d*h*w values.
 *       face field (Simplex1, grid.rs:36-73): one buffer, part 0 = vy faces
 *         (h+1)*w, then part 1 = vx faces h*(w+1).  3D (extension): vz faces
 *         (d+1)*h*w, then vy d*(h+1)*w, then vx d*h*(w+1).
 *   - All calls are asynchronous on the grid's stream (pg_grid_set_stream)
 *     except those that return host scalars (pg_pcg_*, pg_solve_*,
 *     pg_step_*), which synchronise that stream before returning.
 *   - Calls on one grid handle are not thread-safe; distinct handles are.
 *   - Every function returns a pg_status; pg_last_error() gives the
 *     calling thread's last message.  Where the reference panics (shape
 *     mismatch, grid too small) this ABI returns PG_BAD_ARG.
 *   - No call falls back to the CPU: with no usable device, calls return
 *     PG_NO_DEVICE.
 */
#ifndef PANOPAEA_GPU_H
#define PANOPAEA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------------------- */
/* Status codes.  The reference returns () everywhere (pcg.rs:14-82 stops    */
/* silently after max_iterations); these make the outcomes explicit.         */
typedef enum pg_status {
    PG_OK = 0,
    PG_NOT_CONVERGED = 1,  /* max_iterations reached above the threshold */
    PG_NAN_DETECTED = 2,   /* NaN/Inf met in a CG reduction */
    PG_TIMEOUT = 3,        /* a bounded device-side wait gave up */
    PG_BAD_ARG = 4,        /* null pointer, bad shape, unsupported dims */
    PG_CUDA_ERROR = 5,     /* a CUDA runtime call failed */
    PG_NO_DEVICE = 6,      /* no CUDA device available */
    PG_OUT_OF_MEMORY = 7,
    PG_BREAKDOWN = 8       /* p.Ap <= 0 in CG (operator not SPD on p) */
} pg_status;

typedef enum pg_dtype { PG_F32 = 0, PG_F64 = 1 } pg_dtype;

/* Field kinds, named by simplex degree as in dec/manifold.rs:19-84. */
typedef enum pg_field_kind { PG_FACES = 1 /* Simplex1 */, PG_CELLS = 2 /* Simplex2 */ } pg_field_kind;

/* Preconditioner behind pcg.rs:4-6 `trait Preconditioner`.
 * PG_PRECOND_NONE is the reference's identity impl for () (pcg.rs:8-12);
 * JACOBI and MG are extensions. */
typedef enum pg_precond { PG_PRECOND_NONE = 0, PG_PRECOND_JACOBI = 1, PG_PRECOND_MG = 2 } pg_precond;

typedef struct pg_grid pg_grid;

/* Solve statistics (the reference prints "Iterations i", pcg.rs:61). */
typedef struct pg_pcg_stats {
    int64_t iterations;        /* operator applications (all rounds) */
    int64_t refinements;       /* FP64 residual rounds (0 for plain PCG) */
    double residual_max;       /* last ||r||inf the stop rule saw */
    double b_max;              /* ||b||inf */
    double threshold;          /* absolute threshold used */
    double true_residual_max;  /* ||b - A x||inf in FP64 after the solve; -1 if not computed */
    int32_t status;            /* pg_status of the solve */
    int32_t reserved;
} pg_pcg_stats;

/* Pressure-solve parameters for pg_solve_pressure_* and pg_step_*. */
typedef struct pg_solver_params {
    int32_t precond;       /* pg_precond */
    int32_t rel_stop;      /* 0: stop when ||r||inf < threshold (pcg.rs:58-60);
                              1: threshold = rel_tol * ||b||inf */
    double threshold;      /* absolute threshold (rel_stop = 0) */
    double rel_tol;        /* relative tolerance (rel_stop = 1) */
    int64_t max_iter;      /* max operator applications per CG run (pcg.rs:48) */
    int32_t refine;        /* 0: one plain CG run (the reference's algorithm);
                              n > 0: up to n FP64 residual refinement rounds */
    int32_t check_every;   /* iterations between host convergence polls (0 = auto) */
    double inner_rel_tol;  /* per-round relative tolerance with refine > 0 (0 = auto:
                              half the outer target, at least 1e-5) */
    int32_t mg_levels;     /* MG: number of levels (0 = auto) */
    int32_t mg_smooth;     /* MG: red-black Gauss-Seidel sweeps pre and post (0 = 2) */
    int32_t fp64_native;   /* refine > 0: 0 = the FP64-class residual, pressure
                              accumulation and projection run in double-float
                              (FP32 pairs, ~48-bit significand; GB300 runs
                              FP64 at 1/64 of the FP32 rate); 1 = native FP64 */
    int32_t initial_guess; /* extension, refine > 0 only: 1 = x holds an initial
                              guess (e.g. pg_unet_guess_f32) and the first round
                              solves for the correction of its FP64-class
                              residual; 0 = start from x = 0 (pcg.rs:29) */
} pg_solver_params;

/* One fluid step, examples/dec_fluid.rs:46-141 (the PNG dump at :143-164
 * is not part of the step).  Switches marked "extension" have no
 * reference counterpart and are 0 in the reference's configuration. */
typedef struct pg_step_params {
    double dt;                    /* dec_fluid.rs:43 */
    double buoyancy;              /* extension: vy += dt*buoyancy*mean(rho) on interior y faces */
    int32_t source_enabled;       /* dec_fluid.rs:48-57 inflow box */
    int32_t walls_after_advect;   /* extension: zero boundary faces after advection */
    int64_t source_lo[3];         /* (z, y, x) half-open cell box; 2D uses [1],[2] */
    int64_t source_hi[3];
    double source_density;        /* dec_fluid.rs:53 (1.0) */
    double source_vy;             /* dec_fluid.rs:54 (20.0) */
    const void* source_field;     /* extension: device cell field, density = max(density, field); may be NULL */
    int32_t zero_solid_after_project; /* extension: re-zero solid faces after projection */
    int32_t advect_scheme;        /* density advection: 0 = the reference's (dec_fluid.rs:173-211);
                                     extensions: 1 = MacCormack, 2 = BFECC (see pg_advect2_*) */
    pg_solver_params solver;      /* dec_fluid.rs:91-99: pcg(&(), .., 100, threshold, ..) */
} pg_step_params;

/* ----------------------------------------------------------------------- */
/* Errors */
const char* pg_status_string(int status);
const char* pg_last_error(void);
int pg_version(void);

/* ----------------------------------------------------------------------- */
/* Grids.  Replaces Grid2d::new / Grid2d::dim (domain/grid.rs:2-15);
 * pg_grid_create_3d defines the Grid3d the reference only declares
 * (domain/grid.rs:17-20).  The handle also owns the solid mask, the stream
 * and the solver workspace. */
int pg_grid_create_2d(int64_t h, int64_t w, pg_grid** out);
int pg_grid_create_3d(int64_t d, int64_t h, int64_t w, pg_grid** out);
int pg_grid_destroy(pg_grid* grid);
/* Writes (d, h, w) (d = 1 for 2D) and returns the number of dimensions (2
 * or 3), or a negative pg_status. */
int pg_grid_dim(const pg_grid* grid, int64_t dim_out[3]);
/* Manifold2d::num_elem_1 / num_elem_2 (dec/grid.rs:350-356). */
int64_t pg_grid_num_elem_1(const pg_grid* grid);
int64_t pg_grid_num_elem_2(const pg_grid* grid);
/* Bind a cudaStream_t (NULL = legacy default stream). */
int pg_grid_set_stream(pg_grid* grid, void* cuda_stream);
int pg_grid_synchronize(pg_grid* grid);
/* Solid faces, host array in the face layout (1 = solid).  This is the
 * obstacle masking of examples/dec_fluid.rs:71-78 and :104-112 as data:
 * masked faces carry no flux in the RHS and no coupling in the Laplacian.
 * NULL clears the mask. */
int pg_grid_set_solid_faces(pg_grid* grid, const uint8_t* host_face_solid);
/* Solid cells, host array in the cell layout (1 = solid).  Extension: a
 * face is solid iff an adjacent cell is solid. */
int pg_grid_set_solid_cells(pg_grid* grid, const uint8_t* host_cell_solid);

/* ----------------------------------------------------------------------- */
/* Fields.  Replaces Manifold2d::new_simplex_1 / new_simplex_2
 * (dec/grid.rs:362-371): zero-filled device storage of the layouts above. */
int pg_field_alloc(const pg_grid* grid, int kind, int dtype, void** dev_out);
int pg_field_free(void* dev);
/* Host <-> device copies, stream-ordered on the grid's stream (host
 * memory should be pinned for overlap; pageable memory works). */
int pg_copy_h2d(const pg_grid* grid, void* dev_dst, const void* host_src, size_t bytes);
int pg_copy_d2h(const pg_grid* grid, void* host_dst, const void* dev_src, size_t bytes);

/* ----------------------------------------------------------------------- */
/* DEC operators (2D API parity with dec/manifold.rs:29-83).  The _f64
 * forms take double*.  3D grids accept derivative_0_dual (negative
 * gradient on interior faces) and mask_solid_faces; the hodge_1_* and
 * derivative_1_primal forms are 2D-only (PG_BAD_ARG on a 3D grid). */

/* hodge_1_dual (manifold.rs:74-76 -> grid.rs:223-238): primal.vy = -dual.vy, primal.vx = dual.vx */
int pg_hodge_1_dual_f32(const pg_grid* grid, float* primal, const float* dual);
int pg_hodge_1_dual_f64(const pg_grid* grid, double* primal, const double* dual);
/* hodge_1_primal (manifold.rs:70-72 -> grid.rs:206-221): dual.vy = primal.vy, dual.vx = -primal.vx */
int pg_hodge_1_primal_f32(const pg_grid* grid, float* dual, const float* primal);
int pg_hodge_1_primal_f64(const pg_grid* grid, double* dual, const double* primal);
/* hodge_2_primal (manifold.rs:78-80 -> grid.rs:253-255): copy */
int pg_hodge_2_primal_f32(const pg_grid* grid, float* dual, const float* primal);
int pg_hodge_2_primal_f64(const pg_grid* grid, double* dual, const double* primal);
/* derivative_1_primal (manifold.rs:57-59 -> grid.rs:295-305):
 * face = -bottom + top - left + right */
int pg_derivative_1_primal_f32(const pg_grid* grid, float* faces, const float* edges);
int pg_derivative_1_primal_f64(const pg_grid* grid, double* faces, const double* edges);
/* derivative_0_dual (manifold.rs:50-52 -> grid.rs:318-334): interior faces
 * only, boundary faces keep their value */
int pg_derivative_0_dual_f32(const pg_grid* grid, float* edges, const float* faces);
int pg_derivative_0_dual_f64(const pg_grid* grid, double* edges, const double* faces);
/* Zero every solid face (examples/dec_fluid.rs:71-78, :104-112). */
int pg_mask_solid_faces_f32(const pg_grid* grid, float* edges);
int pg_mask_solid_faces_f64(const pg_grid* grid, double* edges);

/* ----------------------------------------------------------------------- */
/* Fused step operators. */

/* The PCG operator closure of examples/dec_fluid.rs:100-119:
 * out = dt * d1(*1^-1(M d0dual(*2 p))), i.e. dt * (-Laplacian) with solid
 * and boundary faces closed.  One kernel; same arithmetic order. */
int pg_laplacian_f32(const pg_grid* grid, float* out, const float* p, double dt);
int pg_laplacian_f64(const pg_grid* grid, double* out, const double* p, double dt);
/* The RHS of examples/dec_fluid.rs:68-83: b = -d1(*1^-1(M u)). */
int pg_divergence_rhs_f32(const pg_grid* grid, float* b, const float* vel);
int pg_divergence_rhs_f64(const pg_grid* grid, double* b, const double* vel);
/* advect (examples/dec_fluid.rs:173-211): semi-Lagrangian, cell-centred,
 * bilinear (trilinear in 3D).  Needs every dimension >= 2. */
int pg_advect_f32(const pg_grid* grid, float* dst, const float* src, double dt, const float* vel);
int pg_advect_f64(const pg_grid* grid, double* dst, const double* src, double dt, const double* vel);
/* Second-order advection of a cell scalar (extension): scheme 1 =
 * MacCormack, scheme 2 = BFECC, both built from advect above and limited
 * to the range of the source values of the first-order sample (falling
 * back to it where they leave that range).  Scratch is library-owned. */
int pg_advect2_f32(const pg_grid* grid, float* dst, const float* src, double dt, const float* vel, int scheme);
int pg_advect2_f64(const pg_grid* grid, double* dst, const double* src, double dt, const double* vel, int scheme);
/* advect_mac (examples/dec_fluid.rs:213-291): MAC face advection. */
int pg_advect_mac_f32(const pg_grid* grid, float* dst, const float* src, double dt, const float* vel);
int pg_advect_mac_f64(const pg_grid* grid, double* dst, const double* src, double dt, const double* vel);
/* Projection + walls (examples/dec_fluid.rs:123-141):
 * vel += dt * d0dual(p) on interior faces, then boundary faces = 0;
 * zero_solid != 0 (extension) also zeroes solid faces. */
int pg_project_f32(const pg_grid* grid, float* vel, const float* p, double dt, int zero_solid);
int pg_project_f64(const pg_grid* grid, double* vel, const double* p, double dt, int zero_solid);
/* Wall step alone (examples/dec_fluid.rs:128-141). */
int pg_walls_f32(const pg_grid* grid, float* vel);
int pg_walls_f64(const pg_grid* grid, double* vel);

/* ----------------------------------------------------------------------- */
/* Solvers. */

/* pcg::precond_conjugate_gradient (pcg.rs:14-82), operator = the masked
 * Laplacian closure scaled by dt.  Same recurrence and stop rule: x = 0;
 * return if ||b||inf < threshold; stop when ||r||inf < threshold or after
 * max_iterations operator applications.  residual / auxiliary / search
 * are caller-owned work vectors as in the reference (residual ends as r,
 * auxiliary as A*p, search as p).  Reductions are accumulated in FP64. */
int pg_pcg_f32(const pg_grid* grid, int precond, float* x, const float* b, int64_t max_iterations,
               double threshold, float* residual, float* auxiliary, float* search, double dt,
               pg_pcg_stats* stats);
int pg_pcg_f64(const pg_grid* grid, int precond, double* x, const double* b, int64_t max_iterations,
               double threshold, double* residual, double* auxiliary, double* search, double dt,
               pg_pcg_stats* stats);

/* Allocation-free PCG.  No counterpart in the reference.
 *
 * The same solve as pg_pcg_f32 for callers that cannot allocate device
 * memory: code whose device memory is all owned by a host framework's pool
 * or arena (an allocation hidden inside a library call would escape its
 * accounting), and time-critical loops where cudaMalloc / cudaFree would
 * synchronise the device.  It takes no pg_grid (creating one allocates):
 * the grid is (nd, d, h, w) with d = 1 for nd = 2, and the geometry is
 * either NULL (no obstacles: every interior face open) or a device array of
 * one byte per cell of face-open bits (1 = x-low, 2 = x-high, 4 = y-low,
 * 8 = y-high, 16 = z-low, 32 = z-high; set a bit iff that face is interior
 * and not solid).  The caller passes every input and output, as in
 * pg_pcg_f32; cuda_stream may be NULL (legacy default stream).
 *
 * Its scratch -- CG state, reduction partials, a second search-direction
 * buffer, and the wall-only face bits -- is one fixed 5.1 MiB device array
 * in the library (held by every GPU that loads the library until the
 * process exits), so grids are limited to 1,048,576 cells; larger grids
 * are rejected with PG_BAD_ARG.  The first call on each device looks the
 * array's device address up (cudaGetSymbolAddress) with that device
 * current and keeps it for the life of the process; make that first call
 * before any stream capture.  A cudaDeviceReset ends the context that
 * address belongs to: after one, make no further call of this entry point
 * on that device.  Every call shares the array and overwrites what the
 * previous call left there (the state is cleared at the start of each
 * call), so calls that overlap on the GPU -- on different streams, or from
 * different threads -- race.  The call reads the solver state back to the
 * host while it iterates and synchronises cuda_stream before it returns.
 * It calls no cudaMalloc, cudaFree or allocating library routine. */
int pg_pcg_noalloc_f32(int32_t nd, int64_t d, int64_t h, int64_t w, const uint8_t* cell_flags, int precond,
                       float* x, const float* b, int64_t max_iterations, double threshold, float* residual,
                       float* auxiliary, float* search, double dt, void* cuda_stream, pg_pcg_stats* stats);

/* Pressure solve A x = b with library-owned work vectors: the reference's
 * PCG (refine = 0), or FP32 CG inside FP64 residual refinement (refine >
 * 0), with the preconditioner of `params`.  x is overwritten (initial
 * guess 0, as pcg.rs:32). */
int pg_solve_pressure_f32(const pg_grid* grid, const pg_solver_params* params, float* x, const float* b,
                          double dt, pg_pcg_stats* stats);

/* One fluid step (examples/dec_fluid.rs:46-141): source -> advect density
 * (old u) -> advect_mac u (old u) -> [walls] -> [buoyancy] -> -div ->
 * pressure solve -> projection + walls.  vel, density, pressure are
 * device fields updated in place; pressure receives the solution. */
int pg_step_f32(const pg_grid* grid, const pg_step_params* params, float* vel, float* density, float* pressure,
                pg_pcg_stats* stats);
int pg_step_f64(const pg_grid* grid, const pg_step_params* params, double* vel, double* density,
                double* pressure, pg_pcg_stats* stats);

/* ----------------------------------------------------------------------- */
/* Sparse and diagonal matrix products (device pointers; stream may be NULL). */

/* SparseMatrix::mul_vec (panopaea/src/sparse.rs:119-128): CSR with
 * row_indices[rows + 1] and col_indices (int64, as the reference's usize);
 * b[i] = left fold of acc + data[k] * x[col_indices[k]] over row i. */
int pg_csr_mul_vec_f32(int64_t rows, const int64_t* row_indices, const int64_t* col_indices, const float* data,
                       const float* x, float* b, void* cuda_stream);
int pg_csr_mul_vec_f64(int64_t rows, const int64_t* row_indices, const int64_t* col_indices, const double* data,
                       const double* x, double* b, void* cuda_stream);
/* DiagonalMatrix::mul_vec (sparse.rs:20-25): b = x * a. */
int pg_diag_mul_vec_f32(int64_t n, const float* a, const float* x, float* b, void* cuda_stream);
int pg_diag_mul_vec_f64(int64_t n, const double* a, const double* x, double* b, void* cuda_stream);

/* Headless image of a 2D cell field: imgproc::transfer (panopaea_utils/src/
 * imgproc.rs:2-5) in f64 into three equal 8-bit channels, rows flipped as
 * png::export writes them (png.rs:12), i.e. rgb[(y * w + x) * 3 + c] shows
 * field[(h - 1 - y) * w + x]; the density dump of examples/dec_fluid.rs:143-164. */
int pg_transfer_rgb8_f32(int64_t h, int64_t w, const float* field, double lower, double upper, uint8_t* rgb,
                         void* cuda_stream);
int pg_transfer_rgb8_f64(int64_t h, int64_t w, const double* field, double lower, double upper, uint8_t* rgb,
                         void* cuda_stream);

/* ----------------------------------------------------------------------- */
/* Batches of independent 2D grids (extension; the reference steps a single
 * grid, examples/dec_fluid.rs:46-141).  Grids of different sizes are packed
 * back to back: grid i's cell field starts at cell_offsets[i] and its face
 * field at face_offsets[i], each in the reference layout.  Every stage of
 * the step is one launch over all grids; each grid has its own CG scalars
 * and stop rule, converged grids retire, the CG loop is a CUDA graph. */
typedef struct pg_batch pg_batch;
int pg_batch_create_2d(int32_t count, const int64_t* heights, const int64_t* widths, pg_batch** out);
int pg_batch_destroy(pg_batch* batch);
int pg_batch_set_stream(pg_batch* batch, void* cuda_stream);
/* count + 1 offsets each (the last is the packed total). */
int pg_batch_layout(const pg_batch* batch, int64_t* cell_offsets, int64_t* face_offsets);
/* Packed host cell mask (1 = solid; a face is solid iff an adjacent cell is); NULL clears. */
int pg_batch_set_solid_cells(pg_batch* batch, const uint8_t* host_cell_solid);
/* Tile shape (tile_x * tile_y threads, a multiple of 32, <= 256) and whether
 * the search-direction update is fused into the SpMV. */
int pg_batch_tile(const pg_batch* batch, int32_t* tile_x, int32_t* tile_y, int32_t* fused);
int pg_batch_set_tile(pg_batch* batch, int32_t tile_x, int32_t tile_y, int32_t fused);
/* Time the candidate tile shapes and fusion choices on this batch and keep
 * the fastest; with cache_path, reuse / append "key tx ty fused" lines
 * keyed by device and batch shape. */
int pg_batch_autotune(pg_batch* batch, const char* cache_path);
/* One step of every grid.  params->source_enabled must be 0 (use
 * source_field, a packed device cell field); solver: NONE, JACOBI or MG (a
 * batched multigrid V-cycle over every grid's own hierarchy), no
 * refinement.  stats: count entries (may be NULL).  Returns PG_OK, or the
 * first non-OK per-grid status. */
int pg_batch_step_f32(pg_batch* batch, const pg_step_params* params, float* vel, float* density, float* pressure,
                      pg_pcg_stats* stats);

/* ----------------------------------------------------------------------- */
/* BF16-stored density (extension; the reference's density is a Simplex2 of
 * f64, examples/dec_fluid.rs:34-37).  Density values are bfloat16 bit
 * patterns; every stage reads them exactly into FP32, computes as the FP32
 * kernels do and rounds to nearest even on store.  Velocity, pressure and the
 * solve are FP32 (with the solver's refinement options). */

/* advect (dec_fluid.rs:173-211) of a BF16 cell field with FP32 velocity. */
int pg_advect_bf16(const pg_grid* grid, uint16_t* dst, const uint16_t* src, double timestep, const float* vel);
/* pg_step_f32 with the density stored in BF16 (advect_scheme must be 0);
 * source_field, when set, is an FP32 device cell field. */
int pg_step_bf16rho_f32(const pg_grid* grid, const pg_step_params* params, float* vel, uint16_t* density,
                        float* pressure, pg_pcg_stats* stats);

/* ----------------------------------------------------------------------- */
/* Wavelet and divergence-free wavelet transforms (panopaea/src/math/wavelet,
 * mod.rs:1-451, filters of haar.rs and spline.rs; the reference marks the
 * module as early, mostly abandoned tests -- restated as written).  FP64
 * device arrays, row-major (h, w) in 2D; `temp` is a caller scratch array of
 * the same size; stream may be NULL.  Every transformed length must be a
 * multiple of 2^levels and the last level at least the filter length. */
typedef enum pg_wavelet {
    PG_WAVELET_HAAR = 0,    /* haar.rs */
    PG_WAVELET_BIOR13 = 1,  /* spline.rs Bior13 */
    PG_WAVELET_BIOR22 = 2,
    PG_WAVELET_BIOR24 = 3,
    PG_WAVELET_BIOR31 = 4
} pg_wavelet;
typedef enum pg_wavelet_mode {
    PG_WAVELET_ISOTROPIC = 0,   /* fwt_2d_isotropic / ifwt_2d_isotropic (same filter on both axes:
                                   fwt_2d_separate_isotropic is the same forward transform) */
    PG_WAVELET_ANISOTROPIC = 1, /* fwt_2d_anisotropic (forward only, as in the reference) */
    PG_WAVELET_SEPARATE = 2     /* ifwt_2d_separate_isotropic (x, then y) */
} pg_wavelet_mode;
/* fwt_1d / ifwt_1d (mod.rs:114-143), in place: |coarse n|detail n|detail n-1|... */
int pg_wavelet_fwt_1d(int wavelet, double* data, int64_t n, int levels, double* temp, void* cuda_stream);
int pg_wavelet_ifwt_1d(int wavelet, double* data, int64_t n, int levels, double* temp, void* cuda_stream);
/* 2D forward (mod.rs:145-170, 206-231, 262-294) and inverse (mod.rs:172-204, 233-260) */
int pg_wavelet_fwt_2d(int mode, int wavelet_x, int wavelet_y, double* data, int64_t h, int64_t w, int levels,
                      double* temp, void* cuda_stream);
int pg_wavelet_ifwt_2d(int mode, int wavelet_x, int wavelet_y, double* data, int64_t h, int64_t w, int levels,
                       double* temp, void* cuda_stream);
/* div_coeff_2d / inv_div_coeff_2d (mod.rs:296-451): the divergence / n
 * coefficients of the wavelet coefficients of (vx, vy) and back. */
int pg_wavelet_div_coeff_2d(int levels, const double* vx, const double* vy, double* div, double* n, int64_t h,
                            int64_t w, void* cuda_stream);
int pg_wavelet_inv_div_coeff_2d(int levels, const double* div, const double* n, double* vx, double* vy, int64_t h,
                                int64_t w, void* cuda_stream);

/* Border variants (mod.rs:454-681): zero sampling outside a line, bands of
 * s / 2 + 2 B samples for an s-sample line (B = the filter length: 2 Haar,
 * 6 Bior13 and Bior22, 10 Bior24, 4 Bior31), so the transform is larger
 * than its input and the inverse reconstructs the input's leading samples.
 * A transform is one packed FP64 array: the coarse band, then per level
 * (finest first) its detail band (1D) or its three detail bands lyhx,
 * hylx, hyhx (2D, each row-major) -- the (coarse, details) pair the
 * reference returns.  The sizes functions run on the host only (no CUDA
 * call): `packed` elements of the transform, `temp` elements of the
 * scratch array the transforms need (0: none; temp may then be NULL) and
 * the inverse's output length (1D: coarse + detail - 4 B per level) or
 * shape (2D: 2 coarse - 4 B per level), -1 where that arithmetic goes below
 * zero at some level (tiny inputs, many levels: the reference's unsigned
 * sizes underflow there) and the inverse returns PG_BAD_ARG.  Input, output
 * and temp must not overlap.  n, h, w >= 2; levels 0..40. */
int pg_wavelet_border_sizes_1d(int wavelet, int64_t n, int levels, int64_t* packed, int64_t* temp,
                               int64_t* inverse_n);
int pg_wavelet_border_sizes_2d(int wavelet_x, int wavelet_y, int64_t h, int64_t w, int levels, int64_t* packed,
                               int64_t* temp, int64_t* inverse_h, int64_t* inverse_w);
/* fwt_1d_border / ifwt_1d_border (mod.rs:454-486); the inverse takes the
 * forward's n and levels (n and n + 1 give the same bands for even n). */
int pg_wavelet_fwt_1d_border(int wavelet, const double* input, int64_t n, int levels, double* packed, double* temp,
                             void* cuda_stream);
int pg_wavelet_ifwt_1d_border(int wavelet, const double* packed, int64_t n, int levels, double* output, double* temp,
                              void* cuda_stream);
/* fwt_2d_separate_isotropic_border / ifwt_2d_separate_isotropic_border
 * (mod.rs:551-641): x then y forward, y then x inverse. */
int pg_wavelet_fwt_2d_border(int wavelet_x, int wavelet_y, const double* input, int64_t h, int64_t w, int levels,
                             double* packed, double* temp, void* cuda_stream);
int pg_wavelet_ifwt_2d_border(int wavelet_x, int wavelet_y, const double* packed, int64_t h, int64_t w, int levels,
                              double* output, double* temp, void* cuda_stream);
/* div_coeff_2d_border (mod.rs:645-681) of two packed 2D border transforms of
 * (h, w) inputs: the packed div and n transforms. */
int pg_wavelet_div_coeff_2d_border(int wavelet_x, int wavelet_y, const double* vx, const double* vy, int64_t h,
                                   int64_t w, int levels, double* div, double* n, void* cuda_stream);

/* ----------------------------------------------------------------------- */
/* Learned pressure guess (extension, no reference counterpart: panopaea has
 * no learned component).  A 3-level 3D conv U-Net, 16 base channels, BF16
 * weights and activations with FP32 accumulation on the tensor cores, trained
 * on the device by its own forward and backward kernels.  Inputs per cell:
 * b / rms(b) and the open-face count / 6 of the grid's mask; output: a guess
 * of the solution of A p = b (A = dt * the masked Laplacian), 0 on solid
 * cells.  3D grids only; every side a multiple of 4 and >= 16. */

typedef struct pg_unet pg_unet;

typedef struct pg_adam_params {
    double lr;
    double beta1;
    double beta2;
    double eps;
    double grad_scale;     /* gradients are multiplied by this (1 / samples) */
} pg_adam_params;

/* Number of FP32 parameters: 10 conv weights [27][c_in][c_out] in layer
 * order, then the 16 weights of the 1x1 output layer. */
int64_t pg_unet_num_params(void);
/* Network and activations for grids of shape (d, h, w). */
int pg_unet_create(int64_t d, int64_t h, int64_t w, pg_unet** out);
int pg_unet_destroy(pg_unet* net);
int pg_unet_set_stream(pg_unet* net, void* cuda_stream);
/* Host parameters (pg_unet_num_params floats) and the output scale (the
 * typical |p| * dt / rms(b) of the training data); resets the Adam state. */
int pg_unet_set_params(pg_unet* net, const float* host_params, double out_scale);
int pg_unet_get_params(const pg_unet* net, float* host_params, double* out_scale);
/* Accumulated gradients (host copy) and their reset. */
int pg_unet_get_grads(const pg_unet* net, float* host_grads);
int pg_unet_zero_grads(pg_unet* net);
/* Training loss: 0 = mean squared error of the normalised guess q on open
 * cells, sum e^2 / cells; 1 (default) = its energy norm, sum e (A1 e) / cells
 * with A1 the masked Laplacian at dt = 1 (the error norm CG reduces, blind
 * to the constant null-space offset); e = q - p_true dt / (rms(b) out_scale). */
int pg_unet_set_loss(pg_unet* net, int kind);
/* Forward pass and loss for one sample (device b, device target p_true,
 * the grid's solid mask); adds the gradient of the loss to the accumulated
 * gradients.  loss may be NULL (else synchronises). */
int pg_unet_accumulate_f32(pg_unet* net, const pg_grid* grid, const float* b, const float* p_true, double dt,
                           double* loss);
/* One Adam step on the accumulated gradients, then zeroes them. */
int pg_unet_adam_step(pg_unet* net, const pg_adam_params* params);
/* p = the network's raw output for b (no step-length scaling).  Asynchronous. */
int pg_unet_forward_f32(pg_unet* net, const pg_grid* grid, const float* b, double dt, float* p);
/* Guess for A x = b: x = alpha d with d = the network's output for b and
 * alpha = (d.b) / (d.Ad), the step that minimises the energy norm of the
 * error along d (so the guess is never worse than x = 0 in that norm);
 * corrections > 0 repeats it on the residual (x += alpha d, d = net(b - Ax)).
 * Asynchronous. */
int pg_unet_guess_f32(pg_unet* net, const pg_grid* grid, const float* b, double dt, int corrections, float* x);
/* Pressure solve A x = b whose preconditioner is the network plus a Jacobi
 * step (no reference counterpart; it takes the place of the `Preconditioner`
 * of pcg.rs:4-6): for a residual r, q = net(r), a = (q.r) / (q.Aq) and
 * z = a q + D^-1 (r - a A q).  z depends on r non-linearly, so the CG is
 * the flexible one (Polak-Ribiere beta); it runs to params' tolerance,
 * inside FP64-class refinement when params->refine > 0, so the result's
 * accuracy does not depend on the network.  params->precond is not used.
 * Synchronous; returns the solve's status. */
int pg_solve_pressure_learned_f32(const pg_grid* grid, const pg_solver_params* params, pg_unet* net, float* x,
                                  const float* b, double dt, pg_pcg_stats* stats);
/* Waits for the network's stream; PG_TIMEOUT if one of its tensor-core
 * kernels gave up a bounded wait since the last check (its results are then
 * not to be trusted; the flag is cleared), else PG_OK. */
int pg_unet_check(pg_unet* net);

/* ----------------------------------------------------------------------- */
/* Instrumentation (no reference counterpart; the reference only prints
 * wall-clock ms around the PCG, examples/dec_fluid.rs:87,121). */

/* Kernel launches issued by this library since it was loaded. */
int64_t pg_kernel_launches(void);
/* on != 0: record a CUDA event pair around every launch, per kernel kind. */
int pg_profile_enable(int on);
int pg_profile_reset(void);
int pg_profile_num_kinds(void);
const char* pg_profile_kind_name(int kind);
/* Waits for the recorded events and returns the summed device time (ms)
 * and launch count of one kernel kind. */
int pg_profile_read(int kind, double* total_ms, int64_t* launches);
/* The same over the launches that did work (a CG loop polled from the host
 * launches iterations past its stop test, which exit at entry in a few
 * microseconds): those of at least the smaller of a quarter of the kind's
 * longest launch and the geometric mean of its shortest and longest. */
int pg_profile_read_active(int kind, double* total_ms, int64_t* launches);

/* Test hook (no reference counterpart): the poll budget of the TMA
 * pipeline-stage waits of the z-marching kernels.  0 makes every stage wait
 * give up at once, so the give-up path runs without any fault: the block
 * waits (bounded) for its copies in flight, sets PG_TIMEOUT and stops the
 * solve.  A solve that returns PG_TIMEOUT has untrustworthy results; the
 * next solve starts from a fresh state.  Synchronous; restore the budget
 * with pg_debug_stage_wait_polls_default(). */
int pg_debug_set_stage_wait_polls(uint32_t polls);
uint32_t pg_debug_stage_wait_polls_default(void);

/* Diagnostic (no reference counterpart): average device time (ms) of one
 * multigrid V-cycle of the grid's hierarchy for dt with nsmooth sweeps, and
 * of its coarse part (every level below the fine one), each captured once
 * into a CUDA graph and replayed `reps` times on a private stream with r = 0.
 * Needs at least two levels; synchronous. */
int pg_debug_mg_vcycle_ms(pg_grid* g, double dt, int nsmooth, int reps, double* full_ms, double* coarse_ms);

/* Test hook (host only, no GPU needed): the Moore-Penrose pseudo-inverse the
 * multigrid coarsest solve uses, of the symmetric n x n row-major matrix a
 * (overwritten; eigenvalues below 1e-10 of the largest count as zero). */
int pg_debug_sym_pinv(int n, double* a);

#ifdef __cplusplus
}
#endif

#endif /* PANOPAEA_GPU_H */
