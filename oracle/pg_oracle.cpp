// pg_oracle.cpp -- ORACLE: test infrastructure only.
//
// A CPU restatement, in plain C++, of the reference (msiglreith/panopaea, Rust)
// grid-fluid path: DEC operators, the masked Laplacian closure, the
// preconditioned conjugate gradient, semi-Lagrangian advection and the
// projection step.  It exists to CHECK the CUDA library, and to time the
// reference's CPU algorithm; no product code links, loads or calls it.
//
// Parity pinning:
//   * The DEC operators (hodge_1_dual, derivative_1_primal, derivative_0_dual,
//     hodge_2_primal) and the Laplacian closure are pinned by the reference's
//     own golden vectors (panopaea/src/dec/grid.rs:459-465 and :504), which
//     the CPU test-suite checks this file against.
//   * PCG (panopaea/src/pcg.rs), advection and projection
//     (examples/dec_fluid.rs) have no golden vectors in the reference and the
//     reference (Rust, crates.io dependencies not vendored) cannot be built
//     here: those rows are restated from source, parity unpinned.
//   * Everything 3D, buoyancy, the Jacobi preconditioner and the cell-mask
//     rule are extensions with no reference behaviour; they follow the 2D
//     conventions of the cited code and are defined here.
//
// Floating point: all arithmetic is done in T (float or double), in the same
// operation order as the cited Rust; the file must be built with
// -ffp-contract=off so that a*b+c is never fused (Rust never fuses).
//
// Threading: the reference runs derivative_0_dual and derivative_1_primal
// under rayon (par_azip!, grid.rs:298-304,322-333) and everything else
// serially.  `pgo_set_threads(n, all)` reproduces that with OpenMP (all=0),
// or parallelises every loop (all=1, used only to make tests faster).

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

int g_threads = 1;
int g_all = 0;
int g_dot64 = 0;  // 1: accumulate dot products in double (the GPU's choice)

#define PGO_STR(x) #x
#define PGO_PRAGMA(x) _Pragma(PGO_STR(x))
// Loops the reference runs under rayon.
#define PAR_REF PGO_PRAGMA(omp parallel for if (g_threads > 1) num_threads(g_threads) schedule(static))
// Loops the reference runs serially (parallel only in "all" mode).
#define PAR_ALL PGO_PRAGMA(omp parallel for if (g_all && g_threads > 1) num_threads(g_threads) schedule(static))

typedef std::ptrdiff_t idx;

// ---------------------------------------------------------------------------
// math/interp.rs:7-36
template <class T> inline T linear(T a0, T a1, T s) { return a0 * (T(1) - s) + a1 * s; }
template <class T> inline T bilinear(T a00, T a01, T a10, T a11, T s, T t) {
    return linear(linear(a00, a01, s), linear(a10, a11, s), t);
}
template <class T>
inline T trilinear(T a000, T a001, T a010, T a011, T a100, T a101, T a110, T a111, T s, T t, T u) {
    return linear(bilinear(a000, a001, a010, a011, s, t), bilinear(a100, a101, a110, a111, s, t), u);
}

// Rust f64::max / f64::min return the non-NaN operand: std::fmax / std::fmin.
template <class T> inline T rmax(T a, T b) { return std::fmax(a, b); }
template <class T> inline T rmin(T a, T b) { return std::fmin(a, b); }

// ---------------------------------------------------------------------------
// Cell-centred clamp + floor of examples/dec_fluid.rs:194-201, per axis.
// `hi` = n - 1.00001 computed in double then rounded to T.  In float, for
// n >= 257 the bound rounds to n-1; the index is then clamped to n-2 so the
// +1 neighbour stays in range (weight becomes exactly 1).
template <class T> inline void cell_coord(T pos, idx n, idx* i0, T* frac) {
    const T hi = (T)((double)n - 1.00001);
    T p = rmin(rmax(pos - T(0.5), T(0)), hi);
    idx i = (idx)std::floor(p);
    if (i > n - 2) i = n - 2;
    *i0 = i;
    *frac = p - (T)i;
}

// Face-sample coordinate of examples/dec_fluid.rs:236-244 / :274-281:
// p = floor(pos - off).max(0); i0 = min(p, n-1), i1 = min(p+1, n-1);
// frac = ((pos - off) - p).min(1).max(0).  `p` is kept as a T value, which
// equals the reference's usize cast for every finite position below 2^24.
template <class T> inline void face_coord(T pos, T off, idx n, idx* i0, idx* i1, T* frac) {
    const T q = pos - off;
    const T p = rmax(std::floor(q), T(0));
    const T last = (T)(n - 1);
    *i0 = (idx)rmin(p, last);
    *i1 = (idx)rmin(p + T(1), last);
    *frac = rmax(rmin(q - p, T(1)), T(0));
}

// ---------------------------------------------------------------------------
// 2D, storage of panopaea/src/dec/grid.rs:36-100: cells (h,w) row-major;
// faces = [vy (h+1)*w | vx h*(w+1)].

// grid.rs:223-238 (Manifold2d::hodge_1_dual = Hodge<Simplex1>::apply_inv)
template <class T> void hodge_1_dual_2d(T* primal, const T* dual, idx h, idx w) {
    const idx n0 = (h + 1) * w, n = n0 + h * (w + 1);
    PAR_ALL for (idx i = 0; i < n0; ++i) primal[i] = -dual[i];
    PAR_ALL for (idx i = n0; i < n; ++i) primal[i] = dual[i];
}

// grid.rs:206-221 (Manifold2d::hodge_1_primal = Hodge<Simplex1>::apply)
template <class T> void hodge_1_primal_2d(T* dual, const T* primal, idx h, idx w) {
    const idx n0 = (h + 1) * w, n = n0 + h * (w + 1);
    PAR_ALL for (idx i = 0; i < n0; ++i) dual[i] = primal[i];
    PAR_ALL for (idx i = n0; i < n; ++i) dual[i] = -primal[i];
}

// grid.rs:253-255 (hodge_2_primal: assign)
template <class T> void hodge_2_primal(T* dual, const T* primal, idx n) {
    PAR_ALL for (idx i = 0; i < n; ++i) dual[i] = primal[i];
}

// grid.rs:295-305: face = -bottom + top - left + right
template <class T> void derivative_1_primal_2d(T* faces, const T* edges, idx h, idx w) {
    const T* e0 = edges;
    const T* e1 = edges + (h + 1) * w;
    PAR_REF for (idx y = 0; y < h; ++y)
        for (idx x = 0; x < w; ++x) {
            const T top = e0[y * w + x], bottom = e0[(y + 1) * w + x];
            const T left = e1[y * (w + 1) + x], right = e1[y * (w + 1) + x + 1];
            faces[y * w + x] = -bottom + top - left + right;
        }
}

// grid.rs:318-334: interior faces only; boundary faces keep their value.
template <class T> void derivative_0_dual_2d(T* edges, const T* faces, idx h, idx w) {
    T* e0 = edges;
    T* e1 = edges + (h + 1) * w;
    PAR_REF for (idx y = 1; y < h; ++y)
        for (idx x = 0; x < w; ++x) {
            const T f0 = faces[(y - 1) * w + x], f1 = faces[y * w + x];
            e0[y * w + x] = -(f1 - f0);
        }
    PAR_REF for (idx y = 0; y < h; ++y)
        for (idx x = 1; x < w; ++x) {
            const T f0 = faces[y * w + x - 1], f1 = faces[y * w + x];
            e1[y * (w + 1) + x] = f0 - f1;
        }
}

// examples/dec_fluid.rs:71-78, :104-112 generalised: zero every face whose
// solid flag is set (flags in the Simplex1 layout).
template <class T> void mask_faces(T* edges, const uint8_t* solid, idx nf) {
    if (!solid) return;
    PAR_ALL for (idx i = 0; i < nf; ++i)
        if (solid[i]) edges[i] = T(0);
}

// The operator closure of examples/dec_fluid.rs:100-119, composed literally.
// `tmp_face` must have zero boundary faces on entry (dec_fluid.rs:89).
template <class T>
void laplacian_closure_2d(T* out, const T* p, T dt, const uint8_t* face_solid, idx h, idx w, T* tmp_cell,
                          T* tmp_face, T* tmp_face2) {
    const idx nc = h * w, nf = (h + 1) * w + h * (w + 1);
    hodge_2_primal(tmp_cell, p, nc);
    derivative_0_dual_2d(tmp_face, tmp_cell, h, w);
    mask_faces(tmp_face, face_solid, nf);
    hodge_1_dual_2d(tmp_face2, tmp_face, h, w);
    derivative_1_primal_2d(out, tmp_face2, h, w);
    PAR_ALL for (idx i = 0; i < nc; ++i) out[i] = out[i] * dt;
}

// examples/dec_fluid.rs:68-83: b = -d1(*1^-1(M u)).
template <class T> void divergence_rhs_2d(T* b, const T* vel, const uint8_t* face_solid, idx h, idx w, T* tmp_face) {
    const idx nc = h * w, nf = (h + 1) * w + h * (w + 1);
    hodge_1_dual_2d(tmp_face, vel, h, w);
    mask_faces(tmp_face, face_solid, nf);
    derivative_1_primal_2d(b, tmp_face, h, w);
    PAR_ALL for (idx i = 0; i < nc; ++i) b[i] = -b[i];
}

// examples/dec_fluid.rs:173-211
template <class T> void advect_2d(T* dst, const T* q, T dt, const T* vel, idx h, idx w) {
    const T* vy = vel;
    const T* vx = vel + (h + 1) * w;
    const T ndt = -dt;
    PAR_ALL for (idx y = 0; y < h; ++y)
        for (idx x = 0; x < w; ++x) {
            const T vcx = (vx[y * (w + 1) + x] + vx[y * (w + 1) + x + 1]) / T(2);
            const T vcy = (vy[y * w + x] + vy[(y + 1) * w + x]) / T(2);
            const T ppx = ((T)x + T(0.5)) + ndt * vcx;  // integrate_euler, dec_fluid.rs:169-171
            const T ppy = ((T)y + T(0.5)) + ndt * vcy;
            idx ix, iy;
            T u, v;
            cell_coord(ppx, w, &ix, &u);
            cell_coord(ppy, h, &iy, &v);
            dst[y * w + x] = bilinear(q[iy * w + ix], q[iy * w + ix + 1], q[(iy + 1) * w + ix],
                                      q[(iy + 1) * w + ix + 1], u, v);
        }
}

// examples/dec_fluid.rs:213-291
template <class T> void advect_mac_2d(T* dst, const T* src, T dt, const T* vel, idx h, idx w) {
    const T* qy = src;
    const T* qx = src + (h + 1) * w;
    T* dy = dst;
    T* dx = dst + (h + 1) * w;
    const T* vy = vel;
    const T* vx = vel + (h + 1) * w;
    const T ndt = -dt;
    const idx wx = w + 1;  // qx / vx row length
    // x faces: qx dims (h, w+1)
    PAR_ALL for (idx y = 0; y < h; ++y)
        for (idx x = 0; x < w + 1; ++x) {
            const idx xc = std::min(x, w - 1), xm = x > 0 ? x - 1 : 0;
            const T velx = vx[y * wx + x];
            const T vely = (vy[y * w + xc] + vy[(y + 1) * w + xc] + vy[y * w + xm] + vy[(y + 1) * w + xm]) / T(4);
            const T ppx = ((T)x + T(0)) + ndt * velx;
            const T ppy = ((T)y + T(0.5)) + ndt * vely;
            idx x0, x1, y0, y1;
            T s, t;
            face_coord(ppx, T(0), w + 1, &x0, &x1, &s);
            face_coord(ppy, T(0.5), h, &y0, &y1, &t);
            dx[y * wx + x] = bilinear(qx[y0 * wx + x0], qx[y0 * wx + x1], qx[y1 * wx + x0], qx[y1 * wx + x1], s, t);
        }
    // y faces: qy dims (h+1, w)
    PAR_ALL for (idx y = 0; y < h + 1; ++y)
        for (idx x = 0; x < w; ++x) {
            const idx yc = std::min(y, h - 1), ym = y > 0 ? y - 1 : 0;
            const T velx = (vx[yc * wx + x] + vx[yc * wx + x + 1] + vx[ym * wx + x] + vx[ym * wx + x + 1]) / T(4);
            const T vely = vy[y * w + x];
            const T ppx = ((T)x + T(0.5)) + ndt * velx;
            const T ppy = ((T)y + T(0)) + ndt * vely;
            idx x0, x1, y0, y1;
            T s, t;
            face_coord(ppx, T(0.5), w, &x0, &x1, &s);
            face_coord(ppy, T(0), h + 1, &y0, &y1, &t);
            dy[y * w + x] = bilinear(qy[y0 * w + x0], qy[y0 * w + x1], qy[y1 * w + x0], qy[y1 * w + x1], s, t);
        }
}

// ---------------------------------------------------------------------------
// 3D extension (no reference counterpart; domain/grid.rs:17-20 has only the
// struct).  Cells (d,h,w); faces = [vz (d+1)hw | vy d(h+1)w | vx dh(w+1)].
struct D3 {
    idx d, h, w;
    idx nc() const { return d * h * w; }
    idx nz() const { return (d + 1) * h * w; }
    idx ny() const { return d * (h + 1) * w; }
    idx nx() const { return d * h * (w + 1); }
    idx nf() const { return nz() + ny() + nx(); }
    idx c(idx z, idx y, idx x) const { return (z * h + y) * w + x; }
    idx fz(idx z, idx y, idx x) const { return (z * h + y) * w + x; }
    idx fy(idx z, idx y, idx x) const { return nz() + (z * (h + 1) + y) * w + x; }
    idx fx(idx z, idx y, idx x) const { return nz() + ny() + (z * h + y) * (w + 1) + x; }
};

// Negative gradient on interior faces (the 3D analogue of grid.rs:318-334):
// e = p[lo] - p[hi]; boundary faces untouched.
template <class T> void gradient_dual_3d(T* e, const T* p, const D3& g) {
    PAR_REF for (idx z = 0; z < g.d + 1; ++z) {
        if (z == 0 || z == g.d) continue;
        for (idx y = 0; y < g.h; ++y)
            for (idx x = 0; x < g.w; ++x) e[g.fz(z, y, x)] = -(p[g.c(z, y, x)] - p[g.c(z - 1, y, x)]);
    }
    PAR_REF for (idx z = 0; z < g.d; ++z)
        for (idx y = 1; y < g.h; ++y)
            for (idx x = 0; x < g.w; ++x) e[g.fy(z, y, x)] = -(p[g.c(z, y, x)] - p[g.c(z, y - 1, x)]);
    PAR_REF for (idx z = 0; z < g.d; ++z)
        for (idx y = 0; y < g.h; ++y)
            for (idx x = 1; x < g.w; ++x) e[g.fx(z, y, x)] = p[g.c(z, y, x - 1)] - p[g.c(z, y, x)];
}

// 3D divergence-like sum, fixed order extending the 2D one:
// ((((ey_hi - ey_lo) - ex_lo) + ex_hi) - ez_lo) + ez_hi
template <class T> inline T div_sum3(T ey_lo, T ey_hi, T ex_lo, T ex_hi, T ez_lo, T ez_hi) {
    return ((((ey_hi - ey_lo) - ex_lo) + ex_hi) - ez_lo) + ez_hi;
}

template <class T> void div_faces_3d(T* out, const T* e, const D3& g) {
    PAR_REF for (idx z = 0; z < g.d; ++z)
        for (idx y = 0; y < g.h; ++y)
            for (idx x = 0; x < g.w; ++x)
                out[g.c(z, y, x)] = div_sum3(e[g.fy(z, y, x)], e[g.fy(z, y + 1, x)], e[g.fx(z, y, x)],
                                             e[g.fx(z, y, x + 1)], e[g.fz(z, y, x)], e[g.fz(z + 1, y, x)]);
}

template <class T>
void laplacian_3d(T* out, const T* p, T dt, const uint8_t* face_solid, const D3& g, T* tmp_face) {
    gradient_dual_3d(tmp_face, p, g);
    mask_faces(tmp_face, face_solid, g.nf());
    div_faces_3d(out, tmp_face, g);
    PAR_ALL for (idx i = 0; i < g.nc(); ++i) out[i] = out[i] * dt;
}

template <class T> void divergence_rhs_3d(T* b, const T* vel, const uint8_t* face_solid, const D3& g, T* tmp_face) {
    std::memcpy(tmp_face, vel, sizeof(T) * g.nf());
    mask_faces(tmp_face, face_solid, g.nf());
    div_faces_3d(b, tmp_face, g);
    PAR_ALL for (idx i = 0; i < g.nc(); ++i) b[i] = -b[i];
}

template <class T> void advect_3d(T* dst, const T* q, T dt, const T* vel, const D3& g) {
    const T ndt = -dt;
    const idx w = g.w, hw = g.h * g.w;
    PAR_ALL for (idx z = 0; z < g.d; ++z)
        for (idx y = 0; y < g.h; ++y)
            for (idx x = 0; x < g.w; ++x) {
                const T vcx = (vel[g.fx(z, y, x)] + vel[g.fx(z, y, x + 1)]) / T(2);
                const T vcy = (vel[g.fy(z, y, x)] + vel[g.fy(z, y + 1, x)]) / T(2);
                const T vcz = (vel[g.fz(z, y, x)] + vel[g.fz(z + 1, y, x)]) / T(2);
                const T ppx = ((T)x + T(0.5)) + ndt * vcx;
                const T ppy = ((T)y + T(0.5)) + ndt * vcy;
                const T ppz = ((T)z + T(0.5)) + ndt * vcz;
                idx ix, iy, iz;
                T s, t, u;
                cell_coord(ppx, g.w, &ix, &s);
                cell_coord(ppy, g.h, &iy, &t);
                cell_coord(ppz, g.d, &iz, &u);
                const T* q0 = q + iz * hw + iy * w + ix;
                const T* q1 = q0 + hw;
                dst[g.c(z, y, x)] = trilinear(q0[0], q0[1], q0[w], q0[w + 1], q1[0], q1[1], q1[w], q1[w + 1], s, t, u);
            }
}

// Trilinear sample of a face array with dims (nz_, ny_, nx_) at face offsets.
template <class T>
inline T sample_face(const T* q, idx nz_, idx ny_, idx nx_, T ppx, T offx, T ppy, T offy, T ppz, T offz) {
    idx x0, x1, y0, y1, z0, z1;
    T s, t, u;
    face_coord(ppx, offx, nx_, &x0, &x1, &s);
    face_coord(ppy, offy, ny_, &y0, &y1, &t);
    face_coord(ppz, offz, nz_, &z0, &z1, &u);
#define Q(zz, yy, xx) q[((zz) * ny_ + (yy)) * nx_ + (xx)]
    return trilinear(Q(z0, y0, x0), Q(z0, y0, x1), Q(z0, y1, x0), Q(z0, y1, x1), Q(z1, y0, x0), Q(z1, y0, x1),
                     Q(z1, y1, x0), Q(z1, y1, x1), s, t, u);
#undef Q
}

template <class T> void advect_mac_3d(T* dst, const T* src, T dt, const T* vel, const D3& g) {
    const T ndt = -dt;
    const idx d = g.d, h = g.h, w = g.w;
    const T* qz = src;
    const T* qy = src + g.nz();
    const T* qx = src + g.nz() + g.ny();
    // x faces (d, h, w+1)
    PAR_ALL for (idx z = 0; z < d; ++z)
        for (idx y = 0; y < h; ++y)
            for (idx x = 0; x < w + 1; ++x) {
                const idx xc = std::min(x, w - 1), xm = x > 0 ? x - 1 : 0;
                const T vx_ = vel[g.fx(z, y, x)];
                const T vy_ = (vel[g.fy(z, y, xc)] + vel[g.fy(z, y + 1, xc)] + vel[g.fy(z, y, xm)] +
                               vel[g.fy(z, y + 1, xm)]) / T(4);
                const T vz_ = (vel[g.fz(z, y, xc)] + vel[g.fz(z + 1, y, xc)] + vel[g.fz(z, y, xm)] +
                               vel[g.fz(z + 1, y, xm)]) / T(4);
                const T ppx = ((T)x + T(0)) + ndt * vx_;
                const T ppy = ((T)y + T(0.5)) + ndt * vy_;
                const T ppz = ((T)z + T(0.5)) + ndt * vz_;
                dst[g.fx(z, y, x)] = sample_face(qx, d, h, w + 1, ppx, T(0), ppy, T(0.5), ppz, T(0.5));
            }
    // y faces (d, h+1, w)
    PAR_ALL for (idx z = 0; z < d; ++z)
        for (idx y = 0; y < h + 1; ++y)
            for (idx x = 0; x < w; ++x) {
                const idx yc = std::min(y, h - 1), ym = y > 0 ? y - 1 : 0;
                const T vx_ = (vel[g.fx(z, yc, x)] + vel[g.fx(z, yc, x + 1)] + vel[g.fx(z, ym, x)] +
                               vel[g.fx(z, ym, x + 1)]) / T(4);
                const T vy_ = vel[g.fy(z, y, x)];
                const T vz_ = (vel[g.fz(z, yc, x)] + vel[g.fz(z + 1, yc, x)] + vel[g.fz(z, ym, x)] +
                               vel[g.fz(z + 1, ym, x)]) / T(4);
                const T ppx = ((T)x + T(0.5)) + ndt * vx_;
                const T ppy = ((T)y + T(0)) + ndt * vy_;
                const T ppz = ((T)z + T(0.5)) + ndt * vz_;
                dst[g.fy(z, y, x)] = sample_face(qy, d, h + 1, w, ppx, T(0.5), ppy, T(0), ppz, T(0.5));
            }
    // z faces (d+1, h, w)
    PAR_ALL for (idx z = 0; z < d + 1; ++z)
        for (idx y = 0; y < h; ++y)
            for (idx x = 0; x < w; ++x) {
                const idx zc = std::min(z, d - 1), zm = z > 0 ? z - 1 : 0;
                const T vx_ = (vel[g.fx(zc, y, x)] + vel[g.fx(zc, y, x + 1)] + vel[g.fx(zm, y, x)] +
                               vel[g.fx(zm, y, x + 1)]) / T(4);
                const T vy_ = (vel[g.fy(zc, y, x)] + vel[g.fy(zc, y + 1, x)] + vel[g.fy(zm, y, x)] +
                               vel[g.fy(zm, y + 1, x)]) / T(4);
                const T vz_ = vel[g.fz(z, y, x)];
                const T ppx = ((T)x + T(0.5)) + ndt * vx_;
                const T ppy = ((T)y + T(0.5)) + ndt * vy_;
                const T ppz = ((T)z + T(0)) + ndt * vz_;
                dst[g.fz(z, y, x)] = sample_face(qz, d + 1, h, w, ppx, T(0.5), ppy, T(0.5), ppz, T(0));
            }
}

// ---------------------------------------------------------------------------
// Dimension-generic helpers (2D = d 1 with the 2D layout handled separately).
struct Shape {
    int nd;
    idx d, h, w;
    idx nc() const { return d * h * w; }
    idx nf() const { return nd == 2 ? (h + 1) * w + h * (w + 1) : D3{d, h, w}.nf(); }
};

template <class T>
void apply_laplacian(T* out, const T* p, T dt, const uint8_t* fs, const Shape& s, std::vector<T>& tc,
                     std::vector<T>& tf, std::vector<T>& tf2) {
    if (s.nd == 2) {
        laplacian_closure_2d(out, p, dt, fs, s.h, s.w, tc.data(), tf.data(), tf2.data());
    } else {
        laplacian_3d(out, p, dt, fs, D3{s.d, s.h, s.w}, tf.data());
    }
}

// Parallel reductions of the all-loops mode: thread t of nt reduces the
// contiguous slice [n t / nt, n (t + 1) / nt) and the slices' results are
// combined in thread order, so a run is deterministic for a thread count.
inline bool par_reduce(idx n) { return g_all && g_threads > 1 && n >= ((idx)1 << 16); }

template <class T, class F> void slices(idx n, std::vector<T>& part, F f) {
    part.assign(g_threads, T(0));
#ifdef _OPENMP
#pragma omp parallel num_threads(g_threads)
    {
        const int t = omp_get_thread_num(), nt = omp_get_num_threads();
        part[t] = f(n * t / nt, n * (t + 1) / nt);
    }
#else
    part[0] = f(0, n);
#endif
}

// math/linear_view.rs:16-30 (NaN never replaces the running max)
template <class T> T norm_max_range(const T* a, idx lo, idx hi) {
    T m = T(0);
    for (idx i = lo; i < hi; ++i) {
        const T x = a[i];
        m = x > m ? x : (-x > m ? -x : m);
    }
    return m;
}

template <class T> T norm_max(const T* a, idx n) {
    if (!par_reduce(n)) return norm_max_range(a, 0, n);
    std::vector<T> part;
    slices(n, part, [&](idx lo, idx hi) { return norm_max_range(a, lo, hi); });
    T m = T(0);
    for (T v : part) m = v > m ? v : m;
    return m;
}

// math/linear_view.rs:12-14 (ndarray 1-D dot; summation order of ndarray 0.10
// is not pinned: a serial sum in T is used, per slice in the all-loops mode).
template <class T> T dot(const T* a, const T* b, idx n) {
    if (g_dot64) {
        auto f = [&](idx lo, idx hi) {
            double s = 0.0;
            for (idx i = lo; i < hi; ++i) s += (double)a[i] * (double)b[i];
            return s;
        };
        if (!par_reduce(n)) return (T)f(0, n);
        std::vector<double> part;
        slices(n, part, f);
        double s = 0.0;
        for (double v : part) s += v;
        return (T)s;
    }
    auto f = [&](idx lo, idx hi) {
        T s = T(0);
        for (idx i = lo; i < hi; ++i) s = s + a[i] * b[i];
        return s;
    };
    if (!par_reduce(n)) return f(0, n);
    std::vector<T> part;
    slices(n, part, f);
    T s = T(0);
    for (T v : part) s = s + v;
    return s;
}

// Number of open (interior, not solid) faces of each cell: the diagonal of
// the masked Laplacian divided by dt.  Used by the Jacobi preconditioner
// (extension: the reference's `Preconditioner` trait, pcg.rs:4-6, has only
// the identity impl).
template <class T> void open_face_count(std::vector<T>& cnt, const uint8_t* fs, const Shape& s) {
    cnt.assign(s.nc(), T(0));
    if (s.nd == 2) {
        const idx h = s.h, w = s.w, n0 = (h + 1) * w;
        for (idx y = 0; y < h; ++y)
            for (idx x = 0; x < w; ++x) {
                int c = 0;
                if (y > 0 && !(fs && fs[y * w + x])) ++c;
                if (y < h - 1 && !(fs && fs[(y + 1) * w + x])) ++c;
                if (x > 0 && !(fs && fs[n0 + y * (w + 1) + x])) ++c;
                if (x < w - 1 && !(fs && fs[n0 + y * (w + 1) + x + 1])) ++c;
                cnt[y * w + x] = (T)c;
            }
    } else {
        D3 g{s.d, s.h, s.w};
        for (idx z = 0; z < g.d; ++z)
            for (idx y = 0; y < g.h; ++y)
                for (idx x = 0; x < g.w; ++x) {
                    int c = 0;
                    if (z > 0 && !(fs && fs[g.fz(z, y, x)])) ++c;
                    if (z < g.d - 1 && !(fs && fs[g.fz(z + 1, y, x)])) ++c;
                    if (y > 0 && !(fs && fs[g.fy(z, y, x)])) ++c;
                    if (y < g.h - 1 && !(fs && fs[g.fy(z, y + 1, x)])) ++c;
                    if (x > 0 && !(fs && fs[g.fx(z, y, x)])) ++c;
                    if (x < g.w - 1 && !(fs && fs[g.fx(z, y, x + 1)])) ++c;
                    cnt[g.c(z, y, x)] = (T)c;
                }
    }
}

// pcg.rs:14-82, operator = the masked Laplacian closure, preconditioner
// 0 = identity `()` (pcg.rs:8-12), 1 = Jacobi (extension).
// Returns the number of operator applications; *res = last ||r||inf.
template <class T>
long pcg(int precond, T* x, const T* b, long max_iter, T threshold, T* r, T* aux, T* search, T dt,
         const uint8_t* fs, const Shape& s, T* res_out, int* converged) {
    const idx n = s.nc();
    std::vector<T> tc(n), tf(s.nf(), T(0)), tf2(s.nf(), T(0)), diag;
    if (precond == 1) {
        open_face_count(diag, fs, s);
        for (auto& v : diag) v = v * dt;
    }
    auto apply_precond = [&](T* dst, const T* src) {
        if (precond == 1) {
            PAR_ALL for (idx i = 0; i < n; ++i) dst[i] = diag[i] > T(0) ? src[i] / diag[i] : T(0);
        } else {
            PAR_ALL for (idx i = 0; i < n; ++i) dst[i] = src[i];
        }
    };
    PAR_ALL for (idx i = 0; i < n; ++i) x[i] = T(0);
    *converged = 0;
    const T bmax = norm_max(b, n);
    *res_out = bmax;
    if (bmax < threshold) {  // pcg.rs:35-38
        *converged = 1;
        return 0;
    }
    PAR_ALL for (idx i = 0; i < n; ++i) r[i] = b[i];
    apply_precond(aux, r);
    PAR_ALL for (idx i = 0; i < n; ++i) search[i] = aux[i];
    T sigma = dot(aux, r, n);
    long it = 0;
    for (long i = 0; i < max_iter; ++i) {
        apply_laplacian(aux, search, dt, fs, s, tc, tf, tf2);  // a(&mut auxiliary, search)
        ++it;
        const T alpha = sigma / dot(aux, search, n);
        PAR_ALL for (idx k = 0; k < n; ++k) x[k] = x[k] + alpha * search[k];
        const T nalpha = -alpha;
        PAR_ALL for (idx k = 0; k < n; ++k) r[k] = r[k] + nalpha * aux[k];
        const T err = norm_max(r, n);
        *res_out = err;
        if (err < threshold) {
            *converged = 1;
            break;
        }
        apply_precond(aux, r);
        const T sigma_new = dot(aux, r, n);
        const T beta = sigma_new / sigma;
        PAR_ALL for (idx k = 0; k < n; ++k) search[k] = aux[k] + beta * search[k];
        sigma = sigma_new;
    }
    return it;
}

// Wall step of examples/dec_fluid.rs:128-141: zero the domain-boundary
// faces (vx at x=0,w; vy at y=0,h; in 3D also vz at z=0,d).
template <class T> void walls(T* vel, const Shape& s) {
    if (s.nd == 2) {
        const idx h = s.h, w = s.w;
        T* vy = vel;
        T* vx = vel + (h + 1) * w;
        for (idx y = 0; y < h; ++y) {
            vx[y * (w + 1) + 0] = T(0);
            vx[y * (w + 1) + w] = T(0);
        }
        for (idx x = 0; x < w; ++x) {
            vy[0 * w + x] = T(0);
            vy[h * w + x] = T(0);
        }
    } else {
        D3 g{s.d, s.h, s.w};
        for (idx z = 0; z < g.d; ++z)
            for (idx y = 0; y < g.h; ++y) {
                vel[g.fx(z, y, 0)] = T(0);
                vel[g.fx(z, y, g.w)] = T(0);
            }
        for (idx z = 0; z < g.d; ++z)
            for (idx x = 0; x < g.w; ++x) {
                vel[g.fy(z, 0, x)] = T(0);
                vel[g.fy(z, g.h, x)] = T(0);
            }
        for (idx y = 0; y < g.h; ++y)
            for (idx x = 0; x < g.w; ++x) {
                vel[g.fz(0, y, x)] = T(0);
                vel[g.fz(g.d, y, x)] = T(0);
            }
    }
}

// examples/dec_fluid.rs:123-141 (+ optional re-zeroing of solid faces, an
// extension): vel += dt * d0dual(p) on interior faces, then walls.
template <class T> void project(T* vel, const T* p, T dt, const uint8_t* fs, int zero_solid, const Shape& s) {
    std::vector<T> e(s.nf(), T(0));
    if (s.nd == 2) {
        derivative_0_dual_2d(e.data(), p, s.h, s.w);
    } else {
        gradient_dual_3d(e.data(), p, D3{s.d, s.h, s.w});
    }
    const idx nf = s.nf();
    PAR_ALL for (idx i = 0; i < nf; ++i) vel[i] = vel[i] + dt * e[i];  // scaled_add
    walls(vel, s);
    if (zero_solid) mask_faces(vel, fs, nf);
}

}  // namespace

// ===========================================================================
// C ABI for the test-suite (ctypes).  Shapes: nd = 2 uses (h, w) and the 2D
// reference layout; nd = 3 uses (d, h, w).

struct pgo_step_params {
    double dt;
    double buoyancy;             // 0 = off (extension)
    int source_enabled;          // dec_fluid.rs:48-57
    long source_lo[3], source_hi[3];  // (z, y, x) half-open cell box
    double source_density, source_vy;
    const void* source_field;    // optional cell field: density = max(density, field)
    int walls_after_advect;      // extension (0 in the reference)
    int zero_solid_after_project;  // extension (0 in the reference)
    int precond;                 // 0 identity, 1 Jacobi
    int rel_stop;                // 0: abs threshold (pcg.rs:58-60); 1: threshold = rel_tol * ||b||inf
    double threshold, rel_tol;
    long max_iter;
    int advect_scheme;           // density: 0 first order (reference), 1 MacCormack, 2 BFECC (extensions)
    int density_bf16;            // extension: density stored in bfloat16 (rounded after every write)
};

// Round to the nearest bfloat16 (ties to even) and back: the storage rule of
// the BF16 density.  NaN stays NaN, infinities stay.
static float round_bf16(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) {
        if (u & 0x007fffffu) u |= 0x00400000u;
    } else {
        u += 0x7fffu + ((u >> 16) & 1u);
    }
    u &= 0xffff0000u;
    std::memcpy(&x, &u, 4);
    return x;
}
static double round_bf16(double x) { return (double)round_bf16((float)x); }

template <class T> static void advect2(T* dst, const T* q, T dt, const T* vel, int scheme, const Shape& s);

struct pgo_step_stats {
    long iterations;
    double residual, bmax;
    int converged;
    double t_total, t_solve;  // wall seconds: whole step, and the pcg call
};

namespace {

template <class T> void buoyancy_apply(T* vel, const T* rho, double dt, double beta, const Shape& s) {
    const T coef = (T)(dt * beta);
    if (s.nd == 2) {
        const idx h = s.h, w = s.w;
        for (idx y = 1; y < h; ++y)
            for (idx x = 0; x < w; ++x)
                vel[y * w + x] = vel[y * w + x] + coef * (T(0.5) * (rho[(y - 1) * w + x] + rho[y * w + x]));
    } else {
        D3 g{s.d, s.h, s.w};
        for (idx z = 0; z < g.d; ++z)
            for (idx y = 1; y < g.h; ++y)
                for (idx x = 0; x < g.w; ++x) {
                    const idx f = g.fy(z, y, x);
                    vel[f] = vel[f] + coef * (T(0.5) * (rho[g.c(z, y - 1, x)] + rho[g.c(z, y, x)]));
                }
    }
}

// vy face with the same (z, y, x) index as a cell (dec_fluid.rs:54 writes vy[(y, x)]).
inline idx vy_face_index(const Shape& s, idx z, idx y, idx x) {
    if (s.nd == 2) return y * s.w + x;
    return D3{s.d, s.h, s.w}.fy(z, y, x);
}

// One step of examples/dec_fluid.rs:46-141 (PNG dump omitted), with the
// extension switches of pgo_step_params.
template <class T>
void step(const Shape& s, T* vel, T* density, T* pressure, const uint8_t* fs, const pgo_step_params& prm,
          pgo_step_stats* st) {
    const auto t0 = std::chrono::steady_clock::now();
    const idx nc = s.nc(), nf = s.nf();
    const T dt = (T)prm.dt;
    // inflow
    if (prm.source_enabled) {
        for (idx z = prm.source_lo[0]; z < prm.source_hi[0]; ++z)
            for (idx y = prm.source_lo[1]; y < prm.source_hi[1]; ++y)
                for (idx x = prm.source_lo[2]; x < prm.source_hi[2]; ++x) {
                    density[(z * s.h + y) * s.w + x] =
                        prm.density_bf16 ? (T)round_bf16((T)prm.source_density) : (T)prm.source_density;
                    vel[vy_face_index(s, z, y, x)] = (T)prm.source_vy;
                }
    }
    if (prm.source_field) {
        const T* sf = (const T*)prm.source_field;
        for (idx i = 0; i < nc; ++i) density[i] = rmax(density[i], sf[i]);
        if (prm.density_bf16)
            for (idx i = 0; i < nc; ++i) density[i] = round_bf16(density[i]);
    }
    std::vector<T> temp(nc), vel_temp(nf);
    if (s.nd == 2) {
        advect_2d(temp.data(), density, dt, vel, s.h, s.w);
        advect_mac_2d(vel_temp.data(), vel, dt, vel, s.h, s.w);
    } else {
        D3 g{s.d, s.h, s.w};
        advect_3d(temp.data(), density, dt, vel, g);
        advect_mac_3d(vel_temp.data(), vel, dt, vel, g);
    }
    if (prm.advect_scheme) advect2(temp.data(), density, dt, vel, prm.advect_scheme, s);
    if (prm.density_bf16)
        for (idx i = 0; i < nc; ++i) temp[i] = round_bf16(temp[i]);
    std::memcpy(density, temp.data(), sizeof(T) * nc);
    std::memcpy(vel, vel_temp.data(), sizeof(T) * nf);
    if (prm.walls_after_advect) walls(vel, s);
    if (prm.buoyancy != 0.0) buoyancy_apply(vel, density, prm.dt, prm.buoyancy, s);
    // -div
    std::vector<T> b(nc);
    if (s.nd == 2) {
        divergence_rhs_2d(b.data(), vel, fs, s.h, s.w, vel_temp.data());
    } else {
        divergence_rhs_3d(b.data(), vel, fs, D3{s.d, s.h, s.w}, vel_temp.data());
    }
    std::vector<T> r(nc), aux(nc), search(nc);
    T thr = (T)prm.threshold;
    if (prm.rel_stop) thr = (T)(prm.rel_tol * (double)norm_max(b.data(), nc));
    T res;
    int conv;
    const auto t1 = std::chrono::steady_clock::now();
    long it = pcg(prm.precond, pressure, b.data(), prm.max_iter, thr, r.data(), aux.data(), search.data(), dt, fs, s,
                  &res, &conv);
    const auto t2 = std::chrono::steady_clock::now();
    project(vel, pressure, dt, fs, prm.zero_solid_after_project, s);
    const auto t3 = std::chrono::steady_clock::now();
    if (st) {
        st->t_total = std::chrono::duration<double>(t3 - t0).count();
        st->t_solve = std::chrono::duration<double>(t2 - t1).count();
        st->iterations = it;
        st->residual = (double)res;
        st->bmax = (double)norm_max(b.data(), nc);
        st->converged = conv;
    }
}

inline Shape shape2(long h, long w) { return Shape{2, 1, h, w}; }
inline Shape shape_of(int nd, long d, long h, long w) { return nd == 2 ? shape2(h, w) : Shape{3, d, h, w}; }

}  // namespace

#define PGO_EXPORT extern "C" __attribute__((visibility("default")))

PGO_EXPORT void pgo_set_threads(int n, int all) {
    g_threads = n < 1 ? 1 : n;
    g_all = all;
}

// 1: dot products accumulate in double (as the CUDA library does); 0: in T.
PGO_EXPORT void pgo_set_dot64(int on) { g_dot64 = on; }

PGO_EXPORT long pgo_num_faces(int nd, long d, long h, long w) { return shape_of(nd, d, h, w).nf(); }

#define PGO_BOTH(MACRO) MACRO(float, f32) MACRO(double, f64)

#define PGO_DEFS(T, SFX)                                                                                          \
    PGO_EXPORT void pgo_hodge_1_dual_##SFX(T* primal, const T* dual, long h, long w) {                          \
        hodge_1_dual_2d(primal, dual, h, w);                                                                     \
    }                                                                                                            \
    PGO_EXPORT void pgo_hodge_1_primal_##SFX(T* dual, const T* primal, long h, long w) {                        \
        hodge_1_primal_2d(dual, primal, h, w);                                                                   \
    }                                                                                                            \
    PGO_EXPORT void pgo_hodge_2_primal_##SFX(T* dual, const T* primal, long n) { hodge_2_primal(dual, primal, n); } \
    PGO_EXPORT void pgo_derivative_1_primal_##SFX(T* faces, const T* edges, long h, long w) {                   \
        derivative_1_primal_2d(faces, edges, h, w);                                                              \
    }                                                                                                            \
    PGO_EXPORT void pgo_derivative_0_dual_##SFX(T* edges, const T* faces, int nd, long d, long h, long w) {     \
        if (nd == 2)                                                                                             \
            derivative_0_dual_2d(edges, faces, h, w);                                                            \
        else                                                                                                     \
            gradient_dual_3d(edges, faces, D3{d, h, w});                                                         \
    }                                                                                                            \
    PGO_EXPORT void pgo_mask_faces_##SFX(T* edges, const uint8_t* solid, long nf) { mask_faces(edges, solid, nf); } \
    PGO_EXPORT void pgo_laplacian_##SFX(T* out, const T* p, double dt, const uint8_t* fs, int nd, long d, long h,   \
                                        long w) {                                                                \
        Shape s = shape_of(nd, d, h, w);                                                                         \
        std::vector<T> tc(s.nc()), tf(s.nf(), T(0)), tf2(s.nf(), T(0));                                          \
        apply_laplacian(out, p, (T)dt, fs, s, tc, tf, tf2);                                                      \
    }                                                                                                            \
    PGO_EXPORT void pgo_divergence_rhs_##SFX(T* b, const T* vel, const uint8_t* fs, int nd, long d, long h, long w) { \
        Shape s = shape_of(nd, d, h, w);                                                                         \
        std::vector<T> tf(s.nf());                                                                               \
        if (nd == 2)                                                                                             \
            divergence_rhs_2d(b, vel, fs, h, w, tf.data());                                                      \
        else                                                                                                     \
            divergence_rhs_3d(b, vel, fs, D3{d, h, w}, tf.data());                                               \
    }                                                                                                            \
    PGO_EXPORT void pgo_advect_##SFX(T* dst, const T* src, double dt, const T* vel, int nd, long d, long h, long w) { \
        if (nd == 2)                                                                                             \
            advect_2d(dst, src, (T)dt, vel, h, w);                                                               \
        else                                                                                                     \
            advect_3d(dst, src, (T)dt, vel, D3{d, h, w});                                                        \
    }                                                                                                            \
    PGO_EXPORT void pgo_advect_mac_##SFX(T* dst, const T* src, double dt, const T* vel, int nd, long d, long h,     \
                                         long w) {                                                               \
        if (nd == 2)                                                                                             \
            advect_mac_2d(dst, src, (T)dt, vel, h, w);                                                           \
        else                                                                                                     \
            advect_mac_3d(dst, src, (T)dt, vel, D3{d, h, w});                                                    \
    }                                                                                                            \
    PGO_EXPORT void pgo_project_##SFX(T* vel, const T* p, double dt, const uint8_t* fs, int zero_solid, int nd,     \
                                      long d, long h, long w) {                                                  \
        project(vel, p, (T)dt, fs, zero_solid, shape_of(nd, d, h, w));                                           \
    }                                                                                                            \
    PGO_EXPORT long pgo_pcg_##SFX(int precond, T* x, const T* b, long max_iter, double threshold, T* r, T* aux,     \
                                  T* search, double dt, const uint8_t* fs, int nd, long d, long h, long w,         \
                                  double* res, int* converged) {                                                 \
        T rr;                                                                                                    \
        long it = pcg(precond, x, b, max_iter, (T)threshold, r, aux, search, (T)dt, fs, shape_of(nd, d, h, w),   \
                      &rr, converged);                                                                           \
        *res = (double)rr;                                                                                       \
        return it;                                                                                               \
    }                                                                                                            \
    PGO_EXPORT void pgo_walls_##SFX(T* vel, int nd, long d, long h, long w) { walls(vel, shape_of(nd, d, h, w)); } \
    PGO_EXPORT double pgo_norm_max_##SFX(const T* a, long n) { return (double)norm_max(a, n); }                  \
    PGO_EXPORT void pgo_step_##SFX(T* vel, T* density, T* pressure, const uint8_t* fs, const pgo_step_params* prm,  \
                                   pgo_step_stats* st, int nd, long d, long h, long w) {                         \
        step(shape_of(nd, d, h, w), vel, density, pressure, fs, *prm, st);                                       \
    }                                                                                                            \
    PGO_EXPORT void pgo_open_face_count_##SFX(T* cnt, const uint8_t* fs, int nd, long d, long h, long w) {       \
        std::vector<T> c;                                                                                        \
        Shape s = shape_of(nd, d, h, w);                                                                         \
        open_face_count(c, fs, s);                                                                               \
        std::memcpy(cnt, c.data(), sizeof(T) * s.nc());                                                          \
    }

PGO_BOTH(PGO_DEFS)

// ---------------------------------------------------------------------------
// Second-order limited advection of a cell scalar (extension; no reference
// behaviour): MacCormack (scheme 1) and BFECC (scheme 2) built from the
// first-order advect above; where the result leaves [min, max] of the
// corner values the first-order sample of q interpolated, it falls back to
// that sample.
template <class T>
static void corner_range(const T* q, const T* vel, T dt, const Shape& s, idx i, T* lo, T* hi) {
    const T ndt = -dt;
    if (s.nd == 2) {
        const idx h = s.h, w = s.w;
        const T* vy = vel;
        const T* vx = vel + (h + 1) * w;
        const idx y = i / w, x = i - y * w;
        const T vcx = (vx[y * (w + 1) + x] + vx[y * (w + 1) + x + 1]) / T(2);
        const T vcy = (vy[y * w + x] + vy[(y + 1) * w + x]) / T(2);
        idx ix, iy;
        T u, v;
        cell_coord(((T)x + T(0.5)) + ndt * vcx, w, &ix, &u);
        cell_coord(((T)y + T(0.5)) + ndt * vcy, h, &iy, &v);
        const T* q0 = q + iy * w + ix;
        *lo = std::fmin(std::fmin(q0[0], q0[1]), std::fmin(q0[w], q0[w + 1]));
        *hi = std::fmax(std::fmax(q0[0], q0[1]), std::fmax(q0[w], q0[w + 1]));
        return;
    }
    D3 g{s.d, s.h, s.w};
    const idx w = g.w, hw = g.h * g.w;
    const idx zy = i / w, x = i - zy * w, z = zy / g.h, y = zy - z * g.h;
    const T vcx = (vel[g.fx(z, y, x)] + vel[g.fx(z, y, x + 1)]) / T(2);
    const T vcy = (vel[g.fy(z, y, x)] + vel[g.fy(z, y + 1, x)]) / T(2);
    const T vcz = (vel[g.fz(z, y, x)] + vel[g.fz(z + 1, y, x)]) / T(2);
    idx ix, iy, iz;
    T a, b, c;
    cell_coord(((T)x + T(0.5)) + ndt * vcx, g.w, &ix, &a);
    cell_coord(((T)y + T(0.5)) + ndt * vcy, g.h, &iy, &b);
    cell_coord(((T)z + T(0.5)) + ndt * vcz, g.d, &iz, &c);
    const T* q0 = q + iz * hw + iy * w + ix;
    const T* q1 = q0 + hw;
    *lo = std::fmin(std::fmin(std::fmin(q0[0], q0[1]), std::fmin(q0[w], q0[w + 1])),
                    std::fmin(std::fmin(q1[0], q1[1]), std::fmin(q1[w], q1[w + 1])));
    *hi = std::fmax(std::fmax(std::fmax(q0[0], q0[1]), std::fmax(q0[w], q0[w + 1])),
                    std::fmax(std::fmax(q1[0], q1[1]), std::fmax(q1[w], q1[w + 1])));
}

template <class T> static void advect_any(T* dst, const T* src, T dt, const T* vel, const Shape& s) {
    if (s.nd == 2) advect_2d(dst, src, dt, vel, s.h, s.w);
    else advect_3d(dst, src, dt, vel, D3{s.d, s.h, s.w});
}

template <class T> static void advect2(T* dst, const T* q, T dt, const T* vel, int scheme, const Shape& s) {
    const idx n = s.nc();
    std::vector<T> q1(n), q2(n);
    advect_any(q1.data(), q, dt, vel, s);
    advect_any(q2.data(), q1.data(), -dt, vel, s);
    if (scheme == 1) {
        for (idx i = 0; i < n; ++i) {
            T lo, hi;
            corner_range(q, vel, dt, s, i, &lo, &hi);
            const T v = q1[i] + T(0.5) * (q[i] - q2[i]);
            dst[i] = (v < lo || v > hi || v != v) ? q1[i] : v;
        }
    } else {
        for (idx i = 0; i < n; ++i) q2[i] = q[i] + T(0.5) * (q[i] - q2[i]);
        advect_any(dst, q2.data(), dt, vel, s);
        for (idx i = 0; i < n; ++i) {
            T lo, hi;
            corner_range(q, vel, dt, s, i, &lo, &hi);
            if (dst[i] < lo || dst[i] > hi || dst[i] != dst[i]) dst[i] = q1[i];
        }
    }
}

#define PGO_ADV2(T, SFX)                                                                                       \
    PGO_EXPORT void pgo_advect2_##SFX(T* dst, const T* src, double dt, const T* vel, int scheme, int nd, long d, \
                                      long h, long w) {                                                        \
        advect2(dst, src, (T)dt, vel, scheme, shape_of(nd, d, h, w));                                          \
    }
PGO_BOTH(PGO_ADV2)

// advect of a bfloat16 cell field (bit patterns) with a float velocity: the
// float advection of the exactly widened values, rounded to bfloat16.
PGO_EXPORT void pgo_advect_bf16(uint16_t* dst, const uint16_t* src, double dt, const float* vel, int nd, long d, long h,
                                long w) {
    const Shape s = shape_of(nd, d, h, w);
    const idx n = s.nc();
    std::vector<float> q(n), out(n);
    for (idx i = 0; i < n; ++i) {
        const uint32_t u = (uint32_t)src[i] << 16;
        std::memcpy(&q[i], &u, 4);
    }
    if (nd == 2)
        advect_2d(out.data(), q.data(), (float)dt, vel, s.h, s.w);
    else
        advect_3d(out.data(), q.data(), (float)dt, vel, D3{s.d, s.h, s.w});
    for (idx i = 0; i < n; ++i) {
        const float r = round_bf16(out[i]);
        uint32_t u;
        std::memcpy(&u, &r, 4);
        dst[i] = (uint16_t)(u >> 16);
    }
}

// ---------------------------------------------------------------------------
// panopaea/src/sparse.rs:119-128 SparseMatrix::mul_vec (CSR, usize indices):
// b[i] = fold(0, |acc, (k, j)| acc + data[start + k] * x[j]) over row i.
template <class T> static void csr_mul_vec(long rows, const long* rowp, const long* cols, const T* data, const T* x, T* b) {
    for (long i = 0; i < rows; ++i) {
        T acc = T(0);
        for (long k = rowp[i]; k < rowp[i + 1]; ++k) acc = acc + data[k] * x[cols[k]];
        b[i] = acc;
    }
}

// sparse.rs:20-25 DiagonalMatrix::mul_vec: b = x * a.
template <class T> static void diag_mul_vec(long n, const T* a, const T* x, T* b) {
    for (long i = 0; i < n; ++i) b[i] = x[i] * a[i];
}

// panopaea_utils/src/imgproc.rs:2-5 transfer, laid out as png.rs:6-18 writes
// the image (row y of the image shows field row h-1-y), three channels.
template <class T>
static void transfer_rgb8(long h, long w, const T* f, double lo, double hi, unsigned char* rgb) {
    for (long y = 0; y < h; ++y)
        for (long x = 0; x < w; ++x) {
            const double v = std::fmax(std::fmin((double)f[(h - 1 - y) * w + x], hi), lo);
            const double s = (v - lo) / (hi - lo) * 255.0;
            const unsigned char u = (s != s) ? 0 : (s <= 0.0 ? 0 : (s >= 255.0 ? 255 : (unsigned char)s));
            for (int c = 0; c < 3; ++c) rgb[(y * w + x) * 3 + c] = u;
        }
}

#define PGO_EXTRA(T, SFX)                                                                                       \
    PGO_EXPORT void pgo_csr_mul_vec_##SFX(long rows, const long* rowp, const long* cols, const T* data,         \
                                          const T* x, T* b) {                                                   \
        csr_mul_vec(rows, rowp, cols, data, x, b);                                                              \
    }                                                                                                           \
    PGO_EXPORT void pgo_diag_mul_vec_##SFX(long n, const T* a, const T* x, T* b) { diag_mul_vec(n, a, x, b); }  \
    PGO_EXPORT void pgo_transfer_rgb8_##SFX(long h, long w, const T* f, double lo, double hi, unsigned char* rgb) { \
        transfer_rgb8(h, w, f, lo, hi, rgb);                                                                    \
    }

PGO_BOTH(PGO_EXTRA)
