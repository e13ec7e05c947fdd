// pg_dec.cu -- DEC operators and the fused per-step operators.
//
// Every kernel here reproduces the reference's floating-point operation
// order (add/sub/mul with explicit round-to-nearest intrinsics, never fused
// into FMA), so results are bit-identical to a sequential evaluation of the
// cited Rust in the same precision.
#include "pg_internal.cuh"

namespace pg {

constexpr int kThreads = 256;

#define GRID_STRIDE(i, n) for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (i64)gridDim.x * blockDim.x)
#define GRID_STRIDE_I(i, n) for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (I)gridDim.x * blockDim.x)

// grid.rs:206-238: sign flip of one part of the face buffer.
template <class T> __global__ void k_hodge1(T* __restrict__ out, const T* __restrict__ in, i64 n0, i64 n, int neg_first) {
    GRID_STRIDE(i, n) {
        const bool neg = (i < n0) == (neg_first != 0);
        const T v = in[i];
        out[i] = neg ? -v : v;
    }
}

template <class T> __global__ void k_copy(T* __restrict__ out, const T* __restrict__ in, i64 n) {
    GRID_STRIDE(i, n) out[i] = in[i];
}

// grid.rs:295-305: face = -bottom + top - left + right (2D).
template <class T, class I> __global__ void k_d1primal_2d(T* __restrict__ faces, const T* __restrict__ edges, I h, I w) {
    const T* e0 = edges;
    const T* e1 = edges + (h + 1) * w;
    GRID_STRIDE_I(i, h * w) {
        const I y = i / w, x = i - y * w;
        const T top = e0[y * w + x], bottom = e0[(y + 1) * w + x];
        const T left = e1[y * (w + 1) + x], right = e1[y * (w + 1) + x + 1];
        faces[i] = add_rn(sub_rn(add_rn(-bottom, top), left), right);
    }
}

// grid.rs:318-334 and its 3D extension: interior faces get the negative
// gradient, boundary faces are not written.
template <class T, class I> __global__ void k_d0dual(T* __restrict__ e, const T* __restrict__ p, Dims D) {
    const I nz = (I)D.nfz(), ny = (I)D.nfy(), nf = (I)D.nf();
    const I h = D.h, w = D.w, hw = h * w;
    GRID_STRIDE_I(i, nf) {
        if (i < nz) {  // vz faces (d+1, h, w)
            const I z = i / hw, r = i - z * hw;
            if (z == 0 || z == (I)D.d) continue;
            const I c = z * hw + r;
            e[i] = -sub_rn(p[c], p[c - hw]);
        } else if (i < nz + ny) {  // vy faces (d, h+1, w)
            const I j = i - nz;
            const I zy = j / w, x = j - zy * w;
            const I z = zy / (h + 1), y = zy - z * (h + 1);
            if (y == 0 || y == h) continue;
            const I c = (z * h + y) * w + x;
            e[i] = -sub_rn(p[c], p[c - w]);
        } else {  // vx faces (d, h, w+1)
            const I j = i - nz - ny;
            const I zy = j / (w + 1), x = j - zy * (w + 1);
            if (x == 0 || x == w) continue;
            const I c = zy * w + x;
            e[i] = sub_rn(p[c - 1], p[c]);
        }
    }
}

template <class T> __global__ void k_mask(T* __restrict__ e, const uint8_t* __restrict__ solid, i64 nf) {
    GRID_STRIDE(i, nf) if (solid[i]) e[i] = T(0);
}

// Closure of examples/dec_fluid.rs:100-119 in one pass: face gradients
// (grid.rs:318-334) closed on solid/boundary faces, then the 2D order of
// grid.rs:295-305 after the *1^-1 sign flip, extended by the z pair in 3D,
// then * dt.
template <class T, int ND>
__device__ __forceinline__ T lap_cell(const T* __restrict__ p, i64 c, uint8_t f, i64 w, i64 hw, T dt) {
    const T pc = p[c];
    const T gy_lo = (f & YLO) ? -sub_rn(pc, p[c - w]) : T(0);
    const T gy_hi = (f & YHI) ? -sub_rn(p[c + w], pc) : T(0);
    const T gx_lo = (f & XLO) ? sub_rn(p[c - 1], pc) : T(0);
    const T gx_hi = (f & XHI) ? sub_rn(pc, p[c + 1]) : T(0);
    T v = add_rn(sub_rn(sub_rn(gy_hi, gy_lo), gx_lo), gx_hi);
    if (ND == 3) {
        const T gz_lo = (f & ZLO) ? -sub_rn(pc, p[c - hw]) : T(0);
        const T gz_hi = (f & ZHI) ? -sub_rn(p[c + hw], pc) : T(0);
        v = add_rn(sub_rn(v, gz_lo), gz_hi);
    }
    return mul_rn(v, dt);
}

template <class T, int ND>
__global__ void k_laplacian(T* __restrict__ out, const T* __restrict__ p, const uint8_t* __restrict__ flags, Dims D, T dt) {
    const i64 w = D.w, hw = D.h * D.w;
    GRID_STRIDE(c, D.nc()) out[c] = lap_cell<T, ND>(p, c, flags[c], w, hw, dt);
}

// RHS of examples/dec_fluid.rs:68-83.  Interior faces are masked through the
// cell's open bits; boundary faces through the per-face solid array (the
// reference never masks them, and then face_solid is NULL).
template <class T, int ND, class I>
__global__ void k_rhs(T* __restrict__ b, const T* __restrict__ vel, const uint8_t* __restrict__ flags,
                      const uint8_t* __restrict__ fsolid, Dims D, FastDiv fw, FastDiv fh) {
    const I h = D.h, w = D.w;
    GRID_STRIDE_I(c, (I)D.nc()) {
        I x, y;
        const I zy = split(c, w, fw, x);
        const I z = split(zy, h, fh, y);
        const uint8_t f = flags[c];
        // Is a face masked?  Interior faces: the cell's open bit; boundary
        // faces: the per-face solid array (NULL = never masked).
        auto masked = [&](I idx, bool interior, uint8_t bit) -> bool {
            if (interior) return !(f & bit);
            return fsolid != nullptr && fsolid[idx] != 0;
        };
        const I iyl = (I)D.fy(z, y, x), iyh = (I)D.fy(z, y + 1, x);
        const I ixl = (I)D.fx(z, y, x), ixh = (I)D.fx(z, y, x + 1);
        const bool myl = masked(iyl, y > 0, YLO), myh = masked(iyh, y < h - 1, YHI);
        const T ux_lo = masked(ixl, x > 0, XLO) ? T(0) : vel[ixl];
        const T ux_hi = masked(ixh, x < w - 1, XHI) ? T(0) : vel[ixh];
        T v;
        if (ND == 2) {
            // hodge_1_dual then mask (grid.rs:223-238, dec_fluid.rs:69-78):
            // part 0 holds -vy, masked faces +0; then grid.rs:304.
            const T top = myl ? T(0) : -vel[iyl];
            const T bottom = myh ? T(0) : -vel[iyh];
            v = add_rn(sub_rn(add_rn(-bottom, top), ux_lo), ux_hi);
        } else {
            const T uy_lo = myl ? T(0) : vel[iyl];
            const T uy_hi = myh ? T(0) : vel[iyh];
            const I izl = (I)D.fz(z, y, x), izh = (I)D.fz(z + 1, y, x);
            const T uz_lo = masked(izl, z > 0, ZLO) ? T(0) : vel[izl];
            const T uz_hi = masked(izh, z < (I)D.d - 1, ZHI) ? T(0) : vel[izh];
            v = add_rn(sub_rn(add_rn(sub_rn(sub_rn(uy_hi, uy_lo), ux_lo), ux_hi), uz_lo), uz_hi);
        }
        b[c] = -v;
    }
}

// Projection of examples/dec_fluid.rs:123-141: interior faces
// vel = vel + dt * e (scaled_add) with e from grid.rs:318-334, boundary
// faces zeroed (walls).  zero_solid: solid interior faces zeroed after.
// P is the pressure type: T (the reference's arithmetic), or double for a
// float field projected with the FP64 pressure of the refined solve.
template <class T, class P, class I>
__global__ void k_project(T* vel, const T* src, const P* __restrict__ p, const uint8_t* __restrict__ flags, Dims D, P dt,
                          int zero_solid) {
    const I nz = (I)D.nfz(), ny = (I)D.nfy(), nf = (I)D.nf();
    const I h = D.h, w = D.w, hw = h * w;
    GRID_STRIDE_I(i, nf) {
        P e;
        bool open;
        if (i < nz) {
            const I z = i / hw, r = i - z * hw;
            if (z == 0 || z == (I)D.d) { vel[i] = T(0); continue; }
            const I c = z * hw + r;
            e = -sub_rn(p[c], p[c - hw]);
            open = flags[c] & ZLO;
        } else if (i < nz + ny) {
            const I j = i - nz;
            const I zy = j / w, x = j - zy * w;
            const I z = zy / (h + 1), y = zy - z * (h + 1);
            if (y == 0 || y == h) { vel[i] = T(0); continue; }
            const I c = (z * h + y) * w + x;
            e = -sub_rn(p[c], p[c - w]);
            open = flags[c] & YLO;
        } else {
            const I j = i - nz - ny;
            const I zy = j / (w + 1), x = j - zy * (w + 1);
            if (x == 0 || x == w) { vel[i] = T(0); continue; }
            const I c = zy * w + x;
            e = sub_rn(p[c - 1], p[c]);
            open = flags[c] & XLO;
        }
        vel[i] = (zero_solid && !open) ? T(0) : add_rn(src[i], (T)mul_rn(dt, e));
    }
}

// Wall step of examples/dec_fluid.rs:128-141 (3D: also vz at z = 0, d).
// Only the boundary faces are visited: 2dh x-walls, 2dw y-walls, 2hw z-walls.
template <class T, class I> __global__ void k_walls(T* __restrict__ vel, Dims D) {
    const I d = (I)D.d, h = (I)D.h, w = (I)D.w;
    const I nx = 2 * d * h, ny = 2 * d * w, nz = D.nd == 3 ? 2 * h * w : 0;
    const I offy = (I)D.offy(), offx = (I)D.offx();
    GRID_STRIDE_I(i, nx + ny + nz) {
        if (i < nx) {  // vx at x = 0 and x = w, rows (z, y)
            const I row = i >> 1;
            vel[offx + row * (w + 1) + ((i & 1) ? w : 0)] = T(0);
        } else if (i < nx + ny) {  // vy at y = 0 and y = h, (z, x)
            const I j = i - nx, side = j / (d * w), k = j - side * d * w;
            const I z = k / w, x = k - z * w;
            vel[offy + (z * (h + 1) + (side ? h : 0)) * w + x] = T(0);
        } else {  // vz at z = 0 and z = d, (y, x)
            const I j = i - nx - ny, side = j / (h * w), k = j - side * h * w;
            vel[(side ? d : 0) * h * w + k] = T(0);
        }
    }
}

// Inflow box of examples/dec_fluid.rs:48-57: density = sd and the vy face
// with the cell's index = sv, for cells in [lo, hi).
template <class T, class I>
__global__ void k_source_box(T* __restrict__ rho, T* __restrict__ vel, Dims D, I z0, I y0, I x0, I bz, I by,
                             I bx, T sd, T sv) {
    GRID_STRIDE_I(i, bz * by * bx) {
        const I zy = i / bx, x = x0 + (i - zy * bx);
        const I z = z0 + zy / by, y = y0 + zy % by;
        rho[(I)D.cell(z, y, x)] = sd;
        vel[(I)D.fy(z, y, x)] = sv;
    }
}

template <class T> __global__ void k_source_field(T* __restrict__ rho, const T* __restrict__ src, i64 n) {
    GRID_STRIDE(i, n) rho[i] = fmax(rho[i], src[i]);
}

// Buoyancy (extension): vy = vy + coef * (0.5 * (rho[y-1] + rho[y])) on
// interior y faces.
template <class T, class I> __global__ void k_buoyancy(T* __restrict__ vel, const T* __restrict__ rho, Dims D, T coef) {
    const I h = D.h, w = D.w;
    GRID_STRIDE_I(j, (I)D.nfy()) {
        const I zy = j / w, x = j - zy * w;
        const I z = zy / (h + 1), y = zy - z * (h + 1);
        if (y == 0 || y == h) continue;
        const I c = (z * h + y) * w + x;
        const I f = (I)D.offy() + j;
        vel[f] = add_rn(vel[f], mul_rn(coef, mul_rn(T(0.5), add_rn(rho[c - w], rho[c]))));
    }
}

// ---------------------------------------------------------------------------
// Host launchers (used by the C ABI below and by the step in pg_solve.cu).

template <class T> int launch_hodge1(const pg_grid* g, T* out, const T* in, int neg_first) {
    const Dims& D = g->dims;
    const i64 n0 = D.nfy(), n = D.nf();
    PG_LAUNCH(KK_DEC_OP, g->stream, k_hodge1<T><<<grid_blocks(g, n, kThreads), kThreads, 0, g->stream>>>(out, in, n0, n, neg_first));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template <class T> int launch_copy(const pg_grid* g, T* out, const T* in, i64 n) {
    PG_LAUNCH(KK_DEC_OP, g->stream, k_copy<T><<<grid_blocks(g, n, kThreads), kThreads, 0, g->stream>>>(out, in, n));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template <class T> int launch_laplacian(const pg_grid* g, T* out, const T* p, double dt) {
    const Dims& D = g->dims;
    if (D.nd == 2)
        PG_LAUNCH(KK_DEC_OP, g->stream, k_laplacian<T, 2><<<grid_blocks(g, D.nc(), kThreads), kThreads, 0, g->stream>>>(out, p, g->flags, D, (T)dt));
    else
        PG_LAUNCH(KK_DEC_OP, g->stream, k_laplacian<T, 3><<<grid_blocks(g, D.nc(), kThreads), kThreads, 0, g->stream>>>(out, p, g->flags, D, (T)dt));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template <class T> int launch_rhs(const pg_grid* g, T* b, const T* vel) {
    const Dims& D = g->dims;
    if (D.nd == 2)
        PG_IDX(g, PG_LAUNCH(KK_RHS, g->stream, k_rhs<T, 2, I><<<grid_blocks(g, D.nc(), kThreads), kThreads, 0, g->stream>>>(b, vel, g->flags, g->face_solid, D, fast_div_for<I>(D.w), fast_div_for<I>(D.h))));
    else
        PG_IDX(g, PG_LAUNCH(KK_RHS, g->stream, k_rhs<T, 3, I><<<grid_blocks(g, D.nc(), kThreads), kThreads, 0, g->stream>>>(b, vel, g->flags, g->face_solid, D, fast_div_for<I>(D.w), fast_div_for<I>(D.h))));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template <class T> int launch_project(const pg_grid* g, T* vel, const T* p, double dt, int zero_solid, const T* src) {
    const Dims& D = g->dims;
    PG_IDX(g, PG_LAUNCH(KK_PROJECT, g->stream, k_project<T, T, I><<<grid_blocks(g, D.nf(), kThreads), kThreads, 0, g->stream>>>(vel, src ? src : vel, p, g->flags, D, (T)dt, zero_solid)));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

int launch_project_p64(const pg_grid* g, float* vel, const double* p, double dt, int zero_solid, const float* src) {
    const Dims& D = g->dims;
    PG_IDX(g, PG_LAUNCH(KK_PROJECT, g->stream,
              k_project<float, double, I><<<grid_blocks(g, D.nf(), kThreads), kThreads, 0, g->stream>>>(
                  vel, src ? src : vel, p, g->flags, D, dt, zero_solid)));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

// Projection with a double-float pressure p = ph + pl: the difference
// p_lo - p_hi is formed exactly in the high parts (TwoSum), so the gradient
// keeps its FP32 relative accuracy however large p is.
__device__ __forceinline__ float df_diff(float ah, float al, float bh, float bl) {
    const float s = __fsub_rn(ah, bh);
    const float bb = __fsub_rn(s, ah);
    const float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(-bh, bb));
    return __fadd_rn(s, __fadd_rn(e, __fsub_rn(al, bl)));
}

// One thread per index (z, y, x) of the (d+1) x (h+1) x (w+1) box: it
// computes the x, y and z faces that share that index, so the double-float
// pressure of a cell is read once for its three low faces (a sweep per face
// part read it three times); pout (optional) receives p = ph + pl rounded to
// float, the refined solve's pressure output.
template <class I>
__global__ void k_project_dfj(float* vel, const float* src, const float* __restrict__ ph, const float* __restrict__ pl,
                              const uint8_t* __restrict__ flags, Dims D, float dt, int zero_solid,
                              float* __restrict__ pout, FastDiv fexy, FastDiv fex) {
    const I d = (I)D.d, h = (I)D.h, w = (I)D.w, hw = h * w;
    const I nz = (I)D.nfz(), ny = (I)D.nfy();
    const bool three = D.nd == 3;
    const I ex = w + 1, exy = (h + 1) * ex;
    const I n = (three ? d + 1 : d) * exy;
    auto face = [&](I i, I lo, I c, uint8_t bit, float chh, float chl) {
        const bool open = flags[c] & bit;
        const float e = df_diff(ph[lo], pl[lo], chh, chl);  // p_lo - p_hi = -grad p
        vel[i] = (zero_solid && !open) ? 0.f : __fadd_rn(src[i], __fmul_rn(dt, e));
    };
    GRID_STRIDE_I(t, n) {
        I r, x;
        const I z = split(t, exy, fexy, r);
        const I y = split(r, ex, fex, x);
        const I c = (z * h + y) * w + x;
        float chh = 0.f, chl = 0.f;
        if (z < d && y < h && x < w) {
            chh = ph[c];
            chl = pl[c];
            if (pout) pout[c] = __fadd_rn(chh, chl);
        }
        if (z < d && y < h) {  // x face (z, y, x)
            const I i = nz + ny + (z * h + y) * (w + 1) + x;
            if (x == 0 || x == w) vel[i] = 0.f;
            else face(i, c - 1, c, XLO, chh, chl);
        }
        if (z < d && x < w) {  // y face (z, y, x)
            const I i = nz + (z * (h + 1) + y) * w + x;
            if (y == 0 || y == h) vel[i] = 0.f;
            else face(i, c - w, c, YLO, chh, chl);
        }
        if (three && y < h && x < w) {  // z face (z, y, x)
            const I i = c;
            if (z == 0 || z == d) vel[i] = 0.f;
            else face(i, c - hw, c, ZLO, chh, chl);
        }
    }
}

int launch_project_df(const pg_grid* g, float* vel, const float* ph, const float* pl, double dt, int zero_solid,
                      const float* src, float* pout) {
    const Dims& D = g->dims;
    const i64 n = (D.nd == 3 ? D.d + 1 : D.d) * (D.h + 1) * (D.w + 1);
    PG_IDX(g, PG_LAUNCH(KK_PROJECT, g->stream,
              k_project_dfj<I><<<grid_blocks(g, n, kThreads), kThreads, 0, g->stream>>>(
                  vel, src ? src : vel, ph, pl, g->flags, D, (float)dt, zero_solid, pout,
                  fast_div_for<I>((D.h + 1) * (D.w + 1)), fast_div_for<I>(D.w + 1))));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template <class T> int launch_walls(const pg_grid* g, T* vel) {
    const Dims& D = g->dims;
    PG_IDX(g, PG_LAUNCH(KK_DEC_OP, g->stream, k_walls<T, I><<<grid_blocks(g, D.nf(), kThreads), kThreads, 0, g->stream>>>(vel, D)));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template <class T> int launch_source_box(const pg_grid* g, T* rho, T* vel, const pg_step_params* prm) {
    const Dims& D = g->dims;
    i64 lo[3], hi[3];
    const i64 ext[3] = {D.d, D.h, D.w};
    for (int a = 0; a < 3; ++a) {
        lo[a] = prm->source_lo[a];
        hi[a] = prm->source_hi[a];
        if (D.nd == 2 && a == 0) { lo[a] = 0; hi[a] = 1; }
        if (lo[a] < 0 || hi[a] > ext[a] || lo[a] > hi[a]) return bad_arg("source box outside the grid");
    }
    const i64 n = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
    if (n == 0) return PG_OK;
    PG_IDX(g, PG_LAUNCH(KK_STEP_MISC, g->stream, k_source_box<T, I><<<grid_blocks(g, n, kThreads), kThreads, 0, g->stream>>>(
        rho, vel, D, lo[0], lo[1], lo[2], hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2], (T)prm->source_density,
        (T)prm->source_vy)));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template <class T> int launch_source_field(const pg_grid* g, T* rho, const T* src) {
    const i64 n = g->dims.nc();
    PG_LAUNCH(KK_STEP_MISC, g->stream, k_source_field<T><<<grid_blocks(g, n, kThreads), kThreads, 0, g->stream>>>(rho, src, n));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template <class T> int launch_buoyancy(const pg_grid* g, T* vel, const T* rho, double dt, double beta) {
    const Dims& D = g->dims;
    PG_IDX(g, PG_LAUNCH(KK_STEP_MISC, g->stream, k_buoyancy<T, I><<<grid_blocks(g, D.nfy(), kThreads), kThreads, 0, g->stream>>>(vel, rho, D, (T)(dt * beta))));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

#define PG_INST(T)                                                                     \
    template int launch_hodge1<T>(const pg_grid*, T*, const T*, int);                  \
    template int launch_copy<T>(const pg_grid*, T*, const T*, i64);                    \
    template int launch_laplacian<T>(const pg_grid*, T*, const T*, double);            \
    template int launch_rhs<T>(const pg_grid*, T*, const T*);                          \
    template int launch_project<T>(const pg_grid*, T*, const T*, double, int, const T*); \
    template int launch_walls<T>(const pg_grid*, T*);                                  \
    template int launch_source_box<T>(const pg_grid*, T*, T*, const pg_step_params*);  \
    template int launch_source_field<T>(const pg_grid*, T*, const T*);                 \
    template int launch_buoyancy<T>(const pg_grid*, T*, const T*, double, double);
PG_INST(float)
PG_INST(double)

}  // namespace pg

using namespace pg;

#define NEED(cond, msg) \
    if (!(cond)) return bad_arg(msg)

#define PG_DEC_ABI(T, SFX)                                                                                  \
    extern "C" int pg_hodge_1_dual_##SFX(const pg_grid* g, T* primal, const T* dual) {                     \
        NEED(g && primal && dual, "pg_hodge_1_dual: NULL argument");                                        \
        NEED(g->dims.nd == 2, "pg_hodge_1_dual: 2D grids only");                                            \
        return launch_hodge1<T>(g, primal, dual, 1);                                                        \
    }                                                                                                       \
    extern "C" int pg_hodge_1_primal_##SFX(const pg_grid* g, T* dual, const T* primal) {                   \
        NEED(g && primal && dual, "pg_hodge_1_primal: NULL argument");                                      \
        NEED(g->dims.nd == 2, "pg_hodge_1_primal: 2D grids only");                                          \
        return launch_hodge1<T>(g, dual, primal, 0);                                                        \
    }                                                                                                       \
    extern "C" int pg_hodge_2_primal_##SFX(const pg_grid* g, T* dual, const T* primal) {                   \
        NEED(g && primal && dual, "pg_hodge_2_primal: NULL argument");                                      \
        return launch_copy<T>(g, dual, primal, g->dims.nc());                                               \
    }                                                                                                       \
    extern "C" int pg_derivative_1_primal_##SFX(const pg_grid* g, T* faces, const T* edges) {              \
        NEED(g && faces && edges, "pg_derivative_1_primal: NULL argument");                                 \
        NEED(g->dims.nd == 2, "pg_derivative_1_primal: 2D grids only");                                     \
        const i64 n = g->dims.nc();                                                                         \
        PG_IDX(g, PG_LAUNCH(KK_DEC_OP, g->stream, k_d1primal_2d<T, I><<<grid_blocks(g, n, kThreads), kThreads, 0, g->stream>>>(faces, edges, g->dims.h,  \
                                                                                  g->dims.w)));               \
        PG_CHECK_LAUNCH();                                                                                  \
        return PG_OK;                                                                                       \
    }                                                                                                       \
    extern "C" int pg_derivative_0_dual_##SFX(const pg_grid* g, T* edges, const T* faces) {                \
        NEED(g && faces && edges, "pg_derivative_0_dual: NULL argument");                                   \
        const i64 n = g->dims.nf();                                                                         \
        PG_IDX(g, PG_LAUNCH(KK_DEC_OP, g->stream, k_d0dual<T, I><<<grid_blocks(g, n, kThreads), kThreads, 0, g->stream>>>(edges, faces, g->dims)));        \
        PG_CHECK_LAUNCH();                                                                                  \
        return PG_OK;                                                                                       \
    }                                                                                                       \
    extern "C" int pg_mask_solid_faces_##SFX(const pg_grid* g, T* edges) {                                 \
        NEED(g && edges, "pg_mask_solid_faces: NULL argument");                                             \
        if (!g->face_solid) return PG_OK;                                                                   \
        const i64 n = g->dims.nf();                                                                         \
        PG_LAUNCH(KK_DEC_OP, g->stream, k_mask<T><<<grid_blocks(g, n, kThreads), kThreads, 0, g->stream>>>(edges, g->face_solid, n));        \
        PG_CHECK_LAUNCH();                                                                                  \
        return PG_OK;                                                                                       \
    }                                                                                                       \
    extern "C" int pg_laplacian_##SFX(const pg_grid* g, T* out, const T* p, double dt) {                   \
        NEED(g && out && p, "pg_laplacian: NULL argument");                                                 \
        return launch_laplacian<T>(g, out, p, dt);                                                          \
    }                                                                                                       \
    extern "C" int pg_divergence_rhs_##SFX(const pg_grid* g, T* b, const T* vel) {                         \
        NEED(g && b && vel, "pg_divergence_rhs: NULL argument");                                            \
        return launch_rhs<T>(g, b, vel);                                                                    \
    }                                                                                                       \
    extern "C" int pg_project_##SFX(const pg_grid* g, T* vel, const T* p, double dt, int zero_solid) {     \
        NEED(g && vel && p, "pg_project: NULL argument");                                                   \
        return launch_project<T>(g, vel, p, dt, zero_solid, vel);                                           \
    }                                                                                                       \
    extern "C" int pg_walls_##SFX(const pg_grid* g, T* vel) {                                              \
        NEED(g && vel, "pg_walls: NULL argument");                                                          \
        return launch_walls<T>(g, vel);                                                                     \
    }

PG_DEC_ABI(float, f32)
PG_DEC_ABI(double, f64)
