// pg_advect.cu -- semi-Lagrangian advection (examples/dec_fluid.rs:169-291).
//
// One thread per output sample.  The back-traced position, clamps, floors
// and the lerp form of math/interp.rs:7-36 are evaluated in the reference's
// order with non-fusing round-to-nearest arithmetic (pg_ops2d.cuh), so a
// float (double) result equals a sequential float (double) evaluation of the
// Rust code.  3D is an extension: trilinear (math/interp.rs:23-36) with the
// per-axis rules of the 2D code.
#include "pg_ops2d.cuh"

namespace pg {

constexpr int kThreads = 256;

#define GRID_STRIDE(i, n) for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (I)gridDim.x * blockDim.x)

// advect, 2D (dec_fluid.rs:173-211)
template <class T, class I>
__global__ void k_advect_2d(T* __restrict__ dst, const T* __restrict__ q, const T* __restrict__ vel, I h, I w,
                            T ndt, T hix, T hiy) {
    const T* vy = vel;
    const T* vx = vel + (h + 1) * w;
    GRID_STRIDE(i, h * w) {
        const I y = i / w, x = i - y * w;
        dst[i] = advect2d_at<T, I>(q, vy, vx, h, w, ndt, hix, hiy, y, x);
    }
}

// advect, 3D extension
template <class T, class I>
__global__ void k_advect_3d(T* __restrict__ dst, const T* __restrict__ q, const T* __restrict__ vel, Dims D, T ndt,
                            T hix, T hiy, T hiz, FastDiv fw, FastDiv fh) {
    const I d = (I)D.d, h = (I)D.h, w = (I)D.w, hw = h * w;
    const I offy = (I)D.offy(), offx = (I)D.offx();
    auto FX = [&](I z, I y, I x) { return offx + (z * h + y) * (w + 1) + x; };
    auto FY = [&](I z, I y, I x) { return offy + (z * (h + 1) + y) * w + x; };
    auto FZ = [&](I z, I y, I x) { return (z * h + y) * w + x; };
    GRID_STRIDE(i, d * hw) {
        I x, y;
        const I zy = split(i, w, fw, x);
        const I z = split(zy, h, fh, y);
        const T vcx = half_rn(add_rn(vel[FX(z, y, x)], vel[FX(z, y, x + 1)]));
        const T vcy = half_rn(add_rn(vel[FY(z, y, x)], vel[FY(z, y + 1, x)]));
        const T vcz = half_rn(add_rn(vel[FZ(z, y, x)], vel[FZ(z + 1, y, x)]));
        const T ppx = back(add_rn((T)x, T(0.5)), ndt, vcx);
        const T ppy = back(add_rn((T)y, T(0.5)), ndt, vcy);
        const T ppz = back(add_rn((T)z, T(0.5)), ndt, vcz);
        I ix, iy, iz;
        T s, t, u;
        cell_coord(ppx, w, hix, ix, s);
        cell_coord(ppy, h, hiy, iy, t);
        cell_coord(ppz, d, hiz, iz, u);
        const T* q0 = q + iz * hw + iy * w + ix;
        const T* q1 = q0 + hw;
        dst[i] = lerp_ref(bilerp(q0[0], q0[1], q0[w], q0[w + 1], s, t), bilerp(q1[0], q1[1], q1[w], q1[w + 1], s, t), u);
    }
}

// advect_mac, 2D (dec_fluid.rs:213-291); src/dst/vel share the face layout.
template <class T, class I>
__global__ void k_advect_mac_2d(T* __restrict__ dst, const T* __restrict__ src, const T* __restrict__ vel, I h, I w,
                                T ndt) {
    const I n0 = (h + 1) * w, nf = n0 + h * (w + 1), wx = w + 1;
    const T* vy = vel;
    const T* vx = vel + n0;
    GRID_STRIDE(i, nf) {
        if (i >= n0) {  // x faces, qx dims (h, w+1)
            const I j = i - n0;
            const I y = j / wx, x = j - y * wx;
            dst[i] = advect_mac2d_x_at<T, I>(src + n0, vy, vx, h, w, ndt, y, x);
        } else {  // y faces, qy dims (h+1, w)
            const I y = i / w, x = i - y * w;
            dst[i] = advect_mac2d_y_at<T, I>(src, vy, vx, h, w, ndt, y, x);
        }
    }
}

// The three face parts of a 3D MAC field: part 0 = z faces (d+1, h, w) at
// offset 0, part 1 = y faces (d, h+1, w), part 2 = x faces (d, h, w+1).
// Every 3D MAC advection sample reads its velocity and source values
// through an accessor, so the plain and the shared-memory-staged kernels run
// the same arithmetic on the same values.
template <class T, class I> struct MacGlobal {
    const T* vel;
    const T* src;
    I d, h, w;
    __device__ __forceinline__ I nz() const { return (d + 1) * h * w; }
    __device__ __forceinline__ I ny() const { return d * (h + 1) * w; }
    __device__ __forceinline__ I ix(I z, I y, I x) const { return nz() + ny() + (z * h + y) * (w + 1) + x; }
    __device__ __forceinline__ I iy(I z, I y, I x) const { return nz() + (z * (h + 1) + y) * w + x; }
    __device__ __forceinline__ I iz(I z, I y, I x) const { return (z * h + y) * w + x; }
    __device__ __forceinline__ T vx(I z, I y, I x) const { return vel[ix(z, y, x)]; }
    __device__ __forceinline__ T vy(I z, I y, I x) const { return vel[iy(z, y, x)]; }
    __device__ __forceinline__ T vz(I z, I y, I x) const { return vel[iz(z, y, x)]; }
    // The 8 source values around a sample of part p: c[4 * zi + 2 * yi + xi].
    __device__ __forceinline__ void gather(int p, I z0, I z1, I y0, I y1, I x0, I x1, T c[8]) const {
        const I nyp = p == 1 ? h + 1 : h, nxp = p == 2 ? w + 1 : w;
        const T* q = src + (p == 0 ? I(0) : p == 1 ? nz() : nz() + ny());
        const T* a0 = q + z0 * nyp * nxp;
        const T* a1 = q + z1 * nyp * nxp;
        c[0] = a0[y0 * nxp + x0];
        c[1] = a0[y0 * nxp + x1];
        c[2] = a0[y1 * nxp + x0];
        c[3] = a0[y1 * nxp + x1];
        c[4] = a1[y0 * nxp + x0];
        c[5] = a1[y0 * nxp + x1];
        c[6] = a1[y1 * nxp + x0];
        c[7] = a1[y1 * nxp + x1];
    }
};

// Trilinear face sample of part p with dims (nz, ny, nx).
template <class T, class I, class A>
__device__ __forceinline__ T sample_part(const A& acc, int p, I nz, I ny, I nx, T ppx, T ox, T ppy, T oy, T ppz,
                                         T oz) {
    I x0, x1, y0, y1, z0, z1;
    T s, t, u;
    face_coord(ppx, ox, nx, x0, x1, s);
    face_coord(ppy, oy, ny, y0, y1, t);
    face_coord(ppz, oz, nz, z0, z1, u);
    T c[8];
    acc.gather(p, z0, z1, y0, y1, x0, x1, c);
    const T b0 = bilerp(c[0], c[1], c[2], c[3], s, t);
    const T b1 = bilerp(c[4], c[5], c[6], c[7], s, t);
    return lerp_ref(b0, b1, u);
}

// The x, y and z faces that share index (z, y, x) of the (d+1) x (h+1) x
// (w+1) box (those that exist), advected into dst.
template <class T, class I, class A>
__device__ __forceinline__ void mac3_index(const A& acc, const MacGlobal<T, I>& G, T* __restrict__ dst, T ndt, I z,
                                           I y, I x) {
    const I d = G.d, h = G.h, w = G.w;
    if (z < d && y < h) {  // x face (z, y, x), part dims (d, h, w+1)
        const I xc = x < w - 1 ? x : w - 1, xm = x > 0 ? x - 1 : 0;
        const T vx_ = acc.vx(z, y, x);
        const T vy_ = avg4(acc.vy(z, y, xc), acc.vy(z, y + 1, xc), acc.vy(z, y, xm), acc.vy(z, y + 1, xm));
        const T vz_ = avg4(acc.vz(z, y, xc), acc.vz(z + 1, y, xc), acc.vz(z, y, xm), acc.vz(z + 1, y, xm));
        dst[G.ix(z, y, x)] = sample_part<T, I>(acc, 2, d, h, w + 1, back(add_rn((T)x, T(0)), ndt, vx_), T(0),
                                               back(add_rn((T)y, T(0.5)), ndt, vy_), T(0.5),
                                               back(add_rn((T)z, T(0.5)), ndt, vz_), T(0.5));
    }
    if (z < d && x < w) {  // y face (z, y, x), part dims (d, h+1, w)
        const I yc = y < h - 1 ? y : h - 1, ym = y > 0 ? y - 1 : 0;
        const T vx_ = avg4(acc.vx(z, yc, x), acc.vx(z, yc, x + 1), acc.vx(z, ym, x), acc.vx(z, ym, x + 1));
        const T vy_ = acc.vy(z, y, x);
        const T vz_ = avg4(acc.vz(z, yc, x), acc.vz(z + 1, yc, x), acc.vz(z, ym, x), acc.vz(z + 1, ym, x));
        dst[G.iy(z, y, x)] = sample_part<T, I>(acc, 1, d, h + 1, w, back(add_rn((T)x, T(0.5)), ndt, vx_), T(0.5),
                                               back(add_rn((T)y, T(0)), ndt, vy_), T(0),
                                               back(add_rn((T)z, T(0.5)), ndt, vz_), T(0.5));
    }
    if (y < h && x < w) {  // z face (z, y, x), part dims (d+1, h, w)
        const I zc = z < d - 1 ? z : d - 1, zm = z > 0 ? z - 1 : 0;
        const T vx_ = avg4(acc.vx(zc, y, x), acc.vx(zc, y, x + 1), acc.vx(zm, y, x), acc.vx(zm, y, x + 1));
        const T vy_ = avg4(acc.vy(zc, y, x), acc.vy(zc, y + 1, x), acc.vy(zm, y, x), acc.vy(zm, y + 1, x));
        const T vz_ = acc.vz(z, y, x);
        dst[G.iz(z, y, x)] = sample_part<T, I>(acc, 0, d + 1, h, w, back(add_rn((T)x, T(0.5)), ndt, vx_), T(0.5),
                                               back(add_rn((T)y, T(0.5)), ndt, vy_), T(0.5),
                                               back(add_rn((T)z, T(0)), ndt, vz_), T(0));
    }
}

// advect_mac, 3D extension
template <class T, class I>
__global__ void k_advect_mac_3d(T* __restrict__ dst, const T* __restrict__ src, const T* __restrict__ vel, Dims D,
                                T ndt, FastDiv fexy, FastDiv fex) {
    const MacGlobal<T, I> G{vel, src, (I)D.d, (I)D.h, (I)D.w};
    // One thread per index (z, y, x) of the (d+1) x (h+1) x (w+1) box: it
    // computes the x, y and z faces that share that index, so the gathers of
    // the three components hit the same cache lines (processing the three
    // parts one after another re-reads each part from DRAM).
    const I ex = G.w + 1, exy = (G.h + 1) * ex;
    GRID_STRIDE(t, (G.d + 1) * exy) {
        I r, x;
        const I z = split(t, exy, fexy, r);
        const I y = split(r, ex, fex, x);
        mac3_index(G, G, dst, ndt, z, y, x);
    }
}

template <class T> int launch_advect(const pg_grid* g, T* dst, const T* src, double dt, const T* vel) {
    const Dims& D = g->dims;
    if (D.h < 2 || D.w < 2 || (D.nd == 3 && D.d < 2))
        return bad_arg("pg_advect: every dimension must be >= 2 (the reference indexes the +1 neighbour)");
    const T ndt = -(T)dt;
    const T hix = (T)((double)D.w - 1.00001), hiy = (T)((double)D.h - 1.00001), hiz = (T)((double)D.d - 1.00001);
    const int nb = grid_blocks(g, D.nc(), kThreads);
    cudaStream_t s = g->stream;
    if (D.nf() < ((i64)1 << 31)) {
        if (D.nd == 2)
            PG_LAUNCH(KK_ADVECT, s, k_advect_2d<T, int><<<nb, kThreads, 0, s>>>(dst, src, vel, (int)D.h, (int)D.w, ndt, hix, hiy));
        else
            PG_LAUNCH(KK_ADVECT, s,
                      k_advect_3d<T, int><<<nb, kThreads, 0, s>>>(dst, src, vel, D, ndt, hix, hiy, hiz,
                                                                  fast_div((unsigned)D.w), fast_div((unsigned)D.h)));
    } else {
        if (D.nd == 2)
            PG_LAUNCH(KK_ADVECT, s, k_advect_2d<T, i64><<<nb, kThreads, 0, s>>>(dst, src, vel, D.h, D.w, ndt, hix, hiy));
        else
            PG_LAUNCH(KK_ADVECT, s,
                      k_advect_3d<T, i64><<<nb, kThreads, 0, s>>>(dst, src, vel, D, ndt, hix, hiy, hiz, FastDiv{},
                                                                  FastDiv{}));
    }
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template <class T> int launch_advect_mac(const pg_grid* g, T* dst, const T* src, double dt, const T* vel) {
    const Dims& D = g->dims;
    const T ndt = -(T)dt;
    const int nb = grid_blocks(g, D.nf(), kThreads);
    cudaStream_t s = g->stream;
    if (D.nf() < ((i64)1 << 31)) {
        if (D.nd == 2)
            PG_LAUNCH(KK_ADVECT_MAC, s, k_advect_mac_2d<T, int><<<nb, kThreads, 0, s>>>(dst, src, vel, (int)D.h, (int)D.w, ndt));
        else
            PG_LAUNCH(KK_ADVECT_MAC, s,
                      k_advect_mac_3d<T, int><<<nb, kThreads, 0, s>>>(
                          dst, src, vel, D, ndt, fast_div((unsigned)((D.h + 1) * (D.w + 1))), fast_div((unsigned)(D.w + 1))));
    } else {
        if (D.nd == 2)
            PG_LAUNCH(KK_ADVECT_MAC, s, k_advect_mac_2d<T, i64><<<nb, kThreads, 0, s>>>(dst, src, vel, D.h, D.w, ndt));
        else
            PG_LAUNCH(KK_ADVECT_MAC, s,
                      k_advect_mac_3d<T, i64><<<nb, kThreads, 0, s>>>(dst, src, vel, D, ndt, FastDiv{}, FastDiv{}));
    }
    PG_CHECK_LAUNCH();
    return PG_OK;
}

// ---------------------------------------------------------------------------
// Second-order advection of cell scalars (extension; the reference has only
// the first-order scheme of examples/dec_fluid.rs:173-211).  With A(q, dt)
// that scheme:
//   MacCormack: q1 = A(q, dt), q2 = A(q1, -dt), q' = q1 + 0.5 (q - q2)
//   BFECC:      q1 = A(q, dt), q2 = A(q1, -dt), qt = q + 0.5 (q - q2),
//               q' = A(qt, dt)
// both limited: where q' leaves [min, max] of the source values of q the
// first-order sample interpolated from, q' = q1 (Selle et al. 2008).

// min / max of the corner values of q at cell i's first-order back-trace.
template <class T, class I>
__device__ __forceinline__ void corner_range(const T* __restrict__ q, const T* __restrict__ vel, const Dims& D, T ndt,
                                             T hix, T hiy, T hiz, I i, T& lo, T& hi) {
    const I w = (I)D.w, h = (I)D.h;
    if (D.nd == 2) {
        const T* vy = vel;
        const T* vx = vel + (h + 1) * w;
        const I y = i / w, x = i - y * w;
        const T vcx = half_rn(add_rn(vx[y * (w + 1) + x], vx[y * (w + 1) + x + 1]));
        const T vcy = half_rn(add_rn(vy[y * w + x], vy[(y + 1) * w + x]));
        I ix, iy;
        T u, v;
        cell_coord(back(add_rn((T)x, T(0.5)), ndt, vcx), w, hix, ix, u);
        cell_coord(back(add_rn((T)y, T(0.5)), ndt, vcy), h, hiy, iy, v);
        const T* q0 = q + iy * w + ix;
        lo = fmin(fmin(q0[0], q0[1]), fmin(q0[w], q0[w + 1]));
        hi = fmax(fmax(q0[0], q0[1]), fmax(q0[w], q0[w + 1]));
        return;
    }
    const I d = (I)D.d, hw = h * w;
    const I offy = (I)D.offy(), offx = (I)D.offx();
    const I zy = i / w, x = i - zy * w;
    const I z = zy / h, y = zy - z * h;
    const T vcx = half_rn(add_rn(vel[offx + (z * h + y) * (w + 1) + x], vel[offx + (z * h + y) * (w + 1) + x + 1]));
    const T vcy = half_rn(add_rn(vel[offy + (z * (h + 1) + y) * w + x], vel[offy + (z * (h + 1) + y + 1) * w + x]));
    const T vcz = half_rn(add_rn(vel[(z * h + y) * w + x], vel[((z + 1) * h + y) * w + x]));
    I ix, iy, iz;
    T s, t, u;
    cell_coord(back(add_rn((T)x, T(0.5)), ndt, vcx), w, hix, ix, s);
    cell_coord(back(add_rn((T)y, T(0.5)), ndt, vcy), h, hiy, iy, t);
    cell_coord(back(add_rn((T)z, T(0.5)), ndt, vcz), d, hiz, iz, u);
    const T* q0 = q + iz * hw + iy * w + ix;
    const T* q1 = q0 + hw;
    lo = fmin(fmin(fmin(q0[0], q0[1]), fmin(q0[w], q0[w + 1])), fmin(fmin(q1[0], q1[1]), fmin(q1[w], q1[w + 1])));
    hi = fmax(fmax(fmax(q0[0], q0[1]), fmax(q0[w], q0[w + 1])), fmax(fmax(q1[0], q1[1]), fmax(q1[w], q1[w + 1])));
}

// MacCormack: dst = q1 + 0.5 (q - q2), limited.
template <class T, class I>
__global__ void k_maccormack(T* __restrict__ dst, const T* __restrict__ q, const T* __restrict__ q1,
                             const T* __restrict__ q2, const T* __restrict__ vel, Dims D, T ndt, T hix, T hiy, T hiz) {
    GRID_STRIDE(i, (I)D.nc()) {
        T lo, hi;
        corner_range<T, I>(q, vel, D, ndt, hix, hiy, hiz, i, lo, hi);
        const T a = q1[i];
        const T v = add_rn(a, mul_rn(T(0.5), sub_rn(q[i], q2[i])));
        dst[i] = (v < lo || v > hi || v != v) ? a : v;
    }
}

// BFECC: qt = q + 0.5 (q - q2)
template <class T, class I> __global__ void k_bfecc_pre(T* qt, const T* q, const T* q2, I n) {  // qt may alias q2
    GRID_STRIDE(i, n) qt[i] = add_rn(q[i], mul_rn(T(0.5), sub_rn(q[i], q2[i])));
}

// BFECC limiter: keep A(qt) where it stays in the first-order range, else q1.
template <class T, class I>
__global__ void k_bfecc_limit(T* __restrict__ dst, const T* __restrict__ q, const T* __restrict__ q1,
                              const T* __restrict__ vel, Dims D, T ndt, T hix, T hiy, T hiz) {
    GRID_STRIDE(i, (I)D.nc()) {
        T lo, hi;
        corner_range<T, I>(q, vel, D, ndt, hix, hiy, hiz, i, lo, hi);
        const T v = dst[i];
        if (v < lo || v > hi || v != v) dst[i] = q1[i];
    }
}

// dst = second-order advection of src; t1, t2 are caller scratch cell fields.
template <class T>
int launch_advect2(const pg_grid* g, T* dst, const T* src, double dt, const T* vel, int scheme, T* t1, T* t2) {
    int rc;
    if ((rc = launch_advect<T>(g, t1, src, dt, vel))) return rc;    // q1 = A(q, dt)
    if ((rc = launch_advect<T>(g, t2, t1, -dt, vel))) return rc;    // q2 = A(q1, -dt)
    const Dims& D = g->dims;
    const T ndt = -(T)dt;
    const T hix = (T)((double)D.w - 1.00001), hiy = (T)((double)D.h - 1.00001), hiz = (T)((double)D.d - 1.00001);
    const int nb = grid_blocks(g, D.nc(), kThreads);
    cudaStream_t s = g->stream;
    if (D.nf() >= ((i64)1 << 31)) return bad_arg("second-order advection: grid too large for 32-bit indexing");
    if (scheme == 1) {
        PG_LAUNCH(KK_ADVECT, s, k_maccormack<T, int><<<nb, kThreads, 0, s>>>(dst, src, t1, t2, vel, D, ndt, hix, hiy, hiz));
    } else {
        PG_LAUNCH(KK_ADVECT, s, k_bfecc_pre<T, int><<<nb, kThreads, 0, s>>>(t2, src, t2, (int)D.nc()));
        if ((rc = launch_advect<T>(g, dst, t2, dt, vel))) return rc;  // A(qt, dt)
        PG_LAUNCH(KK_ADVECT, s, k_bfecc_limit<T, int><<<nb, kThreads, 0, s>>>(dst, src, t1, vel, D, ndt, hix, hiy, hiz));
    }
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template int launch_advect2<float>(const pg_grid*, float*, const float*, double, const float*, int, float*, float*);
template int launch_advect2<double>(const pg_grid*, double*, const double*, double, const double*, int, double*,
                                    double*);

template int launch_advect<float>(const pg_grid*, float*, const float*, double, const float*);
template int launch_advect<double>(const pg_grid*, double*, const double*, double, const double*);
template int launch_advect_mac<float>(const pg_grid*, float*, const float*, double, const float*);
template int launch_advect_mac<double>(const pg_grid*, double*, const double*, double, const double*);

}  // namespace pg

using namespace pg;

#define PG_ADV_ABI(T, SFX)                                                                               \
    extern "C" int pg_advect_##SFX(const pg_grid* g, T* dst, const T* src, double dt, const T* vel) {   \
        if (!g || !dst || !src || !vel) return bad_arg("pg_advect: NULL argument");                     \
        if (dst == src) return bad_arg("pg_advect: dst must not alias src");                            \
        return launch_advect<T>(g, dst, src, dt, vel);                                                   \
    }                                                                                                    \
    extern "C" int pg_advect_mac_##SFX(const pg_grid* g, T* dst, const T* src, double dt, const T* vel) { \
        if (!g || !dst || !src || !vel) return bad_arg("pg_advect_mac: NULL argument");                 \
        if (dst == src || dst == vel) return bad_arg("pg_advect_mac: dst must not alias src or vel");   \
        return launch_advect_mac<T>(g, dst, src, dt, vel);                                               \
    }

PG_ADV_ABI(float, f32)
PG_ADV_ABI(double, f64)
