// pg_ops2d.cuh -- per-sample 2D operator arithmetic shared by the single-grid
// kernels and the batched (many-grid) kernels, so both produce the same bits.
// Each function evaluates one output sample of the cited reference code in
// its operation order, with non-fusing round-to-nearest arithmetic.
#pragma once
#include "pg_internal.cuh"

namespace pg {

template <class T> __device__ __forceinline__ T bilerp(T a00, T a01, T a10, T a11, T s, T t) {
    return lerp_ref(lerp_ref(a00, a01, s), lerp_ref(a10, a11, s), t);
}

// dec_fluid.rs:194-201 for one axis: p = clamp(pos - 0.5, 0, n - 1.00001);
// i = floor(p); frac = p - i.  `hi` is n - 1.00001 rounded to T; when it
// rounds to n-1 (float, n >= 257) the index is kept at n-2.
template <class T, class I> __device__ __forceinline__ void cell_coord(T pos, I n, T hi, I& i0, T& frac) {
    const T p = fmin(fmax(sub_rn(pos, T(0.5)), T(0)), hi);
    I i = (I)floor(p);
    if (i > n - 2) i = n - 2;
    i0 = i;
    frac = sub_rn(p, (T)i);
}

// dec_fluid.rs:236-244 / :274-281 for one axis of a face sample.
template <class T, class I> __device__ __forceinline__ void face_coord(T pos, T off, I n, I& i0, I& i1, T& frac) {
    const T q = sub_rn(pos, off);
    const T p = fmax(floor(q), T(0));
    const T last = (T)(n - 1);
    i0 = (I)fmin(p, last);
    // = (I)fmin(p + 1, last): p is integer-valued, so either p >= last
    // (both give n - 1) or p <= n - 2 and p + 1 is exact
    i1 = i0 + 1 < n ? i0 + 1 : n - 1;
    // .min(1.0).max(0.0) with Rust's NaN rule: NaN.min(1) = 1.  Written out
    // because the compiler turns fmax(fmin(v, 1), 0) into a saturate, which
    // maps NaN to 0.
    const T v = sub_rn(q, p);
    frac = (v != v) ? T(1) : fmax(fmin(v, T(1)), T(0));
}

// pos + (-dt) * v  (integrate_euler, dec_fluid.rs:169-171)
template <class T> __device__ __forceinline__ T back(T pos, T ndt, T v) { return add_rn(pos, mul_rn(ndt, v)); }

template <class T> __device__ __forceinline__ T avg4(T a, T b, T c, T d) {
    return quarter_rn(add_rn(add_rn(add_rn(a, b), c), d));
}

// advect (dec_fluid.rs:173-211) at cell (y, x); vy = vel, vx = vel + (h+1)w.
template <class T, class I>
__device__ __forceinline__ T advect2d_at(const T* __restrict__ q, const T* __restrict__ vy, const T* __restrict__ vx,
                                         I h, I w, T ndt, T hix, T hiy, I y, I x) {
    const T vcx = half_rn(add_rn(vx[y * (w + 1) + x], vx[y * (w + 1) + x + 1]));
    const T vcy = half_rn(add_rn(vy[y * w + x], vy[(y + 1) * w + x]));
    const T ppx = back(add_rn((T)x, T(0.5)), ndt, vcx);
    const T ppy = back(add_rn((T)y, T(0.5)), ndt, vcy);
    I ix, iy;
    T u, v;
    cell_coord(ppx, w, hix, ix, u);
    cell_coord(ppy, h, hiy, iy, v);
    const T* q0 = q + iy * w + ix;
    return bilerp(q0[0], q0[1], q0[w], q0[w + 1], u, v);
}

// advect_mac x face (y, x), x in [0, w] (dec_fluid.rs:218-253).
template <class T, class I>
__device__ __forceinline__ T advect_mac2d_x_at(const T* __restrict__ qx, const T* __restrict__ vy,
                                               const T* __restrict__ vx, I h, I w, T ndt, I y, I x) {
    const I wx = w + 1;
    const I xc = x < w - 1 ? x : w - 1, xm = x > 0 ? x - 1 : 0;
    const T velx = vx[y * wx + x];
    const T vely = quarter_rn(add_rn(add_rn(add_rn(vy[y * w + xc], vy[(y + 1) * w + xc]), vy[y * w + xm]),
                                 vy[(y + 1) * w + xm]));
    const T ppx = back(add_rn((T)x, T(0)), ndt, velx);
    const T ppy = back(add_rn((T)y, T(0.5)), ndt, vely);
    I x0, x1, y0, y1;
    T s, t;
    face_coord(ppx, T(0), w + 1, x0, x1, s);
    face_coord(ppy, T(0.5), h, y0, y1, t);
    return bilerp(qx[y0 * wx + x0], qx[y0 * wx + x1], qx[y1 * wx + x0], qx[y1 * wx + x1], s, t);
}

// advect_mac y face (y, x), y in [0, h] (dec_fluid.rs:255-290).
template <class T, class I>
__device__ __forceinline__ T advect_mac2d_y_at(const T* __restrict__ qy, const T* __restrict__ vy,
                                               const T* __restrict__ vx, I h, I w, T ndt, I y, I x) {
    const I wx = w + 1;
    const I yc = y < h - 1 ? y : h - 1, ym = y > 0 ? y - 1 : 0;
    const T velx = quarter_rn(add_rn(add_rn(add_rn(vx[yc * wx + x], vx[yc * wx + x + 1]), vx[ym * wx + x]),
                                 vx[ym * wx + x + 1]));
    const T vely = vy[y * w + x];
    const T ppx = back(add_rn((T)x, T(0.5)), ndt, velx);
    const T ppy = back(add_rn((T)y, T(0)), ndt, vely);
    I x0, x1, y0, y1;
    T s, t;
    face_coord(ppx, T(0.5), w, x0, x1, s);
    face_coord(ppy, T(0), h + 1, y0, y1, t);
    return bilerp(qy[y0 * w + x0], qy[y0 * w + x1], qy[y1 * w + x0], qy[y1 * w + x1], s, t);
}

}  // namespace pg
