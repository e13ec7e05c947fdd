// pg_cg.cu -- conjugate gradient on the masked Laplacian (pcg.rs:14-82).
//
// Per iteration two kernels, each one pass over HBM:
//   k_cg_spmv   p = z + beta*p (p = z on the first iteration), Ap = A p with
//               the neighbours' new p recomputed from their inputs, p.Ap;
//   k_cg_update x += alpha p, r -= alpha Ap, ||r||inf and z.r.
// z = M^-1 r is r (identity, pcg.rs:8-12), r / diag (Jacobi, on the fly from
// the face-open bits) or read from a buffer an outer preconditioner wrote
// (multigrid, which then also reduces z.r).
// The scalars (sigma, alpha, beta, the stop test) live in a device-side
// CgState written by the last block of each reduction kernel, so the host
// polls a pinned copy every few iterations and never sits between kernels.
// Once the stop test fires every later kernel returns at entry.
//
// GB300 runs FP64 at 1/64 of the FP32 rate, so no per-cell work is FP64:
// each thread accumulates a compensated FP32 partial (float fields) and
// only the cross-thread and cross-block reduction tree is FP64.
#include <algorithm>
#include <cstdlib>

#include "pg_cg.cuh"

namespace pg {

constexpr int kCgThreads = 256;

template <class T> __device__ __forceinline__ T rcp_rn(T v);
template <> __device__ __forceinline__ float rcp_rn<float>(float v) { return __frcp_rn(v); }
template <> __device__ __forceinline__ double rcp_rn<double>(double v) { return __drcp_rn(v); }

// z = M^-1 r at one cell for PM_NONE / PM_JACOBI.
// zm: the lazily projected mean of z on the fluid cells (PM_ZBUF; 0 = off).
template <class T, int PM> __device__ __forceinline__ T zval(const T* __restrict__ r, const uint8_t* __restrict__ flags,
                                                             const T* __restrict__ zb, i64 k, T dt, T zm = T(0)) {
    if (PM == PM_JACOBI) {
        const int n = __popc((unsigned)flags[k]);
        return n ? r[k] * rcp_rn<T>((T)n * dt) : T(0);
    }
    if (PM == PM_ZBUF) return flags[k] ? zb[k] - zm : zb[k];
    return r[k];
}

// z for a value already in a register (PM_NONE / PM_JACOBI).
template <class T, int PM> __device__ __forceinline__ T zof(T rv, const uint8_t* __restrict__ flags, i64 k, T dt) {
    if (PM == PM_JACOBI) {
        const int n = __popc((unsigned)flags[k]);
        return n ? rv * rcp_rn<T>((T)n * dt) : T(0);
    }
    return rv;
}

// Last block of the init kernels: ||b||inf, z.r (unless the preconditioner
// publishes it) and the stop threshold into the CG state.
template <class T>
__device__ __forceinline__ void cg_init_finish(CgState* st, double* partials, double* sm, double thr, double rel_tol,
                                               i64 max_iter, double nfluid = 0.0) {
    if (!last_block(&st->counter[0])) return;
    const double bmax = reduce_partials<true, kCgThreads>(partials, gridDim.x, sm);
    const double sigma = reduce_partials<false, kCgThreads>(partials + kMaxBlocks, gridDim.x, sm);
    if (threadIdx.x == 0) {
        st->counter[0] = 0;
        // The stop test compares in T, as pcg.rs:35 / :60 do.
        const double t = (double)(T)(rel_tol > 0.0 ? rel_tol * bmax : thr);
        st->threshold = t;
        st->bmax = bmax;
        st->rmax = bmax;
        st->sigma = sigma;  // PM_ZBUF: sum(b) here, z.r set later by the preconditioner
        st->rsum = sigma;
        st->nfluid = nfluid;
        st->zmean = 0.0;
        st->beta = 0.0;
        st->iter = 0;
        st->max_iter = max_iter;
        st->first = 1;
        st->done = 0;
        st->status = PG_NOT_CONVERGED;
        if (st->nan_seen || !isfinite(sigma)) {
            st->status = PG_NAN_DETECTED;
            st->done = 1;
        } else if ((T)bmax < (T)t || bmax == 0.0) {  // early out, pcg.rs:35-38 (b = 0: x = 0 is exact)
            st->status = PG_OK;
            st->done = 1;
        } else if (max_iter <= 0) {
            st->done = 1;
        }
    }
}

template <class T, int PM>
__global__ void __launch_bounds__(kCgThreads) k_cg_init(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ b,
                                                          const uint8_t* __restrict__ flags, i64 n, T dt, double thr,
                                                          double rel_tol, i64 max_iter, int zero_x, CgState* st,
                                                          double* partials, double nfluid = 0.0) {
    __shared__ double sm[32];
    Acc<T> sig;
    T bm = T(0);
    int bad = 0;
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x) {
        const T bv = b[c];
        if (zero_x) x[c] = T(0);
        r[c] = bv;
        bm = fmax(bm, fabs(bv));
        bad |= !isfinite(bv);
        if (PM != PM_ZBUF) sig.add(zof<T, PM>(bv, flags, c, dt) * bv);
        else sig.add(bv);  // sum(b) for the lazy projection
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&st->nan_seen, 1);
    const double bsum = block_max<kCgThreads>((double)bm, sm);
    const double ssum = block_sum<kCgThreads>(sig.value(), sm);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bsum;
        partials[kMaxBlocks + blockIdx.x] = ssum;
    }
    cg_init_finish<T>(st, partials, sm, thr, rel_tol, max_iter, nfluid);
}

// The init of the MG path on float4 vectors (the V-cycle publishes z.r, so
// the only reduction is the order-independent ||b||inf); n4 = n / 4.  With r
// null (a solve whose first update reads b and writes x afresh) it only
// reduces.
__global__ void __launch_bounds__(kCgThreads)
    k_cg_init4(float4* __restrict__ x, float4* __restrict__ r, const float4* __restrict__ b, i64 n4, double thr,
               double rel_tol, i64 max_iter, int zero_x, CgState* st, double* partials, double nfluid,
               float4* __restrict__ xl) {
    __shared__ double sm[32];
    float bm = 0.f;
    int bad = 0;
    float sb = 0.f;  // sum(b) for the lazy projection (feeds a small correction term)
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n4; c += (i64)gridDim.x * blockDim.x) {
        const float4 bv = b[c];
        if (zero_x) {
            x[c] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (xl) xl[c] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        if (r) r[c] = bv;
        bm = fmaxf(fmaxf(fmaxf(bm, fabsf(bv.x)), fmaxf(fabsf(bv.y), fabsf(bv.z))), fabsf(bv.w));
        bad |= !isfinite(bv.x) | !isfinite(bv.y) | !isfinite(bv.z) | !isfinite(bv.w);
        sb += (bv.x + bv.y) + (bv.z + bv.w);
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&st->nan_seen, 1);
    const double bsum = block_max<kCgThreads>((double)bm, sm);
    const double ssum = block_sum<kCgThreads>((double)sb, sm);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bsum;
        partials[kMaxBlocks + blockIdx.x] = ssum;
    }
    cg_init_finish<float>(st, partials, sm, thr, rel_tol, max_iter, nfluid);
}

// Fused search-direction update and operator application.
template <class T, int ND, int PM>
__global__ void __launch_bounds__(kCgThreads)
    k_cg_spmv(const T* __restrict__ r, const T* __restrict__ zb, T* p0, T* p1, T* __restrict__ ap,
              const uint8_t* __restrict__ flags, Dims D, T dt, CgState* st, double* partials) {
    if (st->done) return;
    __shared__ double sm[32];
    // Ping-pong by the device-side iteration count: iteration k reads
    // p[k & 1] and writes p[(k + 1) & 1] (so a CUDA graph can replay it).
    const i64 k = *(volatile const i64*)&st->iter;
    const T* __restrict__ p_old = (k & 1) ? p1 : p0;
    T* __restrict__ p_new = (k & 1) ? p0 : p1;
    const int first = st->first;
    const T beta = first ? T(0) : (T)st->beta;
    const T zm = (PM == PM_ZBUF && st->nfluid > 0.0) ? (T)st->zmean : T(0);
    const i64 n = D.nc(), w = D.w, hw = D.h * D.w;
    auto pn = [&](i64 k) -> T {
        const T z = zval<T, PM>(r, flags, zb, k, dt, zm);
        return first ? z : z + beta * p_old[k];
    };
    Acc<T> acc;
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x) {
        const uint8_t f = flags[c];
        const T pc = pn(c);
        p_new[c] = pc;
        // Reference operator order (grid.rs:295-335 after *1^-1).
        const T gy_lo = (f & YLO) ? -sub_rn(pc, pn(c - w)) : T(0);
        const T gy_hi = (f & YHI) ? -sub_rn(pn(c + w), pc) : T(0);
        const T gx_lo = (f & XLO) ? sub_rn(pn(c - 1), pc) : T(0);
        const T gx_hi = (f & XHI) ? sub_rn(pc, pn(c + 1)) : T(0);
        T v = add_rn(sub_rn(sub_rn(gy_hi, gy_lo), gx_lo), gx_hi);
        if (ND == 3) {
            const T gz_lo = (f & ZLO) ? -sub_rn(pc, pn(c - hw)) : T(0);
            const T gz_hi = (f & ZHI) ? -sub_rn(pn(c + hw), pc) : T(0);
            v = add_rn(sub_rn(v, gz_lo), gz_hi);
        }
        const T a = mul_rn(v, dt);
        ap[c] = a;
        acc.add(pc * a);
    }
    const double s = block_sum<kCgThreads>(acc.value(), sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    if (!last_block(&st->counter[1])) return;
    const double pap = reduce_partials<false, kCgThreads>(partials, gridDim.x, sm);
    if (threadIdx.x == 0) {
        st->counter[1] = 0;
        st->pap = pap;
        if (!isfinite(pap)) {
            st->status = PG_NAN_DETECTED;
            st->done = 1;
        } else if (!(pap > 0.0)) {
            st->status = st->sigma == 0.0 ? PG_NOT_CONVERGED : PG_BREAKDOWN;
            st->done = 1;
        } else {
            st->alpha = st->sigma / pap;  // pcg.rs:53
        }
    }
}

// The same fused SpMV for 3D grids as a z-marching 2.5D tile: a block owns
// a 32 x 8 column tile and walks a chunk of z planes; each cell's inputs are
// loaded once, its x/y neighbours come from a shared-memory plane tile (with
// a one-cell halo the edge threads fill), its z neighbours from the
// registers of the planes below and above.  Work items (tile, z chunk) are
// handed out grid-stride, so the block count (and the reduction partials)
// stays bounded for any grid size.  Same arithmetic as k_cg_spmv.
constexpr int kTX = 32, kTY = 8;

template <class T, int PM>
__global__ void __launch_bounds__(kTX * kTY)
    k_cg_spmv3t(const T* __restrict__ r, const T* __restrict__ zb, T* p0, T* p1, T* __restrict__ ap,
                const uint8_t* __restrict__ flags, Dims D, T dt, CgState* st, double* partials, int tiles_x,
                int tiles_y, int zc, int nwork) {
    if (st->done) return;
    __shared__ T S[kTY + 2][kTX + 2];
    __shared__ double sm[32];
    const i64 kit = *(volatile const i64*)&st->iter;
    const T* __restrict__ p_old = (kit & 1) ? p1 : p0;
    T* __restrict__ p_new = (kit & 1) ? p0 : p1;
    const int first = st->first;
    const T beta = first ? T(0) : (T)st->beta;
    const T zm = (PM == PM_ZBUF && st->nfluid > 0.0) ? (T)st->zmean : T(0);
    auto pn = [&](i64 k) -> T {
        const T z = zval<T, PM>(r, flags, zb, k, dt, zm);
        return first ? z : z + beta * p_old[k];
    };
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    const int w = (int)D.w, h = (int)D.h, d = (int)D.d;
    const i64 hw = (i64)h * w;
    const int per_plane = tiles_x * tiles_y;
    Acc<T> acc;
    for (int item = blockIdx.x; item < nwork; item += gridDim.x) {
        const int tz = item / per_plane, t2 = item - tz * per_plane;
        const int x = (t2 % tiles_x) * kTX + tx, y = (t2 / tiles_x) * kTY + ty;
        const int z0 = tz * zc, z1 = min(z0 + zc, d);
        const bool inside = x < w && y < h;
        const i64 col = (i64)y * w + x;
        T below = T(0), cur = T(0), above = T(0);
        if (inside) {
            if (z0 > 0) below = pn((i64)(z0 - 1) * hw + col);
            cur = pn((i64)z0 * hw + col);
            if (z0 + 1 < d) above = pn((i64)(z0 + 1) * hw + col);
        }
        for (int z = z0; z < z1; ++z) {
            const i64 c = (i64)z * hw + col;
            // Loads for plane z + 2 are issued here and combined only after
            // this plane's stencil, so their latency overlaps the step.
            T rz = T(0), rp = T(0);
            if (inside && z + 2 < d && z + 1 < z1) {
                rz = zval<T, PM>(r, flags, zb, c + 2 * hw, dt, zm);
                if (!first) rp = p_old[c + 2 * hw];
            }
            S[ty + 1][tx + 1] = cur;
            if (inside) {
                if (tx == 0 && x > 0) S[ty + 1][0] = pn(c - 1);
                if (tx == kTX - 1 && x + 1 < w) S[ty + 1][kTX + 1] = pn(c + 1);
                if (ty == 0 && y > 0) S[0][tx + 1] = pn(c - w);
                if (ty == kTY - 1 && y + 1 < h) S[kTY + 1][tx + 1] = pn(c + w);
            }
            __syncthreads();
            if (inside) {
                const uint8_t f = flags[c];
                const T pc = cur;
                const T gy_lo = (f & YLO) ? -sub_rn(pc, S[ty][tx + 1]) : T(0);
                const T gy_hi = (f & YHI) ? -sub_rn(S[ty + 2][tx + 1], pc) : T(0);
                const T gx_lo = (f & XLO) ? sub_rn(S[ty + 1][tx], pc) : T(0);
                const T gx_hi = (f & XHI) ? sub_rn(pc, S[ty + 1][tx + 2]) : T(0);
                T v = add_rn(sub_rn(sub_rn(gy_hi, gy_lo), gx_lo), gx_hi);
                const T gz_lo = (f & ZLO) ? -sub_rn(pc, below) : T(0);
                const T gz_hi = (f & ZHI) ? -sub_rn(above, pc) : T(0);
                v = add_rn(sub_rn(v, gz_lo), gz_hi);
                const T a = mul_rn(v, dt);
                p_new[c] = pc;
                ap[c] = a;
                acc.add(pc * a);
            }
            __syncthreads();
            below = cur;
            cur = above;
            above = first ? rz : rz + beta * rp;
        }
    }
    const double s = block_sum<kTX * kTY>(acc.value(), sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    if (!last_block(&st->counter[1])) return;
    const double pap = reduce_partials<false, kTX * kTY>(partials, gridDim.x, sm);
    if (threadIdx.x == 0) {
        st->counter[1] = 0;
        st->pap = pap;
        if (!isfinite(pap)) {
            st->status = PG_NAN_DETECTED;
            st->done = 1;
        } else if (!(pap > 0.0)) {
            st->status = st->sigma == 0.0 ? PG_NOT_CONVERGED : PG_BREAKDOWN;
            st->done = 1;
        } else {
            st->alpha = st->sigma / pap;  // pcg.rs:53
        }
    }
}

// Launch the fused SpMV: the TMA-staged z-marching kernel for 3D float grids
// where it applies (tma = true), else the 2.5D tile for 3D grids and the
// flat grid-stride kernel for 2D.  Shared by every CG entry point.
template <class T, int PM>
static void spmv_launch(cudaStream_t s, int num_sms, const T* r, const T* zb, T* p0, T* p1, T* ap,
                        const uint8_t* flags, const Dims& D, T dt, CgState* st, double* partials, int nb_flat,
                        bool tma = true) {
    if (tma && sizeof(T) == 4 &&
        spmv_tma_launch(s, num_sms, PM, (const float*)(PM == PM_ZBUF ? zb : r), (float*)p0, (float*)p1, (float*)ap,
                        flags, D, (float)dt, st, partials))
        return;
    if (D.nd == 3) {
        const int tiles_x = (int)((D.w + kTX - 1) / kTX), tiles_y = (int)((D.h + kTY - 1) / kTY);
        const int cap = std::min(num_sms * 8, kMaxBlocks);
        // about two work items per resident block, at least 4 planes each
        const i64 want_chunks = std::max<i64>(1, (2 * (i64)cap + tiles_x * tiles_y - 1) / ((i64)tiles_x * tiles_y));
        const int zc = (int)std::max<i64>(4, (D.d + want_chunks - 1) / want_chunks);
        const int nwork = tiles_x * tiles_y * (int)((D.d + zc - 1) / zc);
        const int nb = std::max(1, std::min(nwork, cap));
        k_cg_spmv3t<T, PM><<<nb, kTX * kTY, 0, s>>>(r, zb, p0, p1, ap, flags, D, dt, st, partials, tiles_x, tiles_y,
                                                    zc, nwork);
    } else {
        k_cg_spmv<T, 2, PM><<<nb_flat, kCgThreads, 0, s>>>(r, zb, p0, p1, ap, flags, D, dt, st, partials);
    }
}

template <class T, int PM>
__global__ void __launch_bounds__(kCgThreads)
    k_cg_update(T* __restrict__ x, T* __restrict__ r, const T* p0, const T* p1, const T* __restrict__ ap,
                const uint8_t* __restrict__ flags, i64 n, T dt, CgState* st, double* partials) {
    if (st->done) return;
    __shared__ double sm[32];
    // The SpMV of this iteration wrote p[(iter + 1) & 1]; the last block
    // increments iter only after every block has read it here.
    const i64 k = *(volatile const i64*)&st->iter;
    const T* __restrict__ p = ((k + 1) & 1) ? p1 : p0;
    const T alpha = (T)st->alpha, nalpha = -alpha;
    T rm = T(0);
    Acc<T> rz;
    int bad = 0;
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x) {
        x[c] = x[c] + alpha * p[c];          // pcg.rs:55
        const T rv = r[c] + nalpha * ap[c];  // pcg.rs:56
        r[c] = rv;
        rm = fmax(rm, fabs(rv));
        bad |= !isfinite(rv);
        if (PM != PM_ZBUF) rz.add(zof<T, PM>(rv, flags, c, dt) * rv);
        else rz.add(rv);  // sum(r) for the lazy projection
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&st->nan_seen, 1);
    const double m = block_max<kCgThreads>((double)rm, sm);
    const double s = block_sum<kCgThreads>(rz.value(), sm);
    if (threadIdx.x == 0) {
        partials[2 * kMaxBlocks + blockIdx.x] = m;
        partials[3 * kMaxBlocks + blockIdx.x] = s;
    }
    if (!last_block(&st->counter[2])) return;
    const double rmax = reduce_partials<true, kCgThreads>(partials + 2 * kMaxBlocks, gridDim.x, sm);
    const double sigma_new = reduce_partials<false, kCgThreads>(partials + 3 * kMaxBlocks, gridDim.x, sm);
    if (threadIdx.x == 0) {
        st->counter[2] = 0;
        const i64 it = st->iter + 1;
        st->iter = it;
        st->rmax = rmax;
        if (st->nan_seen || !isfinite(rmax)) {
            st->status = PG_NAN_DETECTED;
            st->done = 1;
        } else if ((T)rmax < (T)st->threshold) {  // pcg.rs:58-63
            st->status = PG_OK;
            st->done = 1;
        } else {
            if (PM != PM_ZBUF) cg_finish_rz(st, sigma_new);  // pcg.rs:65-68
            else st->rsum = sigma_new;
            if (it >= st->max_iter) st->done = 1;          // loop bound, pcg.rs:48
        }
    }
}

// x + alpha p into the double-float pair (xh, xl): the product's rounding
// error (fma) and the sum's (TwoSum) both go into the low part, so the
// iterate carries the sum of its increments to ~48 bits.
__device__ __forceinline__ void df_axpy(float& xh, float& xl, float alpha, float p) {
    const float d = __fmul_rn(alpha, p);
    const float de = __fmaf_rn(alpha, p, -d);
    const float s = __fadd_rn(xh, d);
    const float bb = __fsub_rn(s, xh);
    const float e = __fadd_rn(__fsub_rn(xh, __fsub_rn(s, bb)), __fsub_rn(d, bb));
    const float lo = __fadd_rn(xl, __fadd_rn(e, de));
    const float h2 = __fadd_rn(s, lo);
    xh = h2;
    xl = __fsub_rn(lo, __fsub_rn(h2, s));
}

// The update of the MG path (z.r comes from the V-cycle, so the only
// reduction is the order-independent ||r||inf) on float4 vectors, two per
// thread and iteration: eight cells' x, p, r, Ap in flight per thread.  Same
// per-cell arithmetic as k_cg_update<float, PM_ZBUF>; n4 = n / 4.  With DFX
// the iterate is the double-float pair (x, xl), updated by df_axpy.  With b0
// set, iteration 0 reads r = b0 and x = xl = 0 without loading them (the
// init then writes neither): the same values, 16 bytes per cell fewer.
template <bool DFX>
__global__ void __launch_bounds__(kCgThreads)
    k_cg_update4(float4* __restrict__ x, float4* __restrict__ r, const float4* p0, const float4* p1,
                 const float4* __restrict__ ap, i64 n4, CgState* st, double* partials, float4* __restrict__ xl,
                 const float4* __restrict__ b0) {
    if (st->done) return;
    __shared__ double sm[32];
    const i64 k = *(volatile const i64*)&st->iter;
    const float4* __restrict__ p = ((k + 1) & 1) ? p1 : p0;
    const float alpha = (float)st->alpha, nalpha = -alpha;
    const bool first = b0 != nullptr && k == 0;  // uniform
    const float4* __restrict__ rin = first ? b0 : r;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float rm = 0.f, rs = 0.f;  // rs: sum(r) for the lazy projection (feeds a small correction term)
    int bad = 0;
    auto one = [&](i64 c) {
        const float4 xv = first ? zero4 : x[c], pv = p[c], rv = rin[c], av = ap[c];
        float4 xo, ro;
        if (DFX) {
            float4 lo = first ? zero4 : xl[c];
            xo = xv;
            df_axpy(xo.x, lo.x, alpha, pv.x);
            df_axpy(xo.y, lo.y, alpha, pv.y);
            df_axpy(xo.z, lo.z, alpha, pv.z);
            df_axpy(xo.w, lo.w, alpha, pv.w);
            xl[c] = lo;
        } else {
            xo.x = xv.x + alpha * pv.x;
            xo.y = xv.y + alpha * pv.y;
            xo.z = xv.z + alpha * pv.z;
            xo.w = xv.w + alpha * pv.w;
        }
        ro.x = rv.x + nalpha * av.x;
        ro.y = rv.y + nalpha * av.y;
        ro.z = rv.z + nalpha * av.z;
        ro.w = rv.w + nalpha * av.w;
        x[c] = xo;
        r[c] = ro;
        rm = fmaxf(fmaxf(fmaxf(rm, fabsf(ro.x)), fmaxf(fabsf(ro.y), fabsf(ro.z))), fabsf(ro.w));
        bad |= !isfinite(ro.x) | !isfinite(ro.y) | !isfinite(ro.z) | !isfinite(ro.w);
        rs += (ro.x + ro.y) + (ro.z + ro.w);
    };
    const i64 stride = (i64)gridDim.x * blockDim.x;
    i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    for (; c + stride < n4; c += 2 * stride) {
        one(c);
        one(c + stride);
    }
    if (c < n4) one(c);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&st->nan_seen, 1);
    const double m = block_max<kCgThreads>((double)rm, sm);
    const double rsb = block_sum<kCgThreads>((double)rs, sm);
    if (threadIdx.x == 0) {
        partials[2 * kMaxBlocks + blockIdx.x] = m;
        partials[3 * kMaxBlocks + blockIdx.x] = rsb;
    }
    if (!last_block(&st->counter[2])) return;
    const double rmax = reduce_partials<true, kCgThreads>(partials + 2 * kMaxBlocks, gridDim.x, sm);
    const double rsum = reduce_partials<false, kCgThreads>(partials + 3 * kMaxBlocks, gridDim.x, sm);
    if (threadIdx.x == 0) {
        st->rsum = rsum;
        st->counter[2] = 0;
        const i64 it = st->iter + 1;
        st->iter = it;
        st->rmax = rmax;
        if (st->nan_seen || !isfinite(rmax)) {
            st->status = PG_NAN_DETECTED;
            st->done = 1;
        } else if ((float)rmax < (float)st->threshold) {  // pcg.rs:58-63
            st->status = PG_OK;
            st->done = 1;
        } else if (it >= st->max_iter) {  // loop bound, pcg.rs:48
            st->done = 1;
        }
    }
}

// The update of the identity / Jacobi CG on float4 vectors, two per thread
// and iteration (eight cells' x, p, r, Ap in flight per thread): the same
// per-cell arithmetic as k_cg_update<float, PM> and the same compensated
// FP32 partial of z.r per thread (summed in a different order); Jacobi reads
// the cells' face-open bits four at a time.  n4 = n / 4.
template <int PM>
__global__ void __launch_bounds__(kCgThreads)
    k_cg_update4r(float4* __restrict__ x, float4* __restrict__ r, const float4* p0, const float4* p1,
                  const float4* __restrict__ ap, const uchar4* __restrict__ flags, i64 n4, float dt, CgState* st,
                  double* partials) {
    if (st->done) return;
    __shared__ double sm[32];
    __shared__ float inv_diag[8];  // Jacobi: 1 / (n dt) for n open faces (0 for n = 0), as zof computes it
    if (PM == PM_JACOBI) {
        if (threadIdx.x < 8) inv_diag[threadIdx.x] = threadIdx.x ? __frcp_rn((float)threadIdx.x * dt) : 0.f;
        __syncthreads();
    }
    const i64 k = *(volatile const i64*)&st->iter;
    const float4* __restrict__ p = ((k + 1) & 1) ? p1 : p0;
    const float alpha = (float)st->alpha, nalpha = -alpha;
    float rm = 0.f;
    Acc<float> rz;
    int bad = 0;
    auto zr = [&](float rv, unsigned f) {
        if (PM == PM_JACOBI) {
            const float z = f ? rv * inv_diag[__popc(f)] : 0.f;
            rz.add(z * rv);
        } else {
            rz.add(rv * rv);
        }
    };
    auto one = [&](i64 c) {
        const float4 xv = x[c], pv = p[c], rv = r[c], av = ap[c];
        uchar4 f = make_uchar4(0, 0, 0, 0);
        if (PM == PM_JACOBI) f = flags[c];
        float4 xo, ro;
        xo.x = xv.x + alpha * pv.x;  // pcg.rs:55
        xo.y = xv.y + alpha * pv.y;
        xo.z = xv.z + alpha * pv.z;
        xo.w = xv.w + alpha * pv.w;
        ro.x = rv.x + nalpha * av.x;  // pcg.rs:56
        ro.y = rv.y + nalpha * av.y;
        ro.z = rv.z + nalpha * av.z;
        ro.w = rv.w + nalpha * av.w;
        x[c] = xo;
        r[c] = ro;
        rm = fmaxf(fmaxf(fmaxf(rm, fabsf(ro.x)), fmaxf(fabsf(ro.y), fabsf(ro.z))), fabsf(ro.w));
        bad |= !isfinite(ro.x) | !isfinite(ro.y) | !isfinite(ro.z) | !isfinite(ro.w);
        zr(ro.x, f.x);
        zr(ro.y, f.y);
        zr(ro.z, f.z);
        zr(ro.w, f.w);
    };
    const i64 stride = (i64)gridDim.x * blockDim.x;
    i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    for (; c + stride < n4; c += 2 * stride) {
        one(c);
        one(c + stride);
    }
    if (c < n4) one(c);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&st->nan_seen, 1);
    const double m = block_max<kCgThreads>((double)rm, sm);
    const double s = block_sum<kCgThreads>(rz.value(), sm);
    if (threadIdx.x == 0) {
        partials[2 * kMaxBlocks + blockIdx.x] = m;
        partials[3 * kMaxBlocks + blockIdx.x] = s;
    }
    if (!last_block(&st->counter[2])) return;
    const double rmax = reduce_partials<true, kCgThreads>(partials + 2 * kMaxBlocks, gridDim.x, sm);
    const double sigma_new = reduce_partials<false, kCgThreads>(partials + 3 * kMaxBlocks, gridDim.x, sm);
    if (threadIdx.x == 0) {
        st->counter[2] = 0;
        const i64 it = st->iter + 1;
        st->iter = it;
        st->rmax = rmax;
        if (st->nan_seen || !isfinite(rmax)) {
            st->status = PG_NAN_DETECTED;
            st->done = 1;
        } else if ((float)rmax < (float)st->threshold) {  // pcg.rs:58-63
            st->status = PG_OK;
            st->done = 1;
        } else {
            cg_finish_rz(st, sigma_new);            // pcg.rs:65-68
            if (it >= st->max_iter) st->done = 1;  // loop bound, pcg.rs:48
        }
    }
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

template <class T>
static bool cg_dfx_ok(const CgBuffers<T>& buf, i64 n, const uint8_t* flags) {
    return sizeof(T) == 4 && n % 4 == 0 && aligned16(buf.x) && aligned16(buf.xl) && aligned16(buf.r) &&
           aligned16(buf.b) && aligned16(buf.p[0]) && aligned16(buf.p[1]) && aligned16(buf.ap) && aligned16(flags);
}

// A double-float solve starts from x = 0: its first update reads b in place
// of r and writes x, xl afresh, so the init writes none of r, x, xl -- unless
// the preconditioner writes its input (then r must be a copy of b).
template <class T>
static bool cg_fold(const CgBuffers<T>& buf, const ZHook* hook) {
    return buf.xl != nullptr && hook != nullptr && !hook->writes_input();
}

bool cg_dfx_supported(const pg_grid* g, const CgBuffers<float>& buf) {
    const char* env = getenv("PG_CG_DFX");
    if (env && env[0] == '0') return false;
    return cg_dfx_ok(buf, g->dims.nc(), g->flags);
}

// After max_iterations the reference has already run aux = M r and
// search = aux + beta*search (pcg.rs:65-77); reproduce that tail.
template <class T, int PM>
__global__ void k_cg_tail(const T* __restrict__ r, const T* __restrict__ p, T* __restrict__ aux, T* __restrict__ search,
                          const uint8_t* __restrict__ flags, i64 n, T dt, const CgState* st) {
    const T beta = (T)st->beta;
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x) {
        const T z = zof<T, PM>(r[c], flags, c, dt);
        const T pv = p[c];
        aux[c] = z;
        search[c] = z + beta * pv;
    }
}

// The identity / Jacobi CG takes the TMA-staged SpMV unless PG_CG_TMA=0 (a
// diagnostic switch, read per launch sequence: a grid's cached CG graphs keep
// the choice they were captured with).
static bool cg_tma_enabled() {
    const char* env = getenv("PG_CG_TMA");
    return !(env && env[0] == '0');
}

// The update of the identity / Jacobi CG: the float4 kernel where every
// vector and the flags are 16-byte aligned and the cell count is a multiple
// of 4, else the scalar kernel.  Every entry point of that CG launches its
// update here, so they compute the same iterates on the same buffers.
template <class T, int PM>
static void update_launch(cudaStream_t s, int nb, T* x, T* r, const T* p0, const T* p1, const T* ap,
                          const uint8_t* flags, i64 n, T dt, CgState* st, double* partials) {
    const bool vec4 = sizeof(T) == 4 && n % 4 == 0 && aligned16(x) && aligned16(r) && aligned16(p0) &&
                      aligned16(p1) && aligned16(ap) && aligned16(flags);
    if (vec4)
        k_cg_update4r<PM><<<nb, kCgThreads, 0, s>>>((float4*)x, (float4*)r, (const float4*)p0, (const float4*)p1,
                                                    (const float4*)ap, (const uchar4*)flags, n / 4, (float)dt, st,
                                                    partials);
    else
        k_cg_update<T, PM><<<nb, kCgThreads, 0, s>>>(x, r, p0, p1, ap, flags, n, dt, st, partials);
}

template <class T, int PM>
static void launch_iter(pg_grid* g, const CgBuffers<T>& buf, T dt, int nb, ZHook* hook) {
    const Dims& D = g->dims;
    cudaStream_t s = g->stream;
    PG_LAUNCH(KK_CG_SPMV, s,
              spmv_launch<T, PM>(s, g->num_sms, buf.r, buf.z, buf.p[0], buf.p[1], buf.ap, g->flags, D, dt,
                                 g->ws.state, g->ws.partials, nb, PM == PM_ZBUF || cg_tma_enabled()));
    const i64 n = D.nc();
    const bool vec4 = sizeof(T) == 4 && n % 4 == 0 && aligned16(buf.x) && aligned16(buf.r) &&
                      aligned16(buf.p[0]) && aligned16(buf.p[1]) && aligned16(buf.ap) && aligned16(g->flags);
    if (PM == PM_ZBUF && vec4 && buf.xl)
        PG_LAUNCH(KK_CG_UPDATE, s,
                  k_cg_update4<true><<<nb, kCgThreads, 0, s>>>(
                      (float4*)buf.x, (float4*)buf.r, (const float4*)buf.p[0], (const float4*)buf.p[1],
                      (const float4*)buf.ap, n / 4, g->ws.state, g->ws.partials, (float4*)buf.xl,
                      cg_fold(buf, hook) ? (const float4*)buf.b : nullptr));
    else if (PM == PM_ZBUF && vec4)
        PG_LAUNCH(KK_CG_UPDATE, s,
                  k_cg_update4<false><<<nb, kCgThreads, 0, s>>>((float4*)buf.x, (float4*)buf.r,
                                                                (const float4*)buf.p[0], (const float4*)buf.p[1],
                                                                (const float4*)buf.ap, n / 4, g->ws.state,
                                                                g->ws.partials, nullptr, nullptr));
    else if (PM != PM_ZBUF)
        PG_LAUNCH(KK_CG_UPDATE, s,
                  update_launch<T, PM>(s, nb, buf.x, buf.r, buf.p[0], buf.p[1], buf.ap, g->flags, n, dt, g->ws.state,
                                       g->ws.partials));
    else
        PG_LAUNCH(KK_CG_UPDATE, s,
                  k_cg_update<T, PM><<<nb, kCgThreads, 0, s>>>(buf.x, buf.r, buf.p[0], buf.p[1], buf.ap, g->flags, n,
                                                               dt, g->ws.state, g->ws.partials));
    if (PM == PM_ZBUF) hook->apply(g, buf.r, buf.z);
}

// ---------------------------------------------------------------------------
// CUDA-graph form of the iteration loop: a WHILE conditional node whose body
// is one iteration (SpMV, update, the outer preconditioner's kernels) and a
// one-thread kernel that clears the condition once the device-side stop
// test has fired.  No host round trip and no launch past convergence.
__global__ void k_cg_cond(const CgState* st, cudaGraphConditionalHandle h) {
    cudaGraphSetConditional(h, st->done ? 0u : 1u);
}

struct CgGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const void* key[9] = {};
    double dt = 0.0;
    int pm = -1, nd = 0;
    uintptr_t hook_key = 0;
    int body_kernels = 0;
};

struct CgGraphCache {
    static constexpr int kSlots = 8;
    CgGraph e[kSlots];
    int next = 0;
    ~CgGraphCache() {
        for (auto& x : e) {
            if (x.exec) cudaGraphExecDestroy(x.exec);
            if (x.graph) cudaGraphDestroy(x.graph);
        }
    }
};

void release_cg_graphs(pg_grid* g) {
    delete (CgGraphCache*)g->ws.graphs;
    g->ws.graphs = nullptr;
}

template <class T, int PM>
static int get_graph(pg_grid* g, const CgBuffers<T>& buf, T dt, int nb, ZHook* hook, CgGraph** out) {
    if (!g->ws.graphs) g->ws.graphs = new CgGraphCache();
    CgGraphCache* C = (CgGraphCache*)g->ws.graphs;
    const void* key[9] = {buf.x, buf.b, buf.r, buf.ap, buf.p[0], buf.p[1], buf.z, g->flags, buf.xl};
    const uintptr_t hk = hook ? hook->key() : 0;
    for (auto& e : C->e) {
        if (e.exec && e.pm == PM && e.dt == (double)dt && e.nd == g->dims.nd && e.hook_key == hk &&
            std::equal(key, key + 9, e.key)) {
            *out = &e;
            return PG_OK;
        }
    }
    CgGraph& E = C->e[C->next];
    C->next = (C->next + 1) % CgGraphCache::kSlots;
    if (E.exec) cudaGraphExecDestroy(E.exec);
    if (E.graph) cudaGraphDestroy(E.graph);
    E = CgGraph();
    PG_CUDA(cudaGraphCreate(&E.graph, 0));
    cudaGraphConditionalHandle h;
    PG_CUDA(cudaGraphConditionalHandleCreate(&h, E.graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    PG_CUDA(cudaGraphAddNode(&node, E.graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaStream_t cs;
    PG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaStream_t saved = g->stream;
    g->stream = cs;
    const int64_t before = prof_capture_begin();
    cudaError_t err = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (err == cudaSuccess) {
        launch_iter<T, PM>(g, buf, dt, nb, hook);
        k_cg_cond<<<1, 1, 0, cs>>>(g->ws.state, h);
        cudaGraph_t captured = nullptr;
        err = cudaStreamEndCapture(cs, &captured);
    }
    E.body_kernels = (int)(prof_capture_end() - before) + 1;
    g->stream = saved;
    cudaStreamDestroy(cs);
    if (err != cudaSuccess) {
        cudaGraphDestroy(E.graph);
        E = CgGraph();
        return cuda_fail(err, "CG graph capture");
    }
    PG_CUDA(cudaGraphInstantiate(&E.exec, E.graph, 0));
    std::copy(key, key + 9, E.key);
    E.pm = PM;
    E.dt = (double)dt;
    E.nd = g->dims.nd;
    E.hook_key = hk;
    *out = &E;
    return PG_OK;
}

template <class T, int PM>
static int run_cg_pm(pg_grid* g, const CgConfig& cfg, CgBuffers<T> buf, pg_pcg_stats* stats, ZHook* hook) {
    int rc = ensure_workspace(g);
    if (rc) return rc;
    const Dims& D = g->dims;
    const i64 n = D.nc();
    const T dt = (T)cfg.dt;
    const int nb = grid_blocks(g, n, kCgThreads, 8);
    Workspace& ws = g->ws;
    cudaStream_t s = g->stream;
    // The double-float iterate exists only in the float4 kernels.
    if (buf.xl && (PM != PM_ZBUF || !cg_dfx_ok(buf, n, g->flags)))
        return bad_arg("run_cg: a double-float iterate needs the float4 MG path");
    PG_CUDA(cudaMemsetAsync(ws.state, 0, sizeof(CgState), s));
    const bool fold = PM == PM_ZBUF && cg_fold(buf, hook);
    if (PM == PM_ZBUF && sizeof(T) == 4 && n % 4 == 0 && aligned16(buf.x) && aligned16(buf.r) && aligned16(buf.b))
        PG_LAUNCH(KK_CG_INIT, s,
                  k_cg_init4<<<nb, kCgThreads, 0, s>>>((float4*)buf.x, fold ? nullptr : (float4*)buf.r,
                                                       (const float4*)buf.b, n / 4, cfg.threshold, cfg.rel_tol,
                                                       cfg.max_iter, fold ? 0 : cfg.zero_x, ws.state, ws.partials,
                                                       cfg.nfluid, (float4*)buf.xl));
    else
        PG_LAUNCH(KK_CG_INIT, s,
              k_cg_init<T, PM><<<nb, kCgThreads, 0, s>>>(buf.x, buf.r, buf.b, g->flags, n, dt, cfg.threshold,
                                                         cfg.rel_tol, cfg.max_iter, cfg.zero_x, ws.state,
                                                         ws.partials, cfg.nfluid));
    PG_CHECK_LAUNCH();
    if (PM == PM_ZBUF) hook->bind(buf.ap);
    if (PM == PM_ZBUF && (rc = hook->apply(g, fold ? (const void*)buf.b : (const void*)buf.r, buf.z))) return rc;
    // Device-side loop: one graph launch runs every iteration.
    CgGraph* G = nullptr;
    if (graphs_enabled() && cfg.max_iter > 0) {
        if ((rc = get_graph<T, PM>(g, buf, dt, nb, hook, &G))) return rc;
        PG_CUDA(cudaGraphLaunch(G->exec, s));
    }
    // Host-polled loop (profiling mode): chunks of about 0.5 ms of device
    // work, two in flight; iterations past the stop test exit at entry.
    int chunk = cfg.check_every;
    if (chunk <= 0) {
        double us_per_iter = 4.0 + (double)n * 41.0 / 5.0e6;  // launch floor + HBM time
        if (PM == PM_ZBUF) us_per_iter = 3.0 * us_per_iter + 100.0;
        chunk = (int)std::min(64.0, std::max(2.0, 600.0 / us_per_iter));
    }
    i64 launched = 0;
    int slot = 0, pending = -1;
    bool done = G != nullptr;
    while (!done && launched < cfg.max_iter) {
        const i64 todo = std::min<i64>(chunk, cfg.max_iter - launched);
        for (i64 k = 0; k < todo; ++k) launch_iter<T, PM>(g, buf, dt, nb, hook);
        PG_CHECK_LAUNCH();
        launched += todo;
        PG_CUDA(cudaMemcpyAsync(ws.state_host + slot, ws.state, sizeof(CgState), cudaMemcpyDeviceToHost, s));
        PG_CUDA(cudaEventRecord(ws.ev[slot], s));
        if (pending >= 0) {
            PG_CUDA(cudaEventSynchronize(ws.ev[pending]));
            done = ws.state_host[pending].done != 0;
        }
        pending = slot;
        slot ^= 1;
    }
    static_assert(sizeof(CgState) % 4 == 0, "CgState words");
    k_words_out<<<1, 64, 0, s>>>((const unsigned*)ws.state, (unsigned*)(ws.state_host + 2),
                                 (int)(sizeof(CgState) / 4));
    PG_CHECK_LAUNCH();
    PG_CUDA(cudaStreamSynchronize(s));
    const CgState st = ws.state_host[2];
    if (G) prof_add_launches((int64_t)G->body_kernels * std::max<i64>(st.iter, 1));
    if (stats) {
        stats->iterations = st.iter;
        stats->refinements = 0;
        stats->residual_max = st.rmax;
        stats->b_max = st.bmax;
        stats->threshold = st.threshold;
        stats->true_residual_max = -1.0;
        stats->status = st.status;
    }
    return PG_OK;
}

template <class T>
int run_cg(pg_grid* g, const CgConfig& cfg, CgBuffers<T> buf, pg_pcg_stats* stats, ZHook* hook) {
    if (cfg.precond == PG_PRECOND_MG) {
        if (!hook || !buf.z) return bad_arg("run_cg: MG preconditioning needs a hook and a z buffer");
        return run_cg_pm<T, PM_ZBUF>(g, cfg, buf, stats, hook);
    }
    if (cfg.precond == PG_PRECOND_JACOBI) return run_cg_pm<T, PM_JACOBI>(g, cfg, buf, stats, nullptr);
    return run_cg_pm<T, PM_NONE>(g, cfg, buf, stats, nullptr);
}

template int run_cg<float>(pg_grid*, const CgConfig&, CgBuffers<float>, pg_pcg_stats*, ZHook*);
template int run_cg<double>(pg_grid*, const CgConfig&, CgBuffers<double>, pg_pcg_stats*, ZHook*);

// pg_pcg_*: the reference signature with caller-owned work vectors.
template <class T>
static int pcg_abi(const pg_grid* cg, int precond, T* x, const T* b, int64_t max_iter, double threshold, T* residual,
                   T* auxiliary, T* search, double dt, pg_pcg_stats* stats) {
    if (!cg || !x || !b || !residual || !auxiliary || !search) return bad_arg("pg_pcg: NULL argument");
    if (precond != PG_PRECOND_NONE && precond != PG_PRECOND_JACOBI)
        return bad_arg("pg_pcg: precond must be PG_PRECOND_NONE or PG_PRECOND_JACOBI");
    if (max_iter < 0) return bad_arg("pg_pcg: max_iterations < 0");
    pg_grid* g = const_cast<pg_grid*>(cg);
    const i64 n = g->dims.nc();
    int rc = ensure_vec(g, sizeof(T) * (size_t)n);
    if (rc) return rc;
    CgBuffers<T> buf;
    buf.x = x;
    buf.b = b;
    buf.r = residual;
    buf.ap = auxiliary;
    buf.p[0] = (T*)g->ws.vec;
    buf.p[1] = search;
    CgConfig cfg{precond, max_iter, threshold, 0.0, dt, 0, 1};
    pg_pcg_stats st{};
    rc = run_cg<T>(g, cfg, buf, &st);
    if (rc) return rc;
    const i64 it = st.iterations;
    T* p_cur = buf.p[it & 1];
    const int nb = grid_blocks(g, n, kCgThreads, 8);
    cudaStream_t s = g->stream;
    if (it > 0 && st.status == PG_NOT_CONVERGED && it >= max_iter) {
        if (precond == PG_PRECOND_JACOBI)
            PG_LAUNCH(KK_CG_TAIL, s,
                      k_cg_tail<T, PM_JACOBI><<<nb, kCgThreads, 0, s>>>(residual, p_cur, auxiliary, search, g->flags,
                                                                       n, (T)dt, g->ws.state));
        else
            PG_LAUNCH(KK_CG_TAIL, s,
                      k_cg_tail<T, PM_NONE><<<nb, kCgThreads, 0, s>>>(residual, p_cur, auxiliary, search, g->flags, n,
                                                                     (T)dt, g->ws.state));
        PG_CHECK_LAUNCH();
    } else if (it > 0 && p_cur != search) {
        PG_CUDA(cudaMemcpyAsync(search, p_cur, sizeof(T) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    }
    PG_CUDA(cudaStreamSynchronize(s));
    if (stats) *stats = st;
    return st.status;
}

}  // namespace pg

extern "C" int pg_pcg_f32(const pg_grid* g, int precond, float* x, const float* b, int64_t max_iter, double threshold,
                          float* residual, float* auxiliary, float* search, double dt, pg_pcg_stats* stats) {
    return pg::pcg_abi<float>(g, precond, x, b, max_iter, threshold, residual, auxiliary, search, dt, stats);
}

extern "C" int pg_pcg_f64(const pg_grid* g, int precond, double* x, const double* b, int64_t max_iter,
                          double threshold, double* residual, double* auxiliary, double* search, double dt,
                          pg_pcg_stats* stats) {
    return pg::pcg_abi<double>(g, precond, x, b, max_iter, threshold, residual, auxiliary, search, dt, stats);
}

// ===========================================================================
// pg_pcg_noalloc_f32 -- the PCG above for callers that cannot allocate
// device memory: code whose device memory is all owned by a host
// framework's pool or arena (a cudaMalloc inside a library call would escape
// its accounting), and time-critical loops where a cudaMalloc / cudaFree
// would synchronise the device.  Its scratch -- the CG state, the per-block
// reduction partials, the second search-direction buffer and, when the
// caller passes no geometry, the wall-only face-open bits -- lives in one
// file-scope device array of fixed size instead of library allocations.
#include <mutex>

namespace pg {
namespace noalloc {

constexpr i64 kMaxCells = (i64)1 << 20;  // 1,048,576 cells (e.g. 1024^2, 101^3)
constexpr size_t kStateBytes = 256;
constexpr size_t kPartialBytes = sizeof(double) * 4 * kMaxBlocks;  // 128 KiB
constexpr size_t kSearchBytes = sizeof(float) * kMaxCells;         // 4 MiB
constexpr size_t kFlagBytes = kMaxCells;                           // 1 MiB
constexpr size_t kBytes = kStateBytes + kPartialBytes + kSearchBytes + kFlagBytes;
static_assert(sizeof(CgState) <= kStateBytes, "CgState must fit the scratch header");
static_assert((kStateBytes + kPartialBytes) % 256 == 0, "search buffer alignment");

// Held by every GPU that loads the library, until the process exits.
static __device__ __align__(256) unsigned char g_scratch[kBytes];

// Device address of g_scratch, looked up once per device with that device
// current (in host code the symbol is only a stand-in, not an address).
static std::mutex g_mu;
static unsigned char* g_addr[256];

static int scratch_address(unsigned char** out) {
    int dev = 0;
    PG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return bad_arg("pg_pcg_noalloc_f32: device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        unsigned char* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(pg_pcg_noalloc_f32 scratch)");
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return PG_OK;
}

// Face-open bits of a grid without obstacles: every interior face open.
__global__ void k_wall_flags(uint8_t* __restrict__ flags, Dims D) {
    const int d = (int)D.d, h = (int)D.h, w = (int)D.w;
    const int n = d * h * w;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const int zy = c / w, x = c - zy * w;
        const int z = zy / h, y = zy - z * h;
        uint8_t f = 0;
        if (x > 0) f |= XLO;
        if (x < w - 1) f |= XHI;
        if (y > 0) f |= YLO;
        if (y < h - 1) f |= YHI;
        if (D.nd == 3) {
            if (z > 0) f |= ZLO;
            if (z < d - 1) f |= ZHI;
        }
        flags[c] = f;
    }
}

template <int PM>
static int run(const Dims& D, const uint8_t* flags, float* x, const float* b, i64 max_iter, double threshold,
               float* residual, float* auxiliary, float* search, double dt, cudaStream_t s, CgState* st,
               double* partials, float* pbuf, pg_pcg_stats* stats) {
    int dev = 0, sms = 0;
    PG_CUDA(cudaGetDevice(&dev));
    PG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const i64 n = D.nc();
    const int nb = (int)std::max<i64>(1, std::min<i64>({(n + kCgThreads - 1) / kCgThreads, (i64)sms * 8,
                                                        (i64)kMaxBlocks}));
    const float fdt = (float)dt;
    float* p[2] = {pbuf, search};
    int64_t launches = 0;
    // The CG state and its last-block tickets must start at zero.
    PG_CUDA(cudaMemsetAsync(st, 0, sizeof(CgState), s));
    k_cg_init<float, PM><<<nb, kCgThreads, 0, s>>>(x, residual, b, flags, n, fdt, threshold, 0.0, max_iter, 1, st,
                                                   partials);
    PG_CHECK_LAUNCH();
    ++launches;
    const double us_per_iter = 4.0 + (double)n * 41.0 / 5.0e6;
    const int chunk = (int)std::min(64.0, std::max(2.0, 600.0 / us_per_iter));
    CgState hs;
    i64 done_launch = 0;
    bool done = false;
    while (!done && done_launch < max_iter) {
        const i64 todo = std::min<i64>(chunk, max_iter - done_launch);
        for (i64 k = 0; k < todo; ++k) {
            spmv_launch<float, PM>(s, sms, residual, nullptr, p[0], p[1], auxiliary, flags, D, fdt, st, partials, nb,
                                   cg_tma_enabled());
            update_launch<float, PM>(s, nb, x, residual, p[0], p[1], auxiliary, flags, n, fdt, st, partials);
        }
        PG_CHECK_LAUNCH();
        launches += 2 * todo;
        done_launch += todo;
        PG_CUDA(cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
        PG_CUDA(cudaStreamSynchronize(s));
        done = hs.done != 0;
    }
    PG_CUDA(cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    // Work vectors end as the reference leaves them (pcg.rs:51-77).
    const i64 it = hs.iter;
    float* p_cur = p[it & 1];
    if (it > 0 && hs.status == PG_NOT_CONVERGED && it >= max_iter) {
        k_cg_tail<float, PM><<<nb, kCgThreads, 0, s>>>(residual, p_cur, auxiliary, search, flags, n, fdt, st);
        PG_CHECK_LAUNCH();
        ++launches;
    } else if (it > 0 && p_cur != search) {
        PG_CUDA(cudaMemcpyAsync(search, p_cur, sizeof(float) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    }
    PG_CUDA(cudaStreamSynchronize(s));
    prof_add_launches(launches);
    if (stats) {
        stats->iterations = hs.iter;
        stats->refinements = 0;
        stats->residual_max = hs.rmax;
        stats->b_max = hs.bmax;
        stats->threshold = hs.threshold;
        stats->true_residual_max = -1.0;
        stats->status = hs.status;
    }
    return hs.status;
}

}  // namespace noalloc
}  // namespace pg

extern "C" int pg_pcg_noalloc_f32(int32_t nd, int64_t d, int64_t h, int64_t w, const uint8_t* cell_flags,
                                  int precond, float* x, const float* b, int64_t max_iterations, double threshold,
                                  float* residual, float* auxiliary, float* search, double dt, void* cuda_stream,
                                  pg_pcg_stats* stats) {
    using namespace pg;
    if (nd != 2 && nd != 3) return bad_arg("pg_pcg_noalloc_f32: nd must be 2 or 3");
    if (nd == 2 && d != 1) return bad_arg("pg_pcg_noalloc_f32: 2D grids take d = 1");
    if (d < 1 || h < 1 || w < 1) return bad_arg("pg_pcg_noalloc_f32: every dimension must be >= 1");
    if (d > noalloc::kMaxCells / h / w || d * h * w > noalloc::kMaxCells)
        return bad_arg("pg_pcg_noalloc_f32: grid larger than 1048576 cells, the size of its fixed scratch; "
                       "use pg_pcg_f32");
    if (!x || !b || !residual || !auxiliary || !search) return bad_arg("pg_pcg_noalloc_f32: NULL argument");
    if (precond != PG_PRECOND_NONE && precond != PG_PRECOND_JACOBI)
        return bad_arg("pg_pcg_noalloc_f32: precond must be PG_PRECOND_NONE or PG_PRECOND_JACOBI");
    if (max_iterations < 0) return bad_arg("pg_pcg_noalloc_f32: max_iterations < 0");
    unsigned char* base = nullptr;
    int rc = noalloc::scratch_address(&base);
    if (rc) return rc;
    CgState* st = (CgState*)base;
    double* partials = (double*)(base + noalloc::kStateBytes);
    float* pbuf = (float*)(base + noalloc::kStateBytes + noalloc::kPartialBytes);
    uint8_t* wflags = base + noalloc::kStateBytes + noalloc::kPartialBytes + noalloc::kSearchBytes;
    const Dims D{nd, d, h, w};
    cudaStream_t s = (cudaStream_t)cuda_stream;
    const uint8_t* flags = cell_flags;
    if (!flags) {
        noalloc::k_wall_flags<<<(int)std::min<i64>((D.nc() + 255) / 256, 1024), 256, 0, s>>>(wflags, D);
        PG_CHECK_LAUNCH();
        prof_add_launches(1);
        flags = wflags;
    }
    if (precond == PG_PRECOND_JACOBI)
        return noalloc::run<PM_JACOBI>(D, flags, x, b, max_iterations, threshold, residual, auxiliary, search, dt, s,
                                       st, partials, pbuf, stats);
    return noalloc::run<PM_NONE>(D, flags, x, b, max_iterations, threshold, residual, auxiliary, search, dt, s, st,
                                 partials, pbuf, stats);
}
