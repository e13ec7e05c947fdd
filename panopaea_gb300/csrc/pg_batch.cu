// pg_batch.cu -- many independent 2D grids of uneven sizes advanced together
// (an extension; the reference steps one grid, examples/dec_fluid.rs:46-141).
//
// Fields of all grids are packed back to back (each grid in the reference
// layout) and every stage -- source, advection, walls, buoyancy, -div, each
// CG kernel, projection -- is ONE launch over a work list of 2D tiles drawn
// from all grids.  Per-grid CG scalars live in a device array; each
// reduction kernel writes one partial per tile and a finalisation kernel
// with one block per grid reduces that grid's tiles in a fixed order
// (deterministic), applies the per-grid stop rule and counts the grids still
// running.  Tiles of grids that have converged return at once (retirement).
// The CG loop runs as a CUDA graph WHILE node until no grid is running.
// The tile shape and whether the search-direction update is fused into the
// SpMV are picked by pg_batch_autotune (timed on the batch itself, cached).
// Per-sample arithmetic is shared with the single-grid kernels
// (pg_ops2d.cuh), so batched and single-grid results agree bit for bit
// outside the CG reductions.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "pg_batch.cuh"

namespace pg {

// ---------------------------------------------------------------------------
// per-stage kernels

__global__ void k_b_source_field(float* __restrict__ rho, const float* __restrict__ src, i64 n) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        rho[i] = fmaxf(rho[i], src[i]);
}

__global__ void k_b_advect(float* __restrict__ dst, const float* __restrict__ q, const float* __restrict__ vel,
                           const GInfo* __restrict__ gi, const Tile* __restrict__ tiles, int ntiles, int tx, int ty,
                           float ndt) {
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const GInfo G = gi[t.grid];
        const int x = t.x0 + (int)threadIdx.x % tx, y = t.y0 + (int)threadIdx.x / tx;
        if (x < G.w && y < G.h) {
            const float* vy = vel + G.foff;
            const float* vx = vy + (i64)(G.h + 1) * G.w;
            dst[G.coff + (i64)y * G.w + x] =
                advect2d_at<float, int>(q + G.coff, vy, vx, G.h, G.w, ndt, G.hix, G.hiy, y, x);
        }
    }
}

// Faces with index (y, x) in the (h+1) x (w+1) box: the x face when y < h,
// the y face when x < w.
__global__ void k_b_advect_mac(float* __restrict__ dst, const float* __restrict__ vel, const GInfo* __restrict__ gi,
                               const Tile* __restrict__ tiles, int ntiles, int tx, int ty, float ndt) {
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const GInfo G = gi[t.grid];
        const int x = t.x0 + (int)threadIdx.x % tx, y = t.y0 + (int)threadIdx.x / tx;
        const float* vy = vel + G.foff;
        const i64 n0 = (i64)(G.h + 1) * G.w;
        const float* vx = vy + n0;
        if (y < G.h && x <= G.w)
            dst[G.foff + n0 + (i64)y * (G.w + 1) + x] = advect_mac2d_x_at<float, int>(vx, vy, vx, G.h, G.w, ndt, y, x);
        if (y <= G.h && x < G.w)
            dst[G.foff + (i64)y * G.w + x] = advect_mac2d_y_at<float, int>(vy, vy, vx, G.h, G.w, ndt, y, x);
    }
}

// Walls (dec_fluid.rs:128-141) and buoyancy (extension) on the face box.
__global__ void k_b_walls_buoyancy(float* __restrict__ vel, const float* __restrict__ rho, const GInfo* __restrict__ gi,
                                   const Tile* __restrict__ tiles, int ntiles, int tx, int ty, int walls, float coef) {
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const GInfo G = gi[t.grid];
        const int x = t.x0 + (int)threadIdx.x % tx, y = t.y0 + (int)threadIdx.x / tx;
        const i64 n0 = (i64)(G.h + 1) * G.w;
        if (walls && y < G.h && (x == 0 || x == G.w)) vel[G.foff + n0 + (i64)y * (G.w + 1) + x] = 0.f;
        if (y <= G.h && x < G.w) {
            const i64 f = G.foff + (i64)y * G.w + x;
            if (walls && (y == 0 || y == G.h)) {
                vel[f] = 0.f;
            } else if (coef != 0.f && y > 0 && y < G.h) {
                const float* rr = rho + G.coff;
                vel[f] = add_rn(vel[f], mul_rn(coef, mul_rn(0.5f, add_rn(rr[(i64)(y - 1) * G.w + x], rr[(i64)y * G.w + x]))));
            }
        }
    }
}

// -div (dec_fluid.rs:68-83), same operation order as the single-grid k_rhs.
__global__ void k_b_rhs(float* __restrict__ b, const float* __restrict__ vel, const uint8_t* __restrict__ flags,
                        const uint8_t* __restrict__ fsolid, const GInfo* __restrict__ gi, const Tile* __restrict__ tiles,
                        int ntiles, int tx, int ty) {
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const GInfo G = gi[t.grid];
        const int x = t.x0 + (int)threadIdx.x % tx, y = t.y0 + (int)threadIdx.x / tx;
        if (x >= G.w || y >= G.h) continue;
        const i64 c = G.coff + (i64)y * G.w + x;
        const uint8_t f = flags[c];
        const i64 n0 = (i64)(G.h + 1) * G.w;
        const i64 iyl = G.foff + (i64)y * G.w + x, iyh = iyl + G.w;
        const i64 ixl = G.foff + n0 + (i64)y * (G.w + 1) + x, ixh = ixl + 1;
        auto masked = [&](i64 idx, bool interior, uint8_t bit) -> bool {
            if (interior) return !(f & bit);
            return fsolid != nullptr && fsolid[idx] != 0;
        };
        const float top = masked(iyl, y > 0, YLO) ? 0.f : -vel[iyl];
        const float bottom = masked(iyh, y < G.h - 1, YHI) ? 0.f : -vel[iyh];
        const float ux_lo = masked(ixl, x > 0, XLO) ? 0.f : vel[ixl];
        const float ux_hi = masked(ixh, x < G.w - 1, XHI) ? 0.f : vel[ixh];
        b[c] = -add_rn(sub_rn(add_rn(-bottom, top), ux_lo), ux_hi);
    }
}

// Projection + walls (dec_fluid.rs:123-141) on the face box.
__global__ void k_b_project(float* __restrict__ vel, const float* __restrict__ p, const uint8_t* __restrict__ flags,
                            const GInfo* __restrict__ gi, const Tile* __restrict__ tiles, int ntiles, int tx, int ty,
                            float dt, int zero_solid) {
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const GInfo G = gi[t.grid];
        const int x = t.x0 + (int)threadIdx.x % tx, y = t.y0 + (int)threadIdx.x / tx;
        const i64 n0 = (i64)(G.h + 1) * G.w;
        const float* pp = p + G.coff;
        const uint8_t* fl = flags + G.coff;
        if (y < G.h && x <= G.w) {  // x face
            const i64 i = G.foff + n0 + (i64)y * (G.w + 1) + x;
            if (x == 0 || x == G.w) {
                vel[i] = 0.f;
            } else {
                const i64 c = (i64)y * G.w + x;
                const float e = sub_rn(pp[c - 1], pp[c]);
                vel[i] = (zero_solid && !(fl[c] & XLO)) ? 0.f : add_rn(vel[i], mul_rn(dt, e));
            }
        }
        if (y <= G.h && x < G.w) {  // y face
            const i64 i = G.foff + (i64)y * G.w + x;
            if (y == 0 || y == G.h) {
                vel[i] = 0.f;
            } else {
                const i64 c = (i64)y * G.w + x;
                const float e = -sub_rn(pp[c], pp[c - G.w]);
                vel[i] = (zero_solid && !(fl[c] & YLO)) ? 0.f : add_rn(vel[i], mul_rn(dt, e));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// CG over all grids (pcg.rs:14-82 per grid)

// PM_ZBUF: r is the MG z buffer, used as z - zm on the fluid cells.
template <int PM> __device__ __forceinline__ float bz(const float* __restrict__ r, const uint8_t* __restrict__ flags,
                                                      i64 k, float dt, float zm = 0.f) {
    if (PM == PM_JACOBI) {
        const int n = __popc((unsigned)flags[k]);
        return n ? r[k] * __frcp_rn((float)n * dt) : 0.f;
    }
    if (PM == PM_ZBUF) return flags[k] ? r[k] - zm : r[k];
    return r[k];
}

template <int PM>
__global__ void k_b_cg_init(float* __restrict__ x, float* __restrict__ r, const float* __restrict__ b,
                            const uint8_t* __restrict__ flags, const GInfo* __restrict__ gi, const Tile* __restrict__ tiles,
                            int ntiles, int tx, int ty, float dt, double* partials) {
    __shared__ F2 sm[64];
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const GInfo G = gi[t.grid];
        const int xx = t.x0 + (int)threadIdx.x % tx, yy = t.y0 + (int)threadIdx.x / tx;
        float bm = 0.f;
        Acc<float> sig;
        if (xx < G.w && yy < G.h) {
            const i64 c = G.coff + (i64)yy * G.w + xx;
            const float bv = b[c];
            x[c] = 0.f;
            r[c] = bv;
            bm = isfinite(bv) ? fabsf(bv) : __int_as_float(0x7f800000);
            if (PM == PM_ZBUF) sig.add(bv);  // sum(b) for the lazy projection
            else sig.add(bz<PM>(b, flags, c, dt) * bv);
        }
        double m, s;
        tmaxsum(bm, f2_of(sig), sm, &m, &s);
        if (threadIdx.x == 0) {
            partials[2 * (i64)ti] = m;
            partials[2 * (i64)ti + 1] = s;
        }
    }
}

// One block per grid: fold the grid's tile partials (fixed order).
// stage 0: after init; 1: after the SpMV (p.Ap); 2: after the update.
// zbuf (stage 2): z comes from an outer preconditioner after the update,
// so beta and sigma are set later (bmg_rz_finalize).
template <int STAGE>
__global__ void k_b_finalize(const GInfo* __restrict__ gi, BState* __restrict__ st, const double* __restrict__ partials,
                             int n, double rel_tol, double thr_abs, int max_iter, int* active, int zbuf = 0,
                             const double* __restrict__ nfluid = nullptr) {
    __shared__ double sm[32];
    const int g = blockIdx.x;
    if (g >= n) return;
    BState& S = st[g];
    if (STAGE != 0 && S.done) return;
    const int t0 = gi[g].t0, t1 = gi[g].t1;
    double a = 0.0, bb = 0.0;
    for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
        const double pa = partials[2 * (i64)t], pb = partials[2 * (i64)t + 1];
        if (STAGE == 1) a += pa;
        else a = fmax(a, pa);
        bb += pb;
    }
    a = STAGE == 1 ? bsum(a, sm) : bmaxr(a, sm);
    bb = bsum(bb, sm);
    if (threadIdx.x != 0) return;
    if (STAGE == 0) {
        S.bmax = a;
        S.rmax = a;
        S.sigma = bb;
        S.thr = (double)(float)(rel_tol > 0.0 ? rel_tol * a : thr_abs);
        S.beta = 0.0;
        S.fbeta = 0.f;
        S.fzm = 0.f;
        S.iter = 0;
        S.max_iter = max_iter;
        S.first = 1;
        S.done = 0;
        S.status = PG_NOT_CONVERGED;
        S.rsum = bb;
        S.zmean = 0.0;
        S.nfluid = nfluid ? nfluid[g] : 0.0;
        if (!isfinite(a) || !isfinite(bb)) {
            S.status = PG_NAN_DETECTED;
            S.done = 1;
        } else if ((float)a < (float)S.thr || a == 0.0) {
            S.status = PG_OK;
            S.done = 1;
        } else if (max_iter <= 0) {
            S.done = 1;
        }
        if (!S.done) atomicAdd(active, 1);
    } else if (STAGE == 1) {
        S.pap = a;
        if (!isfinite(a)) {
            S.status = PG_NAN_DETECTED;
            S.done = 1;
        } else if (!(a > 0.0)) {
            S.status = S.sigma == 0.0 ? PG_NOT_CONVERGED : PG_BREAKDOWN;
            S.done = 1;
        } else {
            S.alpha = S.sigma / a;
            S.falpha = (float)S.alpha;
        }
    } else {
        S.iter += 1;
        S.rmax = a;
        if (!isfinite(a) || !isfinite(bb)) {
            S.status = PG_NAN_DETECTED;
            S.done = 1;
        } else if ((float)a < (float)S.thr) {
            S.status = PG_OK;
            S.done = 1;
        } else {
            if (!zbuf) {
                S.beta = bb / S.sigma;
                S.fbeta = (float)S.beta;
                S.sigma = bb;
            } else {
                S.rsum = bb;
            }
            S.first = 0;
            if (S.iter >= S.max_iter) S.done = 1;
        }
        if (!S.done) atomicAdd(active, 1);
    }
}

// p = z + beta p (ping-pong by the grid's iteration count), A p, p.Ap.
// FUSED = 1 recomputes the neighbours' new p; FUSED = 0 expects p already
// updated by k_b_pupdate and reads it.
template <int PM, int FUSED>
__global__ void k_b_spmv(const float* __restrict__ r, float* p0, float* p1, float* __restrict__ ap,
                         const uint8_t* __restrict__ flags, const GInfo* __restrict__ gi, const Tile* __restrict__ tiles,
                         int ntiles, int tx, int ty, float dt, const BState* __restrict__ st, double* partials) {
    __shared__ F2 sm[32];
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const BState& S = st[t.grid];
        if (S.done) continue;  // uniform per block
        const GInfo G = gi[t.grid];
        const int it = S.iter, first = S.first;
        const float beta = first ? 0.f : S.fbeta;
        const float zm = PM == PM_ZBUF ? S.fzm : 0.f;
        const float* p_old = (it & 1) ? p1 : p0;
        float* p_new = (it & 1) ? p0 : p1;
        // p_new of cell k; `fluid`: k has an open face (a neighbour behind an
        // open face always has), the cells the projected z applies to
        auto pn = [&](i64 k, bool fluid) -> float {
            if (!FUSED) return p_new[k];
            const float z = PM == PM_ZBUF ? (fluid ? r[k] - zm : r[k]) : bz<PM>(r, flags, k, dt);
            return first ? z : z + beta * p_old[k];
        };
        const int xx = t.x0 + (int)threadIdx.x % tx, yy = t.y0 + (int)threadIdx.x / tx;
        Acc<float> acc;
        if (xx < G.w && yy < G.h) {
            const i64 c = G.coff + (i64)yy * G.w + xx;
            const uint8_t f = flags[c];
            const float pc = pn(c, f != 0);
            if (FUSED) p_new[c] = pc;
            const float gy_lo = (f & YLO) ? -sub_rn(pc, pn(c - G.w, true)) : 0.f;
            const float gy_hi = (f & YHI) ? -sub_rn(pn(c + G.w, true), pc) : 0.f;
            const float gx_lo = (f & XLO) ? sub_rn(pn(c - 1, true), pc) : 0.f;
            const float gx_hi = (f & XHI) ? sub_rn(pc, pn(c + 1, true)) : 0.f;
            const float a = mul_rn(add_rn(sub_rn(sub_rn(gy_hi, gy_lo), gx_lo), gx_hi), dt);
            ap[c] = a;
            acc.add(pc * a);
        }
        const double s = tsum(f2_of(acc), sm);
        if (threadIdx.x == 0) {
            partials[2 * (i64)ti] = s;
            partials[2 * (i64)ti + 1] = 0.0;
        }
    }
}

// Unfused search-direction update (autotuner alternative).
template <int PM>
__global__ void k_b_pupdate(const float* __restrict__ r, float* p0, float* p1, const uint8_t* __restrict__ flags,
                            const GInfo* __restrict__ gi, const Tile* __restrict__ tiles, int ntiles, int tx, int ty,
                            float dt, const BState* __restrict__ st) {
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const BState& S = st[t.grid];
        if (S.done) continue;
        const GInfo G = gi[t.grid];
        const int xx = t.x0 + (int)threadIdx.x % tx, yy = t.y0 + (int)threadIdx.x / tx;
        if (xx < G.w && yy < G.h) {
            const i64 c = G.coff + (i64)yy * G.w + xx;
            const float* p_old = (S.iter & 1) ? p1 : p0;
            float* p_new = (S.iter & 1) ? p0 : p1;
            const float z = bz<PM>(r, flags, c, dt, PM == PM_ZBUF ? S.fzm : 0.f);
            p_new[c] = S.first ? z : z + S.fbeta * p_old[c];
        }
    }
}

template <int PM>
__global__ void k_b_update(float* __restrict__ x, float* __restrict__ r, const float* p0, const float* p1,
                           const float* __restrict__ ap, const uint8_t* __restrict__ flags, const GInfo* __restrict__ gi,
                           const Tile* __restrict__ tiles, int ntiles, int tx, int ty, float dt,
                           const BState* __restrict__ st, double* partials) {
    __shared__ F2 sm[64];
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const BState& S = st[t.grid];
        if (S.done) continue;
        const GInfo G = gi[t.grid];
        const float* p = ((S.iter + 1) & 1) ? p1 : p0;
        const float alpha = S.falpha;
        const int xx = t.x0 + (int)threadIdx.x % tx, yy = t.y0 + (int)threadIdx.x / tx;
        float rm = 0.f;
        Acc<float> rz;
        if (xx < G.w && yy < G.h) {
            const i64 c = G.coff + (i64)yy * G.w + xx;
            x[c] = x[c] + alpha * p[c];
            const float rv = r[c] + (-alpha) * ap[c];
            r[c] = rv;
            rm = isfinite(rv) ? fabsf(rv) : __int_as_float(0x7f800000);
            float z = rv;
            if (PM == PM_JACOBI) {
                const int nn = __popc((unsigned)flags[c]);
                z = nn ? rv * __frcp_rn((float)nn * dt) : 0.f;
            }
            if (PM == PM_ZBUF) rz.add(rv);  // sum(r) for the lazy projection
            else rz.add(z * rv);
        }
        double m, s;
        tmaxsum(rm, f2_of(rz), sm, &m, &s);
        if (threadIdx.x == 0) {
            partials[2 * (i64)ti] = m;
            partials[2 * (i64)ti + 1] = s;
        }
    }
}

__global__ void k_b_cond(int* active, cudaGraphConditionalHandle h) {
    const int a = *active;
    *active = 0;
    cudaGraphSetConditional(h, a > 0 ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// host side

static int build_tiles(pg_batch* B, int tx, int ty) {
    std::vector<Tile> t, te;
    B->host_info.resize(B->n);
    for (int g = 0; g < B->n; ++g) {
        GInfo& G = B->host_info[g];
        G.h = B->h[g];
        G.w = B->w[g];
        G.coff = B->coff[g];
        G.foff = B->foff[g];
        G.hix = (float)((double)G.w - 1.00001);
        G.hiy = (float)((double)G.h - 1.00001);
        G.t0 = (int)t.size();
        for (int y0 = 0; y0 < G.h; y0 += ty)
            for (int x0 = 0; x0 < G.w; x0 += tx) t.push_back(Tile{g, y0, x0});
        G.t1 = (int)t.size();
        for (int y0 = 0; y0 <= G.h; y0 += ty)
            for (int x0 = 0; x0 <= G.w; x0 += tx) te.push_back(Tile{g, y0, x0});
    }
    if (B->tiles) cudaFree(B->tiles);
    if (B->tiles_ext) cudaFree(B->tiles_ext);
    if (B->partials) cudaFree(B->partials);
    B->tiles = B->tiles_ext = nullptr;
    B->partials = nullptr;
    PG_CUDA(cudaMalloc(&B->tiles, sizeof(Tile) * t.size()));
    PG_CUDA(cudaMalloc(&B->tiles_ext, sizeof(Tile) * te.size()));
    PG_CUDA(cudaMalloc(&B->partials, sizeof(double) * 2 * t.size()));
    PG_CUDA(cudaMemcpy(B->tiles, t.data(), sizeof(Tile) * t.size(), cudaMemcpyHostToDevice));
    PG_CUDA(cudaMemcpy(B->tiles_ext, te.data(), sizeof(Tile) * te.size(), cudaMemcpyHostToDevice));
    PG_CUDA(cudaMemcpy(B->ginfo, B->host_info.data(), sizeof(GInfo) * B->n, cudaMemcpyHostToDevice));
    B->ntiles = (int)t.size();
    B->ntiles_ext = (int)te.size();
    B->tx = tx;
    B->ty = ty;
    return PG_OK;
}

static int bblocks(const pg_batch* B, int ntiles) {
    return std::max(1, std::min(ntiles, B->num_sms * 8));
}

// One CG iteration over all grids.  PM_ZBUF: z = V(r) by the batched
// multigrid; the SpMV and update run in their identity-preconditioner form
// with z in place of r.
template <int PM> static void b_iter(pg_batch* B, cudaStream_t s, float dt, float* x, int nsmooth = 2) {
    if (PM == PM_ZBUF) {
        const int nt = B->tx * B->ty, nb = bblocks(B, B->ntiles);
        if (B->fused) {
            PG_LAUNCH(KK_CG_SPMV, s,
                      k_b_spmv<PM_ZBUF, 1><<<nb, nt, 0, s>>>(B->z, B->p0, B->p1, B->ap, B->flags, B->ginfo, B->tiles,
                                                             B->ntiles, B->tx, B->ty, dt, B->state, B->partials));
        } else {
            PG_LAUNCH(KK_CG_SPMV, s,
                      k_b_pupdate<PM_ZBUF><<<nb, nt, 0, s>>>(B->z, B->p0, B->p1, B->flags, B->ginfo, B->tiles, B->ntiles,
                                                             B->tx, B->ty, dt, B->state));
            PG_LAUNCH(KK_CG_SPMV, s,
                      k_b_spmv<PM_ZBUF, 0><<<nb, nt, 0, s>>>(B->z, B->p0, B->p1, B->ap, B->flags, B->ginfo, B->tiles,
                                                             B->ntiles, B->tx, B->ty, dt, B->state, B->partials));
        }
        PG_LAUNCH(KK_STEP_MISC, s,
                  k_b_finalize<1><<<B->n, 128, 0, s>>>(B->ginfo, B->state, B->partials, B->n, 0.0, 0.0, 0, B->active));
        PG_LAUNCH(KK_CG_UPDATE, s,
                  k_b_update<PM_ZBUF><<<nb, nt, 0, s>>>(x, B->r, B->p0, B->p1, B->ap, B->flags, B->ginfo, B->tiles,
                                                        B->ntiles, B->tx, B->ty, dt, B->state, B->partials));
        PG_LAUNCH(KK_STEP_MISC, s,
                  k_b_finalize<2><<<B->n, 128, 0, s>>>(B->ginfo, B->state, B->partials, B->n, 0.0, 0.0, 0, B->active, 1));
        bmg_vcycle(B, s, nsmooth);
        bmg_rz_finalize(B, s, 0);
        return;
    }
    const int nt = B->tx * B->ty, nb = bblocks(B, B->ntiles);
    if (B->fused) {
        PG_LAUNCH(KK_CG_SPMV, s,
                  k_b_spmv<PM, 1><<<nb, nt, 0, s>>>(B->r, B->p0, B->p1, B->ap, B->flags, B->ginfo, B->tiles, B->ntiles,
                                                    B->tx, B->ty, dt, B->state, B->partials));
    } else {
        PG_LAUNCH(KK_CG_SPMV, s,
                  k_b_pupdate<PM><<<nb, nt, 0, s>>>(B->r, B->p0, B->p1, B->flags, B->ginfo, B->tiles, B->ntiles, B->tx,
                                                    B->ty, dt, B->state));
        PG_LAUNCH(KK_CG_SPMV, s,
                  k_b_spmv<PM, 0><<<nb, nt, 0, s>>>(B->r, B->p0, B->p1, B->ap, B->flags, B->ginfo, B->tiles, B->ntiles,
                                                    B->tx, B->ty, dt, B->state, B->partials));
    }
    PG_LAUNCH(KK_STEP_MISC, s,
              k_b_finalize<1><<<B->n, 128, 0, s>>>(B->ginfo, B->state, B->partials, B->n, 0.0, 0.0, 0, B->active));
    PG_LAUNCH(KK_CG_UPDATE, s,
              k_b_update<PM><<<nb, nt, 0, s>>>(x, B->r, B->p0, B->p1, B->ap, B->flags, B->ginfo, B->tiles, B->ntiles,
                                               B->tx, B->ty, dt, B->state, B->partials));
    PG_LAUNCH(KK_STEP_MISC, s,
              k_b_finalize<2><<<B->n, 128, 0, s>>>(B->ginfo, B->state, B->partials, B->n, 0.0, 0.0, 0, B->active));
}

template <int PM> static int b_graph(pg_batch* B, float dt, float* x, int nsmooth) {
    const uint64_t mgkey = PM == PM_ZBUF ? (bmg_id(B) << 8) | (uint64_t)(nsmooth & 0xff) : 0;
    if (B->exec && B->graph_tx == B->tx && B->graph_ty == B->ty && B->graph_fused == B->fused &&
        B->graph_pm == PM && B->graph_dt == dt && B->graph_x == x && B->graph_mg == mgkey)
        return PG_OK;
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    B->exec = nullptr;
    B->graph = nullptr;
    PG_CUDA(cudaGraphCreate(&B->graph, 0));
    cudaGraphConditionalHandle h;
    PG_CUDA(cudaGraphConditionalHandleCreate(&h, B->graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    PG_CUDA(cudaGraphAddNode(&node, B->graph, nullptr, nullptr, 0, &cp));
    cudaStream_t cs;
    PG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    prof_capture_begin();
    cudaError_t err = cudaStreamBeginCaptureToGraph(cs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                    cudaStreamCaptureModeThreadLocal);
    if (err == cudaSuccess) {
        b_iter<PM>(B, cs, dt, x, nsmooth);
        k_b_cond<<<1, 1, 0, cs>>>(B->active, h);
        cudaGraph_t g2 = nullptr;
        err = cudaStreamEndCapture(cs, &g2);
    }
    prof_capture_end();
    cudaStreamDestroy(cs);
    if (err != cudaSuccess) return cuda_fail(err, "batch CG graph capture");
    PG_CUDA(cudaGraphInstantiate(&B->exec, B->graph, 0));
    B->graph_tx = B->tx;
    B->graph_ty = B->ty;
    B->graph_fused = B->fused;
    B->graph_pm = PM;
    B->graph_dt = dt;
    B->graph_x = x;
    B->graph_mg = mgkey;
    return PG_OK;
}

// Solve every grid's A x = b (b in B->b); x packed cells.
template <int PM>
static int b_solve(pg_batch* B, const pg_solver_params* prm, float dt, float* x, int max_host_iters) {
    cudaStream_t s = B->stream;
    const int nt = B->tx * B->ty, nb = bblocks(B, B->ntiles);
    const int nsmooth = prm->mg_smooth > 0 ? prm->mg_smooth : 2;
    // init: r = b (PM_ZBUF: z comes from the V-cycle; sum(b) for the lazy projection)
    PG_CUDA(cudaMemsetAsync(B->active, 0, sizeof(int), s));
    PG_LAUNCH(KK_CG_INIT, s,
              k_b_cg_init<PM><<<nb, nt, 0, s>>>(x, B->r, B->b, B->flags, B->ginfo, B->tiles, B->ntiles, B->tx, B->ty,
                                                dt, B->partials));
    PG_LAUNCH(KK_STEP_MISC, s,
              k_b_finalize<0><<<B->n, 128, 0, s>>>(B->ginfo, B->state, B->partials, B->n,
                                                   prm->rel_stop ? prm->rel_tol : 0.0, prm->threshold,
                                                   (int)std::min<i64>(prm->max_iter, 1 << 30), B->active, 0,
                                                   PM == PM_ZBUF ? B->nfluid : nullptr));
    if (PM == PM_ZBUF) {
        bmg_vcycle(B, s, nsmooth);
        bmg_rz_finalize(B, s, 1);
    }
    PG_CHECK_LAUNCH();
    if (max_host_iters < 0 && graphs_enabled()) {
        int rc = b_graph<PM>(B, dt, x, nsmooth);
        if (rc) return rc;
        PG_CUDA(cudaGraphLaunch(B->exec, s));
    } else {
        // host-driven loop (profiling, autotuning): poll the active count
        const int lim = max_host_iters < 0 ? (int)std::min<i64>(prm->max_iter, 1 << 30) : max_host_iters;
        int act = 1;
        for (int it = 0; it < lim && act > 0; it += 8) {
            PG_CUDA(cudaMemsetAsync(B->active, 0, sizeof(int), s));
            for (int k = 0; k < 8 && it + k < lim; ++k) b_iter<PM>(B, s, dt, x, nsmooth);
            PG_CUDA(cudaMemcpyAsync(&act, B->active, sizeof(int), cudaMemcpyDeviceToHost, s));
            PG_CUDA(cudaStreamSynchronize(s));
        }
    }
    PG_CHECK_LAUNCH();
    return PG_OK;
}

static int b_alloc(pg_batch* B) {
    const size_t nc = (size_t)B->ncells, nf = (size_t)B->nfaces;
    PG_CUDA(cudaMalloc(&B->ginfo, sizeof(GInfo) * B->n));
    PG_CUDA(cudaMalloc(&B->flags, nc));
    PG_CUDA(cudaMalloc(&B->state, sizeof(BState) * B->n));
    PG_CUDA(cudaMalloc(&B->active, sizeof(int)));
    float** cells[] = {&B->r, &B->ap, &B->p0, &B->p1, &B->b, &B->tmp};
    for (float** p : cells) PG_CUDA(cudaMalloc(p, 4 * nc));
    PG_CUDA(cudaMalloc(&B->vtmp, 4 * nf));
    return PG_OK;
}

static void b_flags(const pg_batch* B, const uint8_t* cs, std::vector<uint8_t>& flags, std::vector<uint8_t>& fsolid) {
    flags.assign((size_t)B->ncells, 0);
    fsolid.assign(cs ? (size_t)B->nfaces : 0, 0);
    for (int g = 0; g < B->n; ++g) {
        const int h = B->h[g], w = B->w[g];
        const uint8_t* c = cs ? cs + B->coff[g] : nullptr;
        auto solid = [&](int y, int x) { return c && c[(size_t)y * w + x]; };
        uint8_t* f = flags.data() + B->coff[g];
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                uint8_t v = 0;
                const bool me = solid(y, x);
                if (!me) {
                    if (x > 0 && !solid(y, x - 1)) v |= XLO;
                    if (x < w - 1 && !solid(y, x + 1)) v |= XHI;
                    if (y > 0 && !solid(y - 1, x)) v |= YLO;
                    if (y < h - 1 && !solid(y + 1, x)) v |= YHI;
                }
                f[(size_t)y * w + x] = v;
            }
        if (cs) {
            uint8_t* fy = fsolid.data() + B->foff[g];
            uint8_t* fx = fy + (size_t)(h + 1) * w;
            for (int y = 0; y <= h; ++y)
                for (int x = 0; x < w; ++x) fy[(size_t)y * w + x] = (y > 0 && solid(y - 1, x)) || (y < h && solid(y, x));
            for (int y = 0; y < h; ++y)
                for (int x = 0; x <= w; ++x)
                    fx[(size_t)y * (w + 1) + x] = (x > 0 && solid(y, x - 1)) || (x < w && solid(y, x));
        }
    }
}

static std::string tune_key(const pg_batch* B) {
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, B->device);
    unsigned long long hsh = 1469598103934665603ull;
    for (int g = 0; g < B->n; ++g) {
        hsh = (hsh ^ (unsigned long long)B->h[g]) * 1099511628211ull;
        hsh = (hsh ^ (unsigned long long)B->w[g]) * 1099511628211ull;
    }
    char buf[sizeof prop.name + 64];
    snprintf(buf, sizeof buf, "%s|sm%d%d|n%d|%016llx", prop.name, prop.major, prop.minor, B->n, hsh);
    std::string k(buf);
    for (auto& ch : k)
        if (ch == ' ') ch = '_';
    return k;
}

}  // namespace pg

using namespace pg;

extern "C" {

int pg_batch_create_2d(int32_t count, const int64_t* hs, const int64_t* ws, pg_batch** out) {
    if (!out || !hs || !ws || count < 1) return bad_arg("pg_batch_create_2d: bad arguments");
    *out = nullptr;
    for (int g = 0; g < count; ++g)
        if (hs[g] < 2 || ws[g] < 2 || hs[g] > 65536 || ws[g] > 65536)
            return bad_arg("pg_batch_create_2d: every side must be in [2, 65536]");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        set_error("pg_batch_create_2d: no CUDA device");
        return PG_NO_DEVICE;
    }
    pg_batch* B = new pg_batch();
    B->n = count;
    B->coff.assign(count + 1, 0);
    B->foff.assign(count + 1, 0);
    for (int g = 0; g < count; ++g) {
        B->h.push_back((int)hs[g]);
        B->w.push_back((int)ws[g]);
        B->coff[g + 1] = B->coff[g] + hs[g] * ws[g];
        B->foff[g + 1] = B->foff[g] + (hs[g] + 1) * ws[g] + hs[g] * (ws[g] + 1);
    }
    B->ncells = B->coff[count];
    B->nfaces = B->foff[count];
    int rc = PG_OK;
    if (cudaGetDevice(&B->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&B->num_sms, cudaDevAttrMultiProcessorCount, B->device) != cudaSuccess)
        rc = PG_CUDA_ERROR;
    if (!rc) rc = b_alloc(B);
    if (!rc) rc = build_tiles(B, 32, 8);
    if (!rc) rc = pg_batch_set_solid_cells(B, nullptr);
    if (rc) {
        pg_batch_destroy(B);
        return rc;
    }
    *out = B;
    return PG_OK;
}

int pg_batch_destroy(pg_batch* B) {
    if (!B) return PG_OK;
    cudaDeviceSynchronize();
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    bmg_release(B);
    void* ptrs[] = {B->ginfo, B->flags, B->face_solid, B->state, B->active, B->partials, B->r, B->ap, B->p0,
                    B->p1, B->b, B->tmp, B->vtmp, B->tiles, B->tiles_ext, B->z, B->nfluid};
    for (void* p : ptrs) cudaFree(p);
    delete B;
    return PG_OK;
}

int pg_batch_set_stream(pg_batch* B, void* s) {
    if (!B) return bad_arg("pg_batch_set_stream: NULL batch");
    B->stream = (cudaStream_t)s;
    return PG_OK;
}

int pg_batch_layout(const pg_batch* B, int64_t* cell_offsets, int64_t* face_offsets) {
    if (!B || !cell_offsets || !face_offsets) return bad_arg("pg_batch_layout: NULL argument");
    for (int g = 0; g <= B->n; ++g) {
        cell_offsets[g] = B->coff[g];
        face_offsets[g] = B->foff[g];
    }
    return PG_OK;
}

int pg_batch_set_solid_cells(pg_batch* B, const uint8_t* cs) {
    if (!B) return bad_arg("pg_batch_set_solid_cells: NULL batch");
    std::vector<uint8_t> flags, fsolid;
    b_flags(B, cs, flags, fsolid);
    PG_CUDA(cudaStreamSynchronize(B->stream));
    PG_CUDA(cudaMemcpy(B->flags, flags.data(), flags.size(), cudaMemcpyHostToDevice));
    std::vector<double> nfl(B->n, 0.0);  // fluid cells per grid (the MG path's lazy projection)
    for (int g = 0; g < B->n; ++g)
        for (i64 c = B->coff[g]; c < B->coff[g + 1]; ++c) nfl[g] += flags[c] != 0;
    if (!B->nfluid) PG_CUDA(cudaMalloc(&B->nfluid, sizeof(double) * B->n));
    PG_CUDA(cudaMemcpy(B->nfluid, nfl.data(), sizeof(double) * B->n, cudaMemcpyHostToDevice));
    if (cs) {
        if (!B->face_solid) PG_CUDA(cudaMalloc(&B->face_solid, (size_t)B->nfaces));
        PG_CUDA(cudaMemcpy(B->face_solid, fsolid.data(), fsolid.size(), cudaMemcpyHostToDevice));
    } else if (B->face_solid) {
        PG_CUDA(cudaFree(B->face_solid));
        B->face_solid = nullptr;
    }
    B->mask_version += 1;
    return PG_OK;
}

int pg_batch_tile(const pg_batch* B, int32_t* tx, int32_t* ty, int32_t* fused) {
    if (!B) return bad_arg("pg_batch_tile: NULL batch");
    if (tx) *tx = B->tx;
    if (ty) *ty = B->ty;
    if (fused) *fused = B->fused;
    return PG_OK;
}

int pg_batch_set_tile(pg_batch* B, int32_t tx, int32_t ty, int32_t fused) {
    if (!B) return bad_arg("pg_batch_set_tile: NULL batch");
    if (tx < 1 || ty < 1 || tx * ty > kBMaxThreads || (tx * ty) % 32) return bad_arg("pg_batch_set_tile: bad shape");
    B->fused = fused ? 1 : 0;
    if (tx == B->tx && ty == B->ty) return PG_OK;
    PG_CUDA(cudaStreamSynchronize(B->stream));
    return build_tiles(B, tx, ty);
}

int pg_batch_step_f32(pg_batch* B, const pg_step_params* prm, float* vel, float* rho, float* pressure,
                      pg_pcg_stats* stats) {
    if (!B || !prm || !vel || !rho || !pressure) return bad_arg("pg_batch_step_f32: NULL argument");
    if (prm->source_enabled) return bad_arg("pg_batch_step_f32: use source_field for batches");
    const pg_solver_params* sp = &prm->solver;
    if (sp->precond != PG_PRECOND_NONE && sp->precond != PG_PRECOND_JACOBI && sp->precond != PG_PRECOND_MG)
        return bad_arg("pg_batch_step_f32: unknown preconditioner");
    if (sp->refine > 0) return bad_arg("pg_batch_step_f32: refinement is not available for batches");
    if (sp->precond == PG_PRECOND_MG) {
        const int rc = bmg_ensure(B, (float)prm->dt);
        if (rc) return rc;
    }
    cudaStream_t s = B->stream;
    const float dt = (float)prm->dt;
    const int nt = B->tx * B->ty;
    const int nbc = bblocks(B, B->ntiles), nbe = bblocks(B, B->ntiles_ext);
    if (prm->source_field)
        PG_LAUNCH(KK_STEP_MISC, s,
                  k_b_source_field<<<std::max(1, (int)std::min<i64>((B->ncells + 255) / 256, (i64)B->num_sms * 8)), 256, 0, s>>>(
                      rho, (const float*)prm->source_field, B->ncells));
    PG_LAUNCH(KK_ADVECT, s,
              k_b_advect<<<nbc, nt, 0, s>>>(B->tmp, rho, vel, B->ginfo, B->tiles, B->ntiles, B->tx, B->ty, -dt));
    PG_LAUNCH(KK_ADVECT_MAC, s,
              k_b_advect_mac<<<nbe, nt, 0, s>>>(B->vtmp, vel, B->ginfo, B->tiles_ext, B->ntiles_ext, B->tx, B->ty, -dt));
    PG_CUDA(cudaMemcpyAsync(rho, B->tmp, 4 * (size_t)B->ncells, cudaMemcpyDeviceToDevice, s));
    PG_CUDA(cudaMemcpyAsync(vel, B->vtmp, 4 * (size_t)B->nfaces, cudaMemcpyDeviceToDevice, s));
    if (prm->walls_after_advect || prm->buoyancy != 0.0)
        PG_LAUNCH(KK_STEP_MISC, s,
                  k_b_walls_buoyancy<<<nbe, nt, 0, s>>>(vel, rho, B->ginfo, B->tiles_ext, B->ntiles_ext, B->tx, B->ty,
                                                        prm->walls_after_advect, (float)(prm->dt * prm->buoyancy)));
    PG_LAUNCH(KK_RHS, s,
              k_b_rhs<<<nbc, nt, 0, s>>>(B->b, vel, B->flags, B->face_solid, B->ginfo, B->tiles, B->ntiles, B->tx,
                                         B->ty));
    PG_CHECK_LAUNCH();
    int rc = sp->precond == PG_PRECOND_MG       ? b_solve<PM_ZBUF>(B, sp, dt, pressure, -1)
             : sp->precond == PG_PRECOND_JACOBI ? b_solve<PM_JACOBI>(B, sp, dt, pressure, -1)
                                                : b_solve<PM_NONE>(B, sp, dt, pressure, -1);
    if (rc) return rc;
    PG_LAUNCH(KK_PROJECT, s,
              k_b_project<<<nbe, nt, 0, s>>>(vel, pressure, B->flags, B->ginfo, B->tiles_ext, B->ntiles_ext, B->tx,
                                             B->ty, dt, prm->zero_solid_after_project));
    PG_CHECK_LAUNCH();
    PG_CUDA(cudaStreamSynchronize(s));
    std::vector<BState> hs(B->n);
    PG_CUDA(cudaMemcpy(hs.data(), B->state, sizeof(BState) * B->n, cudaMemcpyDeviceToHost));
    int worst = PG_OK;
    for (int g = 0; g < B->n; ++g) {
        if (stats) {
            pg_pcg_stats& o = stats[g];
            o.iterations = hs[g].iter;
            o.refinements = 0;
            o.residual_max = hs[g].rmax;
            o.b_max = hs[g].bmax;
            o.threshold = hs[g].thr;
            o.true_residual_max = -1.0;
            o.status = hs[g].status;
            o.reserved = 0;
        }
        if (hs[g].status != PG_OK && worst == PG_OK) worst = hs[g].status;
    }
    return worst;
}

int pg_batch_autotune(pg_batch* B, const char* cache_path) {
    if (!B) return bad_arg("pg_batch_autotune: NULL batch");
    const std::string key = tune_key(B);
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string k;
        int tx, ty, fu;
        while (in >> k >> tx >> ty >> fu)
            if (k == key) return pg_batch_set_tile(B, tx, ty, fu);
    }
    // Time 24 host-driven CG iterations of a synthetic right-hand side for
    // each candidate tile shape and fusion choice.
    const int cand[][2] = {{32, 8}, {64, 4}, {32, 4}, {16, 16}, {128, 2}, {64, 2}};
    cudaStream_t s = B->stream;
    float* x = nullptr;
    PG_CUDA(cudaMalloc(&x, 4 * (size_t)B->ncells));
    std::vector<float> hb((size_t)B->ncells);
    for (size_t i = 0; i < hb.size(); ++i) hb[i] = (float)((i * 2654435761u) % 1000) * 1e-3f - 0.5f;
    PG_CUDA(cudaMemcpy(B->b, hb.data(), 4 * hb.size(), cudaMemcpyHostToDevice));
    pg_solver_params prm{};
    prm.precond = PG_PRECOND_NONE;
    prm.rel_stop = 1;
    prm.rel_tol = 1e-12;
    prm.max_iter = 1 << 20;
    cudaEvent_t e0, e1;
    PG_CUDA(cudaEventCreate(&e0));
    PG_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int btx = 32, bty = 8, bfu = 1;
    for (const auto& c : cand) {
        for (int fu = 1; fu >= 0; --fu) {
            int rc = pg_batch_set_tile(B, c[0], c[1], fu);
            if (rc) return rc;
            b_solve<PM_NONE>(B, &prm, 1.0f, x, 8);  // warm-up
            PG_CUDA(cudaEventRecord(e0, s));
            b_solve<PM_NONE>(B, &prm, 1.0f, x, 24);
            PG_CUDA(cudaEventRecord(e1, s));
            PG_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            PG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                btx = c[0];
                bty = c[1];
                bfu = fu;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(x);
    int rc = pg_batch_set_tile(B, btx, bty, bfu);
    if (rc) return rc;
    if (cache_path) {
        std::ofstream o(cache_path, std::ios::app);
        o << key << " " << btx << " " << bty << " " << bfu << "\n";
    }
    return PG_OK;
}

}  // extern "C"
