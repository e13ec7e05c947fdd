// pg_batch_mg.cu -- geometric multigrid V-cycle for batches of 2D grids
// (PG_PRECOND_MG in pg_batch_step_f32; an extension behind the reference's
// `Preconditioner` trait, pcg.rs:4-6).
//
// Every grid gets the hierarchy of the single-grid preconditioner
// (pg_mg.cu): cell-centred levels halving each side (rounded up) until the
// shorter side is <= 2 or the level has <= 64 cells; coarse face weights are
// half the sum of the fine weights crossing the coarse face; restriction sums
// the children's residuals, prolongation adds the parent's correction;
// red-black Gauss-Seidel, `nsmooth` sweeps (red, black) before and (black,
// red) after, so the V-cycle is symmetric; the coarsest level is solved in
// shared memory by symmetric sweeps.  Grids have different depths:
// level l of the batch packs level l of every grid deep enough, each stage
// is ONE launch over a tile list of that level (smoothing tiles of 64 x 8
// cells on level 0, 64 x 32 above, one cell of the colour per row and
// thread; restriction tiles of 32 x 8 coarse cells), and the coarsest solve
// is one launch with one block per grid, each at its own coarsest level.  Tiles of grids whose CG has
// converged return at once.  The last fine half-sweep writes one z.r
// partial per tile; a per-grid block folds them in a fixed order.
#include <algorithm>
#include <vector>

#include "pg_batch.cuh"

namespace pg {

constexpr int kBmgMaxLevels = 16;
constexpr int kBmgCoarseMax = 2048;
constexpr int kBmgCoarseThreads = 512;
constexpr int kSmTX = 32, kSmTY = 8;  // smoothing block: 256 threads, 32 x 8
// rows per thread (kSmTY apart) on level 0 and on the coarser levels: a
// smoothing tile is 64 x (8 sm_rows) cells
constexpr int kSmRows0 = 1, kSmRows = 4;
__host__ __device__ constexpr int sm_rows(bool l0) { return l0 ? kSmRows0 : kSmRows; }
constexpr int kRtX = 32, kRtY = 8;    // restriction tile: 32 x 8 coarse cells

struct BLevel {
    int h, w;     // this grid's dims at this level
    i64 off;      // its first cell in the level's packed arrays (level 0: the batch offset)
    int coarse;   // the grid's coarsest level
    int t0, t1;   // its smoothing tiles (level 0)
    int ch, cw;   // dims at the next level (0 if none)
    i64 coff;     // first cell at the next level
};

struct CoarseInfo {
    const float* wx;
    const float* wy;
    const float* invd;
    float* e;
    const float* f;
    int h, w, level;
    i64 off;
};

struct BatchMg {
    int nlev = 0;  // levels of the deepest grid
    float dt = 0.f;
    unsigned long long mask_version = 0;
    uint64_t id = 0;
    std::vector<void*> allocs;
    BLevel* info[kBmgMaxLevels] = {};
    Tile* stiles[kBmgMaxLevels] = {};
    int nst[kBmgMaxLevels] = {};
    int nsmoothing[kBmgMaxLevels] = {};  // grids smoothing at this level
    Tile* rtiles[kBmgMaxLevels] = {};
    int nrt[kBmgMaxLevels] = {};
    float* wx[kBmgMaxLevels] = {};
    float* wy[kBmgMaxLevels] = {};
    float* invd[kBmgMaxLevels] = {};
    float* e[kBmgMaxLevels] = {};
    float* f[kBmgMaxLevels] = {};
    CoarseInfo* coarse = nullptr;
    double* partials = nullptr;
    Pockets pockets;  // fluid components of the grids with more than one
};

// Device view of one level of the batch.
struct BLv {
    const BLevel* info;
    const float* wx;
    const float* wy;
    const float* invd;
    float* e;
    const float* f;
    const uint8_t* flags;  // level 0
    const float* ec;       // next level's correction (prolongation)
    float dt;
    int level;
};

template <bool L0> struct BCell {
    float wxl, wxh, wyl, wyh, inv;
    __device__ __forceinline__ BCell(const BLv& v, i64 c, int y, int x, int h, int w) {
        if (L0) {
            const uint8_t f = v.flags[c];
            wxl = (f & XLO) ? v.dt : 0.f;
            wxh = (f & XHI) ? v.dt : 0.f;
            wyl = (f & YLO) ? v.dt : 0.f;
            wyh = (f & YHI) ? v.dt : 0.f;
            const int n = __popc((unsigned)f);
            inv = n ? __frcp_rn((float)n * v.dt) : 0.f;
        } else {
            wxl = v.wx[c];
            wxh = x + 1 < w ? v.wx[c + 1] : 0.f;
            wyl = v.wy[c];
            wyh = y + 1 < h ? v.wy[c + w] : 0.f;
            inv = v.invd[c];
        }
    }
};

enum { BNB_PLAIN = 0, BNB_FIRST = 1, BNB_PROLONG = 2, BNB_SELF = 3 };

template <bool L0, int MODE>
__device__ __forceinline__ float bnb(const BLv& v, const BLevel& L, i64 k, int y, int x) {
    if (MODE == BNB_FIRST) {
        if (L0) {
            const int n = __popc((unsigned)v.flags[k]);
            return n ? v.f[k] * __frcp_rn((float)n * v.dt) : 0.f;
        }
        return v.f[k] * v.invd[k];
    }
    if (MODE == BNB_PROLONG) return v.e[k] + v.ec[L.coff + (i64)(y >> 1) * L.cw + (x >> 1)];
    return v.e[k];
}

// What one red-black update of cell c = (y, x) reads, loaded before any of
// it is used: a neighbour outside the grid is read at the cell itself (the
// weight of a boundary face is 0, so it is never added), so a thread's
// loads for all its rows issue together instead of waiting on the flags.
template <bool L0, int MODE> struct BUpd {
    float f, inv, w[4], n[4];
    __device__ __forceinline__ void load(const BLv& v, const BLevel& L, i64 c, int y, int x) {
        const int h = L.h, wd = L.w;
        const bool xl = x > 0, xh = x + 1 < wd, yl = y > 0, yh = y + 1 < h;
        f = v.f[c];
        if (L0) {
            const unsigned fl = v.flags[c];
            w[0] = (fl & XLO) ? v.dt : 0.f;
            w[1] = (fl & XHI) ? v.dt : 0.f;
            w[2] = (fl & YLO) ? v.dt : 0.f;
            w[3] = (fl & YHI) ? v.dt : 0.f;
            const int nn = __popc(fl);
            inv = nn ? __frcp_rn((float)nn * v.dt) : 0.f;
        } else {
            const float wxh = v.wx[xh ? c + 1 : c], wyh = v.wy[yh ? c + wd : c];
            w[0] = v.wx[c];
            w[1] = xh ? wxh : 0.f;
            w[2] = v.wy[c];
            w[3] = yh ? wyh : 0.f;
            inv = v.invd[c];
        }
        if (MODE != BNB_SELF) {
            n[0] = bnb<L0, MODE>(v, L, xl ? c - 1 : c, y, xl ? x - 1 : x);
            n[1] = bnb<L0, MODE>(v, L, xh ? c + 1 : c, y, xh ? x + 1 : x);
            n[2] = bnb<L0, MODE>(v, L, yl ? c - wd : c, yl ? y - 1 : y, x);
            n[3] = bnb<L0, MODE>(v, L, yh ? c + wd : c, yh ? y + 1 : y, x);
        }
    }
    // f + sum over the open faces of weight * neighbour, times 1 / diagonal
    __device__ __forceinline__ float value() const {
        float s = f;
        if (MODE != BNB_SELF) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (w[j] != 0.f) s += w[j] * n[j];
        }
        return s * inv;
    }
};

// One red-black half-sweep of colour `color` at one level of every grid
// that smooths there; with RZ (level 0, last) also the per-tile z.r and
// sum(z).  A thread updates one cell of the colour in each of sm_rows(L0)
// rows (kSmTY apart): loads of all rows first, then the updates, then
// the stores.
template <bool L0, int MODE, bool RZ>
__global__ void __launch_bounds__(kSmTX * kSmTY, L0 ? 8 : 3)
    k_bmg_smooth(BLv v, const Tile* __restrict__ tiles, int ntiles, int color, const BState* __restrict__ st,
                 double* __restrict__ partials) {
    __shared__ F2 sm[64];
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        if (st[t.grid].done) continue;  // uniform per block
        const BLevel L = v.info[t.grid];
        const bool upd = L.coarse > v.level;
        if (!upd && !RZ) continue;
        const int iy = threadIdx.x / kSmTX, ix = threadIdx.x % kSmTX;
        Acc<float> acc, zs;  // z.r and sum(z) (RZ)
        constexpr int R = sm_rows(L0);
        BUpd<L0, MODE> u[R];
        float ev[R], eo[R], fo[R];  // the colour's new values; the other colour's e, f (RZ)
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int y = t.y0 + iy + r * kSmTY;
            const int x = t.x0 + 2 * ix + ((y + color) & 1);
            if (y < L.h && x < L.w) {
                const i64 c = L.off + (i64)y * L.w + x;
                if (upd) u[r].load(v, L, c, y, x);
                else if (RZ) {
                    u[r].f = v.f[c];
                    ev[r] = v.e[c];
                }
            }
            // the other colour is not written by this launch: read it now
            const int xo = t.x0 + 2 * ix + ((y + color + 1) & 1);
            if (RZ && y < L.h && xo < L.w) {
                const i64 c = L.off + (i64)y * L.w + xo;
                eo[r] = v.e[c];
                fo[r] = v.f[c];
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int y = t.y0 + iy + r * kSmTY;
            const int x = t.x0 + 2 * ix + ((y + color) & 1);
            if (y < L.h && x < L.w) {
                if (upd) {
                    ev[r] = u[r].value();
                    v.e[L.off + (i64)y * L.w + x] = ev[r];
                }
                if (RZ) {
                    acc.add(ev[r] * u[r].f);
                    zs.add(ev[r]);
                }
            }
            const int xo = t.x0 + 2 * ix + ((y + color + 1) & 1);
            if (RZ && y < L.h && xo < L.w) {
                acc.add(eo[r] * fo[r]);
                zs.add(eo[r]);
            }
        }
        if (RZ) {
            double a, b;
            tsum2(f2_of(acc), f2_of(zs), sm, &a, &b);
            if (threadIdx.x == 0) {
                partials[2 * (i64)ti] = a;
                partials[2 * (i64)ti + 1] = b;
            }
        }
    }
}

// Residual of level l restricted (summed over children) to level l+1.
template <bool L0>
__global__ void __launch_bounds__(kRtX * kRtY)
    k_bmg_restrict(BLv v, float* __restrict__ fc, const Tile* __restrict__ tiles, int ntiles,
                   const BState* __restrict__ st) {
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        if (st[t.grid].done) continue;
        const BLevel L = v.info[t.grid];
        const int Y = t.y0 + (int)threadIdx.x / kRtX, X = t.x0 + (int)threadIdx.x % kRtX;
        if (Y >= L.ch || X >= L.cw) continue;
        // the (up to) four children's loads first, then their residuals in
        // row-major order
        BUpd<L0, BNB_PLAIN> u[4];
        float ec[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int y = 2 * Y + (k >> 1), x = 2 * X + (k & 1);
            if (y < L.h && x < L.w) {
                const i64 c = L.off + (i64)y * L.w + x;
                u[k].load(v, L, c, y, x);
                ec[k] = v.e[c];
            }
        }
        float sum = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int y = 2 * Y + (k >> 1), x = 2 * X + (k & 1);
            if (y < L.h && x < L.w) {
                float a = 0.f;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (u[k].w[j] != 0.f) a += u[k].w[j] * (ec[k] - u[k].n[j]);
                sum += u[k].f - a;
            }
        }
        fc[L.coff + (i64)Y * L.cw + X] = sum;
    }
}

// Each grid's coarsest level: one block per grid, shared memory, symmetric
// red-black sweeps from e = 0 (coarse_pairs of its shape).  A grid too small to
// coarsen is solved this way on level 0 (weights from its flags).
__global__ void __launch_bounds__(kBmgCoarseThreads)
    k_bmg_coarse(const CoarseInfo* __restrict__ ci, const BState* __restrict__ st, float* __restrict__ z,
                 const float* __restrict__ r, const uint8_t* __restrict__ flags, float dt) {
    __shared__ float se[kBmgCoarseMax], sf[kBmgCoarseMax], sx[kBmgCoarseMax], sy[kBmgCoarseMax], si[kBmgCoarseMax];
    const int g = blockIdx.x;
    if (st[g].done) return;
    const CoarseInfo C = ci[g];
    const int n = C.h * C.w;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        se[c] = 0.f;
        if (C.level == 0) {
            const uint8_t fl = flags[C.off + c];
            sf[c] = r[C.off + c];
            sx[c] = (fl & XLO) ? dt : 0.f;
            sy[c] = (fl & YLO) ? dt : 0.f;
            const int k = __popc((unsigned)fl);
            si[c] = k ? __frcp_rn((float)k * dt) : 0.f;
        } else {
            sf[c] = C.f[c];
            sx[c] = C.wx[c];
            sy[c] = C.wy[c];
            si[c] = C.invd[c];
        }
    }
    __syncthreads();
    const int pairs = coarse_pairs(1, C.h, C.w);
    for (int it = 0; it < 4 * pairs; ++it) {
        const int color = it < 2 * pairs ? (it & 1) : ((it & 1) ^ 1);
        for (int c = threadIdx.x; c < n; c += blockDim.x) {
            const int y = c / C.w, x = c - y * C.w;
            if (((x + y) & 1) != color) continue;
            float s = sf[c];
            if (x > 0) s += sx[c] * se[c - 1];
            if (x + 1 < C.w) s += sx[c + 1] * se[c + 1];
            if (y > 0) s += sy[c] * se[c - C.w];
            if (y + 1 < C.h) s += sy[c + C.w] * se[c + C.w];
            se[c] = s * si[c];
        }
        __syncthreads();
    }
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        if (C.level == 0)
            z[C.off + c] = se[c];
        else
            C.e[c] = se[c];
    }
}

// Coarse face weights of level l+1 from level l (tiles over level l+1).
template <bool L0>
__global__ void k_bmg_coarsen(BLv v, float* __restrict__ wxc, float* __restrict__ wyc, const Tile* __restrict__ tiles,
                              int ntiles) {
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const BLevel L = v.info[t.grid];
        const int Y = t.y0 + (int)threadIdx.x / kRtX, X = t.x0 + (int)threadIdx.x % kRtX;
        if (Y >= L.ch || X >= L.cw) continue;
        const int y0 = 2 * Y, y1 = min(2 * Y + 2, L.h), x0 = 2 * X, x1 = min(2 * X + 2, L.w);
        float sx = 0.f, sy = 0.f;
        for (int y = y0; y < y1; ++y)
            for (int x = x0; x < x1; ++x) {
                const i64 c = L.off + (i64)y * L.w + x;
                const BCell<L0> cl(v, c, y, x, L.h, L.w);
                if (x == x0) sx += cl.wxl;
                if (y == y0) sy += cl.wyl;
            }
        const i64 C = L.coff + (i64)Y * L.cw + X;
        wxc[C] = 0.5f * sx;
        wyc[C] = 0.5f * sy;
    }
}

// 1 / diagonal of level l+1 (v = level l+1's view; tiles over its cells).
__global__ void k_bmg_invd(BLv v, float* __restrict__ invd, const Tile* __restrict__ tiles, int ntiles) {
    FOR_TILES(tiles, ntiles) {
        const Tile t = tiles[ti];
        const BLevel L = v.info[t.grid];
        const int y = t.y0 + (int)threadIdx.x / kRtX, x = t.x0 + (int)threadIdx.x % kRtX;
        if (y >= L.h || x >= L.w) continue;
        const i64 c = L.off + (i64)y * L.w + x;
        float s = v.wx[c] + v.wy[c];
        if (x + 1 < L.w) s += v.wx[c + 1];
        if (y + 1 < L.h) s += v.wy[c + L.w];
        invd[c] = s > 0.f ? 1.f / s : 0.f;
    }
}

// Per grid: z.r = sum of its level-0 tile partials (fixed order).
// first: sigma = z.r; else beta = z.r / sigma, sigma = z.r.
__global__ void k_bmg_rz_finalize(const BLevel* __restrict__ info0, BState* __restrict__ st,
                                  const double* __restrict__ partials, int n, int first) {
    __shared__ double sm[32];
    const int g = blockIdx.x;
    if (g >= n) return;
    BState& S = st[g];
    if (S.done) return;
    const BLevel L = info0[g];
    double a = 0.0, zsum = 0.0;
    for (int t = L.t0 + threadIdx.x; t < L.t1; t += blockDim.x) {
        a += partials[2 * (i64)t];
        zsum += partials[2 * (i64)t + 1];
    }
    a = bsum(a, sm);
    zsum = bsum(zsum, sm);
    if (threadIdx.x != 0) return;
    if (S.nfluid > 0.0) {  // z stands for z - m on the fluid cells: (z - m).r = z.r - m sum(r)
        const double m = zsum / S.nfluid;
        S.zmean = m;
        S.fzm = (float)m;
        a -= m * S.rsum;
    }
    if (!isfinite(a)) {
        S.status = PG_NAN_DETECTED;
        S.done = 1;
        return;
    }
    if (first) {
        S.sigma = a;
    } else {
        S.beta = a / S.sigma;
        S.fbeta = (float)S.beta;
        S.sigma = a;
    }
}

// ---------------------------------------------------------------------------
// host side

static uint64_t next_bmg_id() {
    static uint64_t n = 0;
    return ++n;
}

void bmg_release(pg_batch* B) {
    if (!B->mg) return;
    release_pockets(&B->mg->pockets);
    for (void* p : B->mg->allocs) cudaFree(p);
    delete B->mg;
    B->mg = nullptr;
}

uint64_t bmg_id(const pg_batch* B) { return B->mg ? B->mg->id : 0; }

static BLv view(const pg_batch* B, int l) {
    const BatchMg& M = *B->mg;
    BLv v;
    v.info = M.info[l];
    v.wx = M.wx[l];
    v.wy = M.wy[l];
    v.invd = M.invd[l];
    v.e = l == 0 ? B->z : M.e[l];
    v.f = l == 0 ? B->r : M.f[l];
    v.flags = B->flags;
    v.ec = l + 1 < M.nlev ? M.e[l + 1] : nullptr;
    v.dt = M.dt;
    v.level = l;
    return v;
}

static int bmg_blocks(const pg_batch* B, int ntiles) { return std::max(1, std::min(ntiles, B->num_sms * 8)); }

static int bmg_build(pg_batch* B, float dt);

int bmg_ensure(pg_batch* B, float dt) {
    if (B->mg && B->mg->dt == dt && B->mg->mask_version == B->mask_version) return PG_OK;
    bmg_release(B);
    if (!B->z) PG_CUDA(cudaMalloc(&B->z, sizeof(float) * (size_t)B->ncells));
    const int rc = bmg_build(B, dt);
    if (rc) bmg_release(B);
    return rc;
}

static int bmg_build(pg_batch* B, float dt) {
    BatchMg* M = new BatchMg();
    M->dt = dt;
    M->mask_version = B->mask_version;
    M->id = next_bmg_id();
    const int n = B->n;
    // level shapes per grid (the single-grid rule)
    std::vector<std::vector<int>> hs(n), wsz(n);
    std::vector<int> coarse(n);
    int nlev = 1;
    for (int g = 0; g < n; ++g) {
        int h = B->h[g], w = B->w[g];
        hs[g].push_back(h);
        wsz[g].push_back(w);
        while ((int)hs[g].size() < kBmgMaxLevels) {
            if (std::min(h, w) <= 2 || (i64)h * w <= 64) break;
            h = (h + 1) / 2;
            w = (w + 1) / 2;
            hs[g].push_back(h);
            wsz[g].push_back(w);
        }
        coarse[g] = (int)hs[g].size() - 1;
        if ((i64)hs[g].back() * wsz[g].back() > kBmgCoarseMax) {
            delete M;
            return bad_arg("PG_PRECOND_MG: a grid of the batch does not coarsen to a small enough level");
        }
        nlev = std::max(nlev, coarse[g] + 1);
    }
    M->nlev = nlev;
    B->mg = M;
    // packed offsets per level, tiles
    std::vector<std::vector<BLevel>> info(nlev, std::vector<BLevel>(n));
    std::vector<i64> lvcells(nlev, 0);
    for (int l = 0; l < nlev; ++l)
        for (int g = 0; g < n; ++g) {
            BLevel& L = info[l][g];
            L = BLevel{};
            L.coarse = coarse[g];
            if (l > coarse[g]) continue;
            L.h = hs[g][l];
            L.w = wsz[g][l];
            L.off = l == 0 ? B->coff[g] : lvcells[l];
            if (l > 0) lvcells[l] += (i64)L.h * L.w;
        }
    lvcells[0] = B->ncells;
    for (int l = 0; l < nlev; ++l)
        for (int g = 0; g < n; ++g)
            if (l < coarse[g]) {
                info[l][g].ch = hs[g][l + 1];
                info[l][g].cw = wsz[g][l + 1];
                info[l][g].coff = info[l + 1][g].off;
            }
    auto dalloc = [&](void** p, size_t bytes) -> int {
        cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(batch mg)");
        M->allocs.push_back(*p);
        return PG_OK;
    };
    int rc;
    for (int l = 0; l < nlev; ++l) {
        std::vector<Tile> st, rt;
        for (int g = 0; g < n; ++g) {
            BLevel& L = info[l][g];
            if (l == 0) L.t0 = (int)st.size();
            if (l == 0 || l < coarse[g]) {
                for (int y0 = 0; y0 < L.h; y0 += kSmTY * sm_rows(l == 0))
                    for (int x0 = 0; x0 < L.w; x0 += 2 * kSmTX) st.push_back(Tile{g, y0, x0});
                if (l < coarse[g]) M->nsmoothing[l] += 1;
            }
            if (l == 0) L.t1 = (int)st.size();
            if (l < coarse[g])
                for (int y0 = 0; y0 < L.ch; y0 += kRtY)
                    for (int x0 = 0; x0 < L.cw; x0 += kRtX) rt.push_back(Tile{g, y0, x0});
        }
        M->nst[l] = (int)st.size();
        M->nrt[l] = (int)rt.size();
        if ((rc = dalloc((void**)&M->info[l], sizeof(BLevel) * n)) ||
            (rc = dalloc((void**)&M->stiles[l], sizeof(Tile) * st.size())) ||
            (rc = dalloc((void**)&M->rtiles[l], sizeof(Tile) * rt.size())))
            return rc;
        PG_CUDA(cudaMemcpy(M->info[l], info[l].data(), sizeof(BLevel) * n, cudaMemcpyHostToDevice));
        if (!st.empty()) PG_CUDA(cudaMemcpy(M->stiles[l], st.data(), sizeof(Tile) * st.size(), cudaMemcpyHostToDevice));
        if (!rt.empty()) PG_CUDA(cudaMemcpy(M->rtiles[l], rt.data(), sizeof(Tile) * rt.size(), cudaMemcpyHostToDevice));
        if (l >= 1) {
            const size_t b = sizeof(float) * (size_t)lvcells[l];
            if ((rc = dalloc((void**)&M->wx[l], b)) || (rc = dalloc((void**)&M->wy[l], b)) ||
                (rc = dalloc((void**)&M->invd[l], b)) || (rc = dalloc((void**)&M->e[l], b)) ||
                (rc = dalloc((void**)&M->f[l], b)))
                return rc;
        }
        if (l == 0 && (rc = dalloc((void**)&M->partials, 2 * sizeof(double) * st.size()))) return rc;
    }
    std::vector<CoarseInfo> ci(n);
    for (int g = 0; g < n; ++g) {
        const int c = coarse[g];
        const BLevel& L = info[c][g];
        ci[g] = CoarseInfo{M->wx[c] ? M->wx[c] + L.off : nullptr,
                           M->wy[c] ? M->wy[c] + L.off : nullptr,
                           M->invd[c] ? M->invd[c] + L.off : nullptr,
                           M->e[c] ? M->e[c] + L.off : nullptr,
                           M->f[c] ? M->f[c] + L.off : nullptr,
                           L.h, L.w, c, L.off};
        if (c == 0) ci[g].off = B->coff[g];
    }
    // fluid components of every grid with more than one (host labelling, once per mask)
    {
        std::vector<uint8_t> hf((size_t)B->ncells);
        PG_CUDA(cudaMemcpy(hf.data(), B->flags, hf.size(), cudaMemcpyDeviceToHost));
        std::vector<i64> cells;
        std::vector<int> start;
        for (int g = 0; g < n; ++g)
            find_pockets(hf.data() + B->coff[g], 2, 1, B->h[g], B->w[g], B->coff[g], cells, start);
        if ((rc = upload_pockets(cells, start, &M->pockets))) return rc;
    }
    if ((rc = dalloc((void**)&M->coarse, sizeof(CoarseInfo) * n))) return rc;
    PG_CUDA(cudaMemcpy(M->coarse, ci.data(), sizeof(CoarseInfo) * n, cudaMemcpyHostToDevice));
    // coarse operators
    cudaStream_t s = B->stream;
    for (int l = 0; l + 1 < nlev; ++l) {
        if (!M->nrt[l]) continue;
        const BLv v = view(B, l);
        const int nb = bmg_blocks(B, M->nrt[l]);
        if (l == 0)
            PG_LAUNCH(KK_MG_SETUP, s, k_bmg_coarsen<true><<<nb, kRtX * kRtY, 0, s>>>(v, M->wx[1], M->wy[1], M->rtiles[0], M->nrt[0]));
        else
            PG_LAUNCH(KK_MG_SETUP, s, k_bmg_coarsen<false><<<nb, kRtX * kRtY, 0, s>>>(v, M->wx[l + 1], M->wy[l + 1], M->rtiles[l], M->nrt[l]));
        const BLv cv = view(B, l + 1);
        PG_LAUNCH(KK_MG_SETUP, s, k_bmg_invd<<<nb, kRtX * kRtY, 0, s>>>(cv, M->invd[l + 1], M->rtiles[l], M->nrt[l]));
    }
    PG_CHECK_LAUNCH();
    return PG_OK;
}

template <bool L0, int MODE, bool RZ>
static void bsmooth(pg_batch* B, cudaStream_t s, int l, int color) {
    BatchMg& M = *B->mg;
    const BLv v = view(B, l);
    PG_LAUNCH(l == 0 ? KK_MG_SMOOTH : KK_MG_SMOOTH_C, s,
              k_bmg_smooth<L0, MODE, RZ><<<bmg_blocks(B, M.nst[l]), kSmTX * kSmTY, 0, s>>>(v, M.stiles[l], M.nst[l],
                                                                                           color, B->state, M.partials));
}

static void bsmooth_any(pg_batch* B, cudaStream_t s, int l, int color, int mode, bool rz = false) {
    if (l == 0) {
        if (mode == BNB_FIRST) bsmooth<true, BNB_FIRST, false>(B, s, l, color);
        else if (mode == BNB_SELF) bsmooth<true, BNB_SELF, false>(B, s, l, color);
        else if (mode == BNB_PROLONG) bsmooth<true, BNB_PROLONG, false>(B, s, l, color);
        else if (rz) bsmooth<true, BNB_PLAIN, true>(B, s, l, color);
        else bsmooth<true, BNB_PLAIN, false>(B, s, l, color);
    } else {
        if (mode == BNB_FIRST) bsmooth<false, BNB_FIRST, false>(B, s, l, color);
        else if (mode == BNB_SELF) bsmooth<false, BNB_SELF, false>(B, s, l, color);
        else if (mode == BNB_PROLONG) bsmooth<false, BNB_PROLONG, false>(B, s, l, color);
        else bsmooth<false, BNB_PLAIN, false>(B, s, l, color);
    }
}

// z = P V(P r), P removing the mean of every fluid component of the grids
// with more than one (r in place).
void bmg_vcycle(pg_batch* B, cudaStream_t s, int nsmooth) {
    BatchMg& M = *B->mg;
    pocket_project(s, B->r, M.pockets);
    for (int l = 0; l + 1 < M.nlev; ++l) {
        if (!M.nsmoothing[l]) continue;
        bsmooth_any(B, s, l, 1, BNB_FIRST);
        if (nsmooth == 1) bsmooth_any(B, s, l, 0, BNB_SELF);
        for (int k = 1; k < nsmooth; ++k) {
            bsmooth_any(B, s, l, 0, BNB_PLAIN);
            bsmooth_any(B, s, l, 1, BNB_PLAIN);
        }
        const BLv v = view(B, l);
        const int nb = bmg_blocks(B, M.nrt[l]);
        if (l == 0)
            PG_LAUNCH(KK_MG_RESTRICT, s, k_bmg_restrict<true><<<nb, kRtX * kRtY, 0, s>>>(v, M.f[1], M.rtiles[0], M.nrt[0], B->state));
        else
            PG_LAUNCH(KK_MG_RESTRICT_C, s, k_bmg_restrict<false><<<nb, kRtX * kRtY, 0, s>>>(v, M.f[l + 1], M.rtiles[l], M.nrt[l], B->state));
    }
    PG_LAUNCH(KK_MG_COARSE, s,
              k_bmg_coarse<<<B->n, kBmgCoarseThreads, 0, s>>>(M.coarse, B->state, B->z, B->r, B->flags, M.dt));
    bool rz_done = false;
    for (int l = M.nlev - 2; l >= 0; --l) {
        if (!M.nsmoothing[l]) continue;
        bsmooth_any(B, s, l, 1, BNB_PROLONG);
        for (int k = 0; k < nsmooth; ++k) {
            if (k > 0) bsmooth_any(B, s, l, 1, BNB_PLAIN);
            const bool rz = l == 0 && k == nsmooth - 1;
            bsmooth_any(B, s, l, 0, BNB_PLAIN, rz);
            rz_done = rz_done || rz;
        }
    }
    // No grid smooths on level 0 (every grid too small to coarsen): the
    // z.r partials alone.
    if (!rz_done) bsmooth<true, BNB_PLAIN, true>(B, s, 0, 0);
    pocket_project(s, B->z, M.pockets);
}

void bmg_rz_finalize(pg_batch* B, cudaStream_t s, int first) {
    BatchMg& M = *B->mg;
    PG_LAUNCH(KK_STEP_MISC, s, k_bmg_rz_finalize<<<B->n, 128, 0, s>>>(M.info[0], B->state, M.partials, B->n, first));
}

}  // namespace pg
