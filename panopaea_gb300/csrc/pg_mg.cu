// pg_mg.cu -- geometric multigrid V-cycle used as the CG preconditioner
// (PG_PRECOND_MG; an extension behind the reference's `Preconditioner`
// trait, pcg.rs:4-6).
//
// Cell-centred hierarchy; level l+1 halves every dimension (rounded up; 2D
// grids keep d = 1).  The operator on every level is
//     (A_l e)_c = sum over the faces f of c of  w_f (e_c - e_nb(f)),
// with w_f = dt on open faces of the fine grid (the masked Laplacian of the
// CG) and, on coarse levels, half the sum of the fine weights crossing the
// coarse face (the Galerkin operator of piecewise-constant transfer, scaled
// by 1/2 -- the scale that makes its coarse-grid correction match a
// rediscretisation; obstacles coarsen through the face weights).
// Restriction sums the children's residuals; prolongation adds the parent's
// correction.  Smoother: red-black Gauss-Seidel, `nsmooth` sweeps before
// (red, black) and after (black, red) the coarse correction, so the V-cycle
// is a symmetric operator and CG stays valid.  The coarsest level (at most
// kCoarseMax cells) is solved by one block in shared memory with symmetric
// sweeps (coarse_pairs of its shape).  Every level of at most kTailCells
// cells runs inside one single-block kernel (k_mg_tail).
//
// Fusions: the first pre-smoothing red half-sweep starts from e = 0, so red
// values are f*invd and the black half-sweep computes them on the fly; the
// prolongation is only ever read by the first post-smoothing black
// half-sweep (Gauss-Seidel overwrites the cells it updates), so it is done
// on the fly there.  The last fine-level half-sweep writes z and reduces
// z.r into the CG state.
#include <algorithm>

#include "pg_solve.cuh"

namespace pg {

constexpr int kMgThreads = 256;
constexpr int kCoarseMax = 2048;
constexpr int kCoarseThreads = 512;
constexpr int kMaxLevels = 16;
constexpr int kTailCells = 4096;  // levels at most this large run in the single-block tail

struct MgLevel {
    Dims D;
    float* wx = nullptr;  // low-face weights (levels >= 1)
    float* wy = nullptr;
    float* wz = nullptr;
    float* invd = nullptr;
    float* e = nullptr;  // correction (levels >= 1)
    float* f = nullptr;  // right-hand side (levels >= 1)
};

struct MgHierarchy {
    Dims D0;
    const uint8_t* flags = nullptr;
    double dt = 0.0;
    unsigned long long mask_version = 0;
    int nlev = 0;
    MgLevel lv[kMaxLevels];
    void* mem = nullptr;
    uint64_t id = 0;  // unique per build (CUDA-graph cache key)
    Pockets pockets;  // fluid components (empty when the fluid is connected)
    int tail = 0;     // first level handled by the single-block tail kernel (nlev: none)
};

static uint64_t next_hierarchy_id() {
    static uint64_t n = 0;
    return ++n;
}

// Read-only view of one level for the kernels.
struct LV {
    int nd;
    int d, h, w;
    const uint8_t* flags;  // level 0
    const float* wx;
    const float* wy;
    const float* wz;
    const float* invd;
    float dt;
    __device__ __forceinline__ int nc() const { return d * h * w; }
};

// Face weights (lo, hi per axis) and 1/diag of cell c at (z, y, x).
template <bool L0> struct Cell {
    float wxl, wxh, wyl, wyh, wzl, wzh, inv;
    __device__ __forceinline__ Cell(const LV& v, int c, int z, int y, int x) {
        if (L0) {
            const uint8_t f = v.flags[c];
            wxl = (f & XLO) ? v.dt : 0.f;
            wxh = (f & XHI) ? v.dt : 0.f;
            wyl = (f & YLO) ? v.dt : 0.f;
            wyh = (f & YHI) ? v.dt : 0.f;
            wzl = (f & ZLO) ? v.dt : 0.f;
            wzh = (f & ZHI) ? v.dt : 0.f;
            const int n = __popc((unsigned)f);
            inv = n ? __frcp_rn((float)n * v.dt) : 0.f;
        } else {
            const int hw = v.h * v.w;
            wxl = v.wx[c];
            wxh = x + 1 < v.w ? v.wx[c + 1] : 0.f;
            wyl = v.wy[c];
            wyh = y + 1 < v.h ? v.wy[c + v.w] : 0.f;
            if (v.nd == 3) {
                wzl = v.wz[c];
                wzh = z + 1 < v.d ? v.wz[c + hw] : 0.f;
            } else {
                wzl = wzh = 0.f;
            }
            inv = v.invd[c];
        }
    }
};

// Neighbour value accessor modes of the smoother.
enum { NB_PLAIN = 0, NB_FIRST = 1 /* e = f*invd */, NB_PROLONG = 2 /* e + ec[parent] */, NB_SELF = 3 };

template <bool L0, int MODE>
__device__ __forceinline__ float nbval(const LV& v, const float* __restrict__ e, const float* __restrict__ f,
                                       const float* __restrict__ ec, int cw, int ch, int k, int z, int y, int x) {
    if (MODE == NB_FIRST) {
        if (L0) {
            const int n = __popc((unsigned)v.flags[k]);
            return n ? f[k] * __frcp_rn((float)n * v.dt) : 0.f;
        }
        return f[k] * v.invd[k];
    }
    if (MODE == NB_PROLONG) {
        const int pc = ((v.nd == 3 ? (z >> 1) : 0) * ch + (y >> 1)) * cw + (x >> 1);
        return e[k] + ec[pc];
    }
    return e[k];
}

// One red-black half-sweep over the cells with (x + y + z) & 1 == color.
// With RZ, also reduce z.r (z = e) into the CG state (fine level, last).
template <bool L0, int MODE, bool RZ>
__global__ void __launch_bounds__(kMgThreads)
    k_mg_smooth(LV v, float* __restrict__ e, const float* __restrict__ f, const float* __restrict__ ec, int cw, int ch,
                int color, CgState* st, double* partials) {
    if (st->done) return;
    __shared__ double sm[32];
    const int hw = v.h * v.w;
    const int half = (v.w + 1) >> 1;
    const int nrow = v.d * v.h;
    const int total = nrow * half;
    Acc<float> acc;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int row = i / half, k2 = i - row * half;
        const int z = row / v.h, y = row - z * v.h;
        const int x = 2 * k2 + ((y + z + color) & 1);
        if (x < v.w) {
            const int c = row * v.w + x;
            const Cell<L0> cl(v, c, z, y, x);
            float s = f[c];
            if (MODE == NB_SELF) {  // a half-sweep from e = 0: no neighbour terms
                e[c] = s * cl.inv;
                continue;
            }
            if (cl.wxl != 0.f) s += cl.wxl * nbval<L0, MODE>(v, e, f, ec, cw, ch, c - 1, z, y, x - 1);
            if (cl.wxh != 0.f) s += cl.wxh * nbval<L0, MODE>(v, e, f, ec, cw, ch, c + 1, z, y, x + 1);
            if (cl.wyl != 0.f) s += cl.wyl * nbval<L0, MODE>(v, e, f, ec, cw, ch, c - v.w, z, y - 1, x);
            if (cl.wyh != 0.f) s += cl.wyh * nbval<L0, MODE>(v, e, f, ec, cw, ch, c + v.w, z, y + 1, x);
            if (v.nd == 3) {
                if (cl.wzl != 0.f) s += cl.wzl * nbval<L0, MODE>(v, e, f, ec, cw, ch, c - hw, z - 1, y, x);
                if (cl.wzh != 0.f) s += cl.wzh * nbval<L0, MODE>(v, e, f, ec, cw, ch, c + hw, z + 1, y, x);
            }
            const float en = s * cl.inv;
            e[c] = en;
            if (RZ) acc.add(en * f[c]);
        }
    }
    if (!RZ) return;
    // z.r: red cells here, black cells were final after the previous
    // half-sweep -- reduce both colours: the black part is added by the
    // companion pass below (same kernel, other colour read-only).
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int row = i / half, k2 = i - row * half;
        const int z = row / v.h, y = row - z * v.h;
        const int x = 2 * k2 + ((y + z + color + 1) & 1);
        if (x < v.w) {
            const int c = row * v.w + x;
            acc.add(e[c] * f[c]);
        }
    }
    const double s = block_sum<kMgThreads>(acc.value(), sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    if (!last_block(&st->counter[3])) return;
    const double rz = reduce_partials<false, kMgThreads>(partials, gridDim.x, sm);
    if (threadIdx.x == 0) {
        st->counter[3] = 0;
        cg_finish_rz(st, rz);
    }
}

// Residual of level l restricted (summed over children) to level l+1.
template <bool L0>
__global__ void __launch_bounds__(kMgThreads)
    k_mg_restrict(LV v, const float* __restrict__ e, const float* __restrict__ f, float* __restrict__ fc, int cd,
                  int ch, int cw, CgState* st) {
    if (st->done) return;
    const int hw = v.h * v.w;
    const int nc = cd * ch * cw;
    for (int C = blockIdx.x * blockDim.x + threadIdx.x; C < nc; C += gridDim.x * blockDim.x) {
        const int CZY = C / cw, X = C - CZY * cw;
        const int Z = CZY / ch, Y = CZY - Z * ch;
        float sum = 0.f;
        const int z1 = v.nd == 3 ? min(2 * Z + 2, v.d) : 1;
        const int y1 = min(2 * Y + 2, v.h), x1 = min(2 * X + 2, v.w);
        for (int z = (v.nd == 3 ? 2 * Z : 0); z < z1; ++z)
            for (int y = 2 * Y; y < y1; ++y)
                for (int x = 2 * X; x < x1; ++x) {
                    const int c = (z * v.h + y) * v.w + x;
                    const Cell<L0> cl(v, c, z, y, x);
                    const float ecv = e[c];
                    float a = 0.f;
                    if (cl.wxl != 0.f) a += cl.wxl * (ecv - e[c - 1]);
                    if (cl.wxh != 0.f) a += cl.wxh * (ecv - e[c + 1]);
                    if (cl.wyl != 0.f) a += cl.wyl * (ecv - e[c - v.w]);
                    if (cl.wyh != 0.f) a += cl.wyh * (ecv - e[c + v.w]);
                    if (v.nd == 3) {
                        if (cl.wzl != 0.f) a += cl.wzl * (ecv - e[c - hw]);
                        if (cl.wzh != 0.f) a += cl.wzh * (ecv - e[c + hw]);
                    }
                    sum += f[c] - a;
                }
        fc[C] = sum;
    }
}

// Coarsest level: one block, shared memory, `pairs` (red, black) sweeps then
// `pairs` (black, red) sweeps from e = 0.
__global__ void __launch_bounds__(kCoarseThreads) k_mg_coarse(LV v, float* __restrict__ e, const float* __restrict__ f,
                                                               CgState* st) {
    if (st->done) return;
    __shared__ float se[kCoarseMax], sf[kCoarseMax], sx[kCoarseMax], sy[kCoarseMax], sz[kCoarseMax], si[kCoarseMax];
    const int n = v.nc(), hw = v.h * v.w;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        se[c] = 0.f;
        sf[c] = f[c];
        sx[c] = v.wx[c];
        sy[c] = v.wy[c];
        sz[c] = v.nd == 3 ? v.wz[c] : 0.f;
        si[c] = v.invd[c];
    }
    __syncthreads();
    const int pairs = coarse_pairs(v.d, v.h, v.w);
    for (int it = 0; it < 4 * pairs; ++it) {
        // colours: (0, 1) `pairs` times, then (1, 0) `pairs` times
        const int color = it < 2 * pairs ? (it & 1) : ((it & 1) ^ 1);
        for (int c = threadIdx.x; c < n; c += blockDim.x) {
            const int zy = c / v.w, x = c - zy * v.w;
            const int z = zy / v.h, y = zy - z * v.h;
            if (((x + y + z) & 1) != color) continue;
            float s = sf[c];
            if (x > 0) s += sx[c] * se[c - 1];
            if (x + 1 < v.w) s += sx[c + 1] * se[c + 1];
            if (y > 0) s += sy[c] * se[c - v.w];
            if (y + 1 < v.h) s += sy[c + v.w] * se[c + v.w];
            if (v.nd == 3) {
                if (z > 0) s += sz[c] * se[c - hw];
                if (z + 1 < v.d) s += sz[c + hw] * se[c + hw];
            }
            se[c] = s * si[c];
        }
        __syncthreads();
    }
    for (int c = threadIdx.x; c < n; c += blockDim.x) e[c] = se[c];
}

// ---------------------------------------------------------------------------
// The tail of the V-cycle: every level of at most kTailCells cells, from
// level `lt` down to the coarsest and back, in ONE block with all level data
// in shared memory (the same half-sweeps, restriction, coarsest solve and
// prolongation as the per-level kernels; a block barrier replaces each
// kernel boundary).  Input: the restricted right-hand side of level lt;
// output: its correction e_lt, read by level lt-1's prolongation.

struct TailLevel {
    int nd, d, h, w;
    const float* wx;
    const float* wy;
    const float* wz;
    const float* invd;
};

struct TailArgs {
    int lt, nl, nsmooth;
    float* e_out;       // global e of level lt
    const float* f_in;  // global f of level lt
    TailLevel L[kMaxLevels];
};

template <int MODE>
__device__ __forceinline__ void tail_smooth(const LV& v, float* e, const float* f, const float* ec, int cw, int ch,
                                            int color) {
    const int hw = v.h * v.w, half = (v.w + 1) >> 1, total = v.d * v.h * half;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        const int row = i / half, k2 = i - row * half;
        const int z = row / v.h, y = row - z * v.h;
        const int x = 2 * k2 + ((y + z + color) & 1);
        if (x >= v.w) continue;
        const int c = row * v.w + x;
        const Cell<false> cl(v, c, z, y, x);
        float s = f[c];
        if (MODE == NB_SELF) {
            e[c] = s * cl.inv;
            continue;
        }
        if (cl.wxl != 0.f) s += cl.wxl * nbval<false, MODE>(v, e, f, ec, cw, ch, c - 1, z, y, x - 1);
        if (cl.wxh != 0.f) s += cl.wxh * nbval<false, MODE>(v, e, f, ec, cw, ch, c + 1, z, y, x + 1);
        if (cl.wyl != 0.f) s += cl.wyl * nbval<false, MODE>(v, e, f, ec, cw, ch, c - v.w, z, y - 1, x);
        if (cl.wyh != 0.f) s += cl.wyh * nbval<false, MODE>(v, e, f, ec, cw, ch, c + v.w, z, y + 1, x);
        if (v.nd == 3) {
            if (cl.wzl != 0.f) s += cl.wzl * nbval<false, MODE>(v, e, f, ec, cw, ch, c - hw, z - 1, y, x);
            if (cl.wzh != 0.f) s += cl.wzh * nbval<false, MODE>(v, e, f, ec, cw, ch, c + hw, z + 1, y, x);
        }
        e[c] = s * cl.inv;
    }
    __syncthreads();
}

__device__ __forceinline__ void tail_restrict(const LV& v, const float* e, const float* f, float* fc, int cd, int ch,
                                              int cw) {
    const int hw = v.h * v.w, nc = cd * ch * cw;
    for (int C = threadIdx.x; C < nc; C += blockDim.x) {
        const int CZY = C / cw, X = C - CZY * cw;
        const int Z = CZY / ch, Y = CZY - Z * ch;
        float sum = 0.f;
        const int z1 = v.nd == 3 ? min(2 * Z + 2, v.d) : 1;
        const int y1 = min(2 * Y + 2, v.h), x1 = min(2 * X + 2, v.w);
        for (int z = (v.nd == 3 ? 2 * Z : 0); z < z1; ++z)
            for (int y = 2 * Y; y < y1; ++y)
                for (int x = 2 * X; x < x1; ++x) {
                    const int c = (z * v.h + y) * v.w + x;
                    const Cell<false> cl(v, c, z, y, x);
                    const float ecv = e[c];
                    float a = 0.f;
                    if (cl.wxl != 0.f) a += cl.wxl * (ecv - e[c - 1]);
                    if (cl.wxh != 0.f) a += cl.wxh * (ecv - e[c + 1]);
                    if (cl.wyl != 0.f) a += cl.wyl * (ecv - e[c - v.w]);
                    if (cl.wyh != 0.f) a += cl.wyh * (ecv - e[c + v.w]);
                    if (v.nd == 3) {
                        if (cl.wzl != 0.f) a += cl.wzl * (ecv - e[c - hw]);
                        if (cl.wzh != 0.f) a += cl.wzh * (ecv - e[c + hw]);
                    }
                    sum += f[c] - a;
                }
        fc[C] = sum;
    }
    __syncthreads();
}

constexpr int kTailThreads = 1024;
constexpr int kTailSmemMax = 220 * 1024;

__global__ void __launch_bounds__(kTailThreads) k_mg_tail(TailArgs A, CgState* st) {
    if (st->done) return;
    extern __shared__ float tsm[];
    LV v[kMaxLevels];
    float* E[kMaxLevels];
    float* F[kMaxLevels];
    // carve the shared memory: wx, wy, wz, invd, e, f per level
    float* p = tsm;
    for (int l = A.lt; l < A.nl; ++l) {
        const TailLevel& T = A.L[l];
        const int n = T.d * T.h * T.w;
        float* wx = p;
        float* wy = p + n;
        float* wz = p + 2 * n;
        float* iv = p + 3 * n;
        E[l] = p + 4 * n;
        F[l] = p + 5 * n;
        p += 6 * n;
        for (int c = threadIdx.x; c < n; c += blockDim.x) {
            wx[c] = T.wx[c];
            wy[c] = T.wy[c];
            wz[c] = T.nd == 3 ? T.wz[c] : 0.f;
            iv[c] = T.invd[c];
            if (l == A.lt) F[l][c] = A.f_in[c];
        }
        v[l].nd = T.nd;
        v[l].d = T.d;
        v[l].h = T.h;
        v[l].w = T.w;
        v[l].flags = nullptr;
        v[l].wx = wx;
        v[l].wy = wy;
        v[l].wz = wz;
        v[l].invd = iv;
        v[l].dt = 0.f;
    }
    __syncthreads();
    const int nl = A.nl, ns = A.nsmooth;
    // down
    for (int l = A.lt; l + 1 < nl; ++l) {
        const LV& c = v[l + 1];
        tail_smooth<NB_FIRST>(v[l], E[l], F[l], nullptr, c.w, c.h, 1);
        if (ns == 1) tail_smooth<NB_SELF>(v[l], E[l], F[l], nullptr, c.w, c.h, 0);
        for (int k = 1; k < ns; ++k) {
            tail_smooth<NB_PLAIN>(v[l], E[l], F[l], nullptr, c.w, c.h, 0);
            tail_smooth<NB_PLAIN>(v[l], E[l], F[l], nullptr, c.w, c.h, 1);
        }
        tail_restrict(v[l], E[l], F[l], F[l + 1], c.d, c.h, c.w);
    }
    // coarsest: symmetric red-black Gauss-Seidel from e = 0
    {
        const LV& cv = v[nl - 1];
        float* e = E[nl - 1];
        const float* f = F[nl - 1];
        const int n = cv.d * cv.h * cv.w;
        for (int c = threadIdx.x; c < n; c += blockDim.x) e[c] = 0.f;
        __syncthreads();
        const int pairs = coarse_pairs(cv.d, cv.h, cv.w);
        for (int it = 0; it < 4 * pairs; ++it) {
            const int color = it < 2 * pairs ? (it & 1) : ((it & 1) ^ 1);
            tail_smooth<NB_PLAIN>(cv, e, f, nullptr, 1, 1, color);
        }
    }
    // up
    for (int l = nl - 2; l >= A.lt; --l) {
        const LV& c = v[l + 1];
        tail_smooth<NB_PROLONG>(v[l], E[l], F[l], E[l + 1], c.w, c.h, 1);
        for (int k = 0; k < ns; ++k) {
            if (k > 0) tail_smooth<NB_PLAIN>(v[l], E[l], F[l], nullptr, c.w, c.h, 1);
            tail_smooth<NB_PLAIN>(v[l], E[l], F[l], nullptr, c.w, c.h, 0);
        }
    }
    const int n0 = A.L[A.lt].d * A.L[A.lt].h * A.L[A.lt].w;
    for (int c = threadIdx.x; c < n0; c += blockDim.x) A.e_out[c] = E[A.lt][c];
}

// Coarse face weights: half the sum of the fine weights on the coarse face.
template <bool L0>
__global__ void k_mg_coarsen(LV v, float* __restrict__ wx, float* __restrict__ wy, float* __restrict__ wz, int cd,
                             int ch, int cw) {
    const int nc = cd * ch * cw;
    for (int C = blockIdx.x * blockDim.x + threadIdx.x; C < nc; C += gridDim.x * blockDim.x) {
        const int CZY = C / cw, X = C - CZY * cw;
        const int Z = CZY / ch, Y = CZY - Z * ch;
        const int z0 = v.nd == 3 ? 2 * Z : 0, z1 = v.nd == 3 ? min(2 * Z + 2, v.d) : 1;
        const int y0 = 2 * Y, y1 = min(2 * Y + 2, v.h), x0 = 2 * X, x1 = min(2 * X + 2, v.w);
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (int z = z0; z < z1; ++z)
            for (int y = y0; y < y1; ++y)
                for (int x = x0; x < x1; ++x) {
                    const int c = (z * v.h + y) * v.w + x;
                    const Cell<L0> cl(v, c, z, y, x);
                    if (x == x0) sx += cl.wxl;
                    if (y == y0) sy += cl.wyl;
                    if (z == z0) sz += cl.wzl;
                }
        wx[C] = 0.5f * sx;
        wy[C] = 0.5f * sy;
        wz[C] = 0.5f * sz;
    }
}

__global__ void k_mg_invd(LV v, float* __restrict__ invd) {
    const int n = v.nc(), hw = v.h * v.w;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const int zy = c / v.w, x = c - zy * v.w;
        const int z = zy / v.h, y = zy - z * v.h;
        float s = v.wx[c] + v.wy[c];
        if (x + 1 < v.w) s += v.wx[c + 1];
        if (y + 1 < v.h) s += v.wy[c + v.w];
        if (v.nd == 3) {
            s += v.wz[c];
            if (z + 1 < v.d) s += v.wz[c + hw];
        }
        invd[c] = s > 0.f ? 1.f / s : 0.f;
    }
}

// ---------------------------------------------------------------------------

static LV view(const MgHierarchy& H, int l) {
    const MgLevel& L = H.lv[l];
    LV v;
    v.nd = L.D.nd;
    v.d = (int)L.D.d;
    v.h = (int)L.D.h;
    v.w = (int)L.D.w;
    v.flags = l == 0 ? H.flags : nullptr;
    v.wx = L.wx;
    v.wy = L.wy;
    v.wz = L.wz;
    v.invd = L.invd;
    v.dt = (float)H.dt;
    return v;
}

void release_mg(Extras* ex) {
    if (ex->mg) {
        release_pockets(&ex->mg->pockets);
        cudaFree(ex->mg->mem);
        delete ex->mg;
        ex->mg = nullptr;
    }
}

static int blocks_for(const pg_grid* g, i64 n) { return grid_blocks(g, n, kMgThreads, 8); }

// (Re)build the hierarchy for the grid's current mask and dt.
static int ensure_mg(pg_grid* g, double dt, MgHierarchy** out) {
    Extras* ex = extras_of(g);
    if (ex->mg && ex->mg->dt == dt && ex->mg->mask_version == g->mask_version) {
        *out = ex->mg;
        return PG_OK;
    }
    release_mg(ex);
    if (g->dims.nc() >= (i64)1 << 31) return bad_arg("PG_PRECOND_MG: grid too large for 32-bit level indexing");
    MgHierarchy* H = new MgHierarchy();
    H->id = next_hierarchy_id();
    H->D0 = g->dims;
    H->flags = g->flags;
    H->dt = dt;
    H->mask_version = g->mask_version;
    // level shapes
    Dims D = g->dims;
    H->lv[0].D = D;
    int nl = 1;
    while (nl < kMaxLevels) {
        const i64 mn = D.nd == 3 ? std::min(D.d, std::min(D.h, D.w)) : std::min(D.h, D.w);
        if (mn <= 2 || D.nc() <= 64) break;
        Dims C{D.nd, D.nd == 3 ? (D.d + 1) / 2 : 1, (D.h + 1) / 2, (D.w + 1) / 2};
        H->lv[nl++].D = C;
        D = C;
    }
    H->nlev = nl;
    // The levels from the first one of at most kTailCells cells (level >= 1)
    // down to the coarsest run as one single-block kernel in shared memory.
    H->tail = nl;
    for (int l = 1; l < nl; ++l)
        if (H->lv[l].D.nc() <= kTailCells) {
            H->tail = l;
            break;
        }
    if (H->lv[nl - 1].D.nc() > kCoarseMax) {
        delete H;
        return bad_arg("PG_PRECOND_MG: grid shape does not coarsen to a small enough level (too anisotropic)");
    }
    // one allocation for levels >= 1: wx, wy, wz, invd, e, f
    size_t total = 0;
    for (int l = 1; l < nl; ++l) total += 6 * (((size_t)H->lv[l].D.nc() + 63) & ~(size_t)63);
    cudaError_t err = cudaMalloc(&H->mem, std::max<size_t>(total, 1) * sizeof(float));
    if (err != cudaSuccess) {
        delete H;
        return cuda_fail(err, "cudaMalloc(mg levels)");
    }
    float* p = (float*)H->mem;
    for (int l = 1; l < nl; ++l) {
        const size_t n = (size_t)H->lv[l].D.nc();
        const size_t stride = (n + 63) & ~(size_t)63;
        MgLevel& L = H->lv[l];
        L.wx = p;
        L.wy = p + stride;
        L.wz = p + 2 * stride;
        L.invd = p + 3 * stride;
        L.e = p + 4 * stride;
        L.f = p + 5 * stride;
        p += 6 * stride;
    }
    ex->mg = H;
    // fluid components of the mask (host labelling, once per mask)
    {
        std::vector<uint8_t> hf((size_t)g->dims.nc());
        PG_CUDA(cudaMemcpy(hf.data(), g->flags, hf.size(), cudaMemcpyDeviceToHost));
        std::vector<i64> cells;
        std::vector<int> start;
        find_pockets(hf.data(), g->dims.nd, g->dims.d, g->dims.h, g->dims.w, 0, cells, start);
        int prc = upload_pockets(cells, start, &H->pockets);
        if (prc) return prc;
    }
    // coarse operators
    cudaStream_t s = g->stream;
    for (int l = 0; l + 1 < nl; ++l) {
        const LV v = view(*H, l);
        MgLevel& C = H->lv[l + 1];
        const i64 nc = C.D.nc();
        if (l == 0)
            PG_LAUNCH(KK_MG_SETUP, s,
                      k_mg_coarsen<true><<<blocks_for(g, nc), kMgThreads, 0, s>>>(v, C.wx, C.wy, C.wz, (int)C.D.d,
                                                                                (int)C.D.h, (int)C.D.w));
        else
            PG_LAUNCH(KK_MG_SETUP, s,
                      k_mg_coarsen<false><<<blocks_for(g, nc), kMgThreads, 0, s>>>(v, C.wx, C.wy, C.wz, (int)C.D.d,
                                                                                 (int)C.D.h, (int)C.D.w));
        const LV cv = view(*H, l + 1);
        PG_LAUNCH(KK_MG_SETUP, s, k_mg_invd<<<blocks_for(g, nc), kMgThreads, 0, s>>>(cv, C.invd));
    }
    PG_CHECK_LAUNCH();
    *out = H;
    return PG_OK;
}

// Launch one half-sweep over `color` at level l.
template <bool L0, int MODE, bool RZ>
static void smooth(pg_grid* g, const MgHierarchy& H, int l, float* e, const float* f, const float* ec, int color) {
    const LV v = view(H, l);
    const i64 n = (i64)v.d * v.h * ((v.w + 1) / 2);
    int cw = 1, ch = 1;
    if (l + 1 < H.nlev) {
        cw = (int)H.lv[l + 1].D.w;
        ch = (int)H.lv[l + 1].D.h;
    }
    cudaStream_t s = g->stream;
    PG_LAUNCH(l == 0 ? KK_MG_SMOOTH : KK_MG_SMOOTH_C, s,
              k_mg_smooth<L0, MODE, RZ><<<blocks_for(g, n), kMgThreads, 0, s>>>(v, e, f, ec, cw, ch, color,
                                                                                g->ws.state, g->ws.partials));
}

template <bool L0>
static void smooth_any(pg_grid* g, const MgHierarchy& H, int l, float* e, const float* f, const float* ec, int color,
                       int mode, bool rz) {
    if (mode == NB_FIRST) smooth<L0, NB_FIRST, false>(g, H, l, e, f, ec, color);
    else if (mode == NB_SELF) smooth<L0, NB_SELF, false>(g, H, l, e, f, ec, color);
    else if (mode == NB_PROLONG) smooth<L0, NB_PROLONG, false>(g, H, l, e, f, ec, color);
    else if (rz) smooth<L0, NB_PLAIN, true>(g, H, l, e, f, ec, color);
    else smooth<L0, NB_PLAIN, false>(g, H, l, e, f, ec, color);
}

static void smooth_lv(pg_grid* g, const MgHierarchy& H, int l, float* e, const float* f, const float* ec, int color,
                      int mode, bool rz = false) {
    if (l == 0) smooth_any<true>(g, H, l, e, f, ec, color, mode, rz);
    else smooth_any<false>(g, H, l, e, f, ec, color, mode, rz);
}

// Enqueue z = V(r) on the grid's stream.
static int vcycle(pg_grid* g, const MgHierarchy& H, const float* r, float* z, int nsmooth);

// z = P V(P r): P removes the mean of every fluid component when there are
// several (pg_pocket.cu); r is projected in place (the CG's recursive
// residual then measures the consistent part).
static int vcycle_projected(pg_grid* g, const MgHierarchy& H, float* r, float* z, int nsmooth) {
    pocket_project(g->stream, r, H.pockets);
    const int rc = vcycle(g, H, r, z, nsmooth);
    pocket_project(g->stream, z, H.pockets);
    return rc;
}

static int vcycle(pg_grid* g, const MgHierarchy& H, const float* r, float* z, int nsmooth) {
    cudaStream_t s = g->stream;
    const int nl = H.nlev;
    auto E = [&](int l) -> float* { return l == 0 ? z : H.lv[l].e; };
    auto F = [&](int l) -> const float* { return l == 0 ? r : H.lv[l].f; };
    if (nl == 1) {
        // A grid too small to coarsen: symmetric Gauss-Seidel sweeps only.
        smooth_lv(g, H, 0, z, r, nullptr, 1, NB_FIRST);
        for (int k = 1; k < 4 * nsmooth; ++k) {
            smooth_lv(g, H, 0, z, r, nullptr, 0, NB_PLAIN);
            smooth_lv(g, H, 0, z, r, nullptr, 1, NB_PLAIN);
        }
        for (int k = 0; k < 4 * nsmooth; ++k) {
            smooth_lv(g, H, 0, z, r, nullptr, 1, NB_PLAIN);
            smooth_lv(g, H, 0, z, r, nullptr, 0, NB_PLAIN, k == 4 * nsmooth - 1);
        }
        PG_CHECK_LAUNCH();
        return PG_OK;
    }
    // levels [0, top) run as per-level kernels; [top, nl) in the tail kernel
    // (or, without a tail, the coarsest level alone in k_mg_coarse)
    const bool tail = H.tail < nl;
    const int top = tail ? H.tail : nl - 1;
    // down
    for (int l = 0; l < top; ++l) {
        float* e = E(l);
        const float* f = F(l);
        // pre-smoothing: (red, black) x nsmooth from e = 0; the first red is implicit
        smooth_lv(g, H, l, e, f, nullptr, 1, NB_FIRST);
        if (nsmooth == 1) smooth_lv(g, H, l, e, f, nullptr, 0, NB_SELF);  // store the implicit red values
        for (int k = 1; k < nsmooth; ++k) {
            smooth_lv(g, H, l, e, f, nullptr, 0, NB_PLAIN);
            smooth_lv(g, H, l, e, f, nullptr, 1, NB_PLAIN);
        }
        const LV v = view(H, l);
        const MgLevel& C = H.lv[l + 1];
        const i64 nc = C.D.nc();
        if (l == 0)
            PG_LAUNCH(KK_MG_RESTRICT, s,
                      k_mg_restrict<true><<<blocks_for(g, nc), kMgThreads, 0, s>>>(v, e, f, C.f, (int)C.D.d,
                                                                                 (int)C.D.h, (int)C.D.w,
                                                                                 g->ws.state));
        else
            PG_LAUNCH(KK_MG_RESTRICT_C, s,
                      k_mg_restrict<false><<<blocks_for(g, nc), kMgThreads, 0, s>>>(v, e, f, C.f, (int)C.D.d,
                                                                                  (int)C.D.h, (int)C.D.w,
                                                                                  g->ws.state));
    }
    if (tail) {
        TailArgs A;
        A.lt = top;
        A.nl = nl;
        A.nsmooth = nsmooth;
        A.e_out = H.lv[top].e;
        A.f_in = H.lv[top].f;
        size_t smem = 0;
        for (int l = top; l < nl; ++l) {
            const MgLevel& L = H.lv[l];
            A.L[l] = TailLevel{L.D.nd, (int)L.D.d, (int)L.D.h, (int)L.D.w, L.wx, L.wy, L.wz, L.invd};
            smem += 6 * sizeof(float) * (size_t)L.D.nc();
        }
        static bool attr = false;
        if (!attr) {
            PG_CUDA(cudaFuncSetAttribute(k_mg_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmemMax));
            attr = true;
        }
        if (smem > (size_t)kTailSmemMax) return bad_arg("PG_PRECOND_MG: multigrid tail does not fit in shared memory");
        PG_LAUNCH(KK_MG_COARSE, s, k_mg_tail<<<1, kTailThreads, smem, s>>>(A, g->ws.state));
    } else {
        const LV v = view(H, nl - 1);
        PG_LAUNCH(KK_MG_COARSE, s,
                  k_mg_coarse<<<1, kCoarseThreads, 0, s>>>(v, H.lv[nl - 1].e, H.lv[nl - 1].f, g->ws.state));
    }
    // up
    for (int l = top - 1; l >= 0; --l) {
        float* e = E(l);
        const float* f = F(l);
        const float* ec = H.lv[l + 1].e;
        // post-smoothing: (black, red) x nsmooth; the first black reads the
        // prolonged red neighbours
        smooth_lv(g, H, l, e, f, ec, 1, NB_PROLONG);
        for (int k = 0; k < nsmooth; ++k) {
            if (k > 0) smooth_lv(g, H, l, e, f, nullptr, 1, NB_PLAIN);
            smooth_lv(g, H, l, e, f, nullptr, 0, NB_PLAIN, l == 0 && k == nsmooth - 1);
        }
    }
    PG_CHECK_LAUNCH();
    return PG_OK;
}

struct MgHook : ZHook {
    MgHierarchy* H;
    int nsmooth;
    int apply(pg_grid* g, const void* r, void* z) override {
        return vcycle_projected(g, *H, (float*)const_cast<void*>(r), (float*)z, nsmooth);
    }
    uintptr_t key() const override { return (uintptr_t)(H->id << 8) | (uintptr_t)(nsmooth & 0xff); }
};

template <class T>
int solve_mgpcg(pg_grid* g, const pg_solver_params* prm, const CgConfig& cfg, CgBuffers<T> buf, pg_pcg_stats* st) {
    if (sizeof(T) != 4) return bad_arg("PG_PRECOND_MG: float fields only");
    MgHierarchy* H = nullptr;
    int rc = ensure_mg(g, cfg.dt, &H);
    if (rc) return rc;
    Extras* ex = extras_of(g);
    void* z;
    if ((rc = ex->buffer(Extras::kZ, sizeof(float) * (size_t)g->dims.nc(), &z))) return rc;
    buf.z = (T*)z;
    MgHook hook;
    hook.H = H;
    hook.nsmooth = prm->mg_smooth > 0 ? prm->mg_smooth : 2;
    return run_cg<T>(g, cfg, buf, st, &hook);
}

template int solve_mgpcg<float>(pg_grid*, const pg_solver_params*, const CgConfig&, CgBuffers<float>, pg_pcg_stats*);
template int solve_mgpcg<double>(pg_grid*, const pg_solver_params*, const CgConfig&, CgBuffers<double>,
                                 pg_pcg_stats*);

}  // namespace pg
