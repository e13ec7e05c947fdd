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
#include <cmath>
#include <cstdlib>
#include <vector>

#include "pg_solve.cuh"
#include "pg_tma.cuh"

namespace pg {

constexpr int kMgThreads = 256;
constexpr int kCoarseMax = 2048;
constexpr int kCoarseThreads = 512;
constexpr int kMaxLevels = 16;
constexpr int kCinvCells = 64;  // coarsest levels up to this size are solved by a dense pseudo-inverse
constexpr int kRestrictPerChild = 65536;  // restrictions to at most this many cells: a thread per child
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
    float* cinv = nullptr;  // coarsest level of at most kCinvCells cells: its pseudo-inverse (row-major)
    int ct_lt = 0;    // cluster tail (3D): first level (0: not used), first rank-0 level, ranks
    int ct_ls = 0;
    int ct_ranks = 0;
    size_t ct_smem = 0;
    double nfluid = 0;  // cells with an open face (the lazy projection's count)
    // fine level of 3D grids: fused red-black pairs (k_mg_pair) ping-pong
    // between z and e0b; tensor maps of the flags and of the vectors met
    bool pairs = false;
    float* e0b = nullptr;
    CUtensorMap gmap;  // level-0 flags
    CUtensorMap cmap;  // level-1 correction (prolongation)
    CUtensorMap rgmap;  // level-0 flags, the restriction's tile box
    bool restrict_tma = false;  // fine restriction by k_mg_restrict3p (3D, even sides)
    int pair_cap = 0;          // resident k_mg_pair blocks on the device (every mode)
    // the pairs' plane loads carry the L2 evict-last policy: 4.074 -> 4.050
    // ms per 256^3 step (their halo re-reads still come from DRAM; the other
    // kernels' later reads of the same vectors hit more often); PG_MG_L2KEEP=0
    // drops the hint (a diagnostic switch read per build)
    bool l2keep = true;
    int pair_cap_plain = 0;    // the same for the modes without the coarse correction
    struct MapEnt {
        const void* p = nullptr;
        int bx = 0, by = 0;
        CUtensorMap m;
    };
    mutable MapEnt maps[8];
    mutable int next_map = 0;
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
                int color, CgState* st, double* partials, FastDiv fhalf, FastDiv fh) {
    if (st->done) return;
    __shared__ double sm[32];
    const int hw = v.h * v.w;
    const int half = (v.w + 1) >> 1;
    const int nrow = v.d * v.h;
    const int total = nrow * half;
    Acc<float> acc, zs;  // z.r and sum(z) (RZ)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        // the flat index split by invariant-divisor multiplication (the
        // coarse half-sweeps are issue-bound: two integer divisions were
        // a quarter of a cell's instructions)
        int k2, y;
        const int row = split(i, half, fhalf, k2);
        const int z = split(row, v.h, fh, y);
        const int x = 2 * k2 + ((y + z + color) & 1);
        if (!L0 && x < v.w) {
            // Coarse levels (weights in memory): every value the cell may
            // need is loaded before any is used -- a missing neighbour's
            // offset is clamped to the cell itself and its value ignored --
            // so the cell waits for one round of loads; the arithmetic is
            // the same as below.
            const int c = row * v.w + x;
            const bool d3 = v.nd == 3;
            const bool hx = x + 1 < v.w, hy = y + 1 < v.h, hz = d3 && z + 1 < v.d;
            const int ox0 = x > 0 ? -1 : 0, ox1 = hx ? 1 : 0, oy0 = y > 0 ? -v.w : 0, oy1 = hy ? v.w : 0;
            const int oz0 = d3 && z > 0 ? -hw : 0, oz1 = hz ? hw : 0;
            const float wxl = v.wx[c], wxh_ = v.wx[c + ox1], wyl = v.wy[c], wyh_ = v.wy[c + oy1];
            const float wzl = d3 ? v.wz[c] : 0.f, wzh_ = d3 ? v.wz[c + oz1] : 0.f;
            const float inv = v.invd[c];
            float s = f[c];
            if (MODE == NB_SELF) {
                e[c] = s * inv;
                continue;
            }
            const float n0 = nbval<L0, MODE>(v, e, f, ec, cw, ch, c + ox0, z, y, x + (x > 0 ? -1 : 0));
            const float n1 = nbval<L0, MODE>(v, e, f, ec, cw, ch, c + ox1, z, y, x + ox1);
            const float n2 = nbval<L0, MODE>(v, e, f, ec, cw, ch, c + oy0, z, y + (y > 0 ? -1 : 0), x);
            const float n3 = nbval<L0, MODE>(v, e, f, ec, cw, ch, c + oy1, z, y + (hy ? 1 : 0), x);
            const float n4 = nbval<L0, MODE>(v, e, f, ec, cw, ch, c + oz0, z + (oz0 ? -1 : 0), y, x);
            const float n5 = nbval<L0, MODE>(v, e, f, ec, cw, ch, c + oz1, z + (hz ? 1 : 0), y, x);
            const float wxh = hx ? wxh_ : 0.f, wyh = hy ? wyh_ : 0.f, wzh = hz ? wzh_ : 0.f;
            if (wxl != 0.f) s += wxl * n0;
            if (wxh != 0.f) s += wxh * n1;
            if (wyl != 0.f) s += wyl * n2;
            if (wyh != 0.f) s += wyh * n3;
            if (d3) {
                if (wzl != 0.f) s += wzl * n4;
                if (wzh != 0.f) s += wzh * n5;
            }
            const float en = s * inv;
            e[c] = en;
            if (RZ) {
                acc.add(en * f[c]);
                zs.add(en);
            }
        } else if (x < v.w) {
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
            if (RZ) {
                acc.add(en * f[c]);
                zs.add(en);
            }
        }
    }
    if (!RZ) return;
    // z.r: red cells here, black cells were final after the previous
    // half-sweep -- reduce both colours: the black part is added by the
    // companion pass below (same kernel, other colour read-only).
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        int k2, y;
        const int row = split(i, half, fhalf, k2);
        const int z = split(row, v.h, fh, y);
        const int x = 2 * k2 + ((y + z + color + 1) & 1);
        if (x < v.w) {
            const int c = row * v.w + x;
            acc.add(e[c] * f[c]);
            zs.add(e[c]);
        }
    }
    const double s = block_sum<kMgThreads>(acc.value(), sm);
    const double s2 = block_sum<kMgThreads>(zs.value(), sm);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = s;
        partials[kMaxBlocks + blockIdx.x] = s2;
    }
    if (!last_block(&st->counter[3])) return;
    const double rz = reduce_partials<false, kMgThreads>(partials, gridDim.x, sm);
    const double zsum = reduce_partials<false, kMgThreads>(partials + kMaxBlocks, gridDim.x, sm);
    if (threadIdx.x == 0) {
        st->counter[3] = 0;
        cg_finish_rz(st, rz, zsum);
    }
}

// ---------------------------------------------------------------------------
// Fused red-black pair on the fine level of 3D grids.
//
// One launch performs a half-sweep over colour c1 and the following
// half-sweep over the other colour c2, reading the correction from `ein`
// and writing both colours to `eout` (out of place: a neighbouring tile's
// first half-sweep still needs the old c2 values this tile replaces).  A
// block owns a kPX x kPY column tile and walks a chunk of z planes.  TMA
// stages every plane of ein (2-cell halo), f and the face flags (1-cell
// halo) into a kPStages-deep shared-memory ring; for plane p the block
// computes the new c1 values on the tile plus its one-cell ring (the ring
// cells belong to the neighbouring tiles, which compute the same values)
// into a shared slot, then the c2 values of plane p-1 from the c1 slots of
// planes p-2, p-1 and p, and stores both colours of plane p-1 as one float2
// per thread.  Per cell: 4 bytes of ein, 4 of f and 1 of flags read, 4 of
// eout written -- half the traffic of two separate half-sweeps.  The
// arithmetic of every cell is that of k_mg_smooth<true, ...>.
constexpr int kPX = 64;
constexpr int kPWarps = 8, kPRows = 2;  // warps per block, tile rows per thread
constexpr int kPY = kPWarps * kPRows;
constexpr int kPThreads = 32 * kPWarps;  // one (c1, c2) x-pair per thread, row and plane
constexpr int kPMinBlocks = 2;           // resident blocks per SM the registers are sized for
constexpr int kPStages = 6;              // plane ring; loads run kPStages - 3 planes ahead
constexpr int kPEw = kPX + 8, kPEh = kPY + 4;    // ein box from (x0 - 4, y0 - 2)
constexpr int kPFw = kPX + 8, kPFh = kPY + 2;    // f box from (x0 - 4, y0 - 1)
constexpr int kPGw = kPX + 32, kPGh = kPY + 2;   // flags box from (x0 - 16, y0 - 1)
constexpr int kPEBytes = kPEw * kPEh * 4;        // 3456
constexpr int kPFBytes = kPFw * kPFh * 4;        // 2880
constexpr int kPGBytes = kPGw * kPGh;            // 960
constexpr int kPCw = kPX / 2 + 8, kPCh = kPY / 2 + 2;  // coarse-correction box from (x0/2 - 4, y0/2 - 1)
constexpr int kPCBytes = kPCw * kPCh * 4;        // 960
constexpr int kPFOff = kPEBytes;                 // every box starts on 128 bytes
constexpr int kPGOff = kPFOff + ((kPFBytes + 127) / 128) * 128;
constexpr int kPCOff = kPGOff + ((kPGBytes + 127) / 128) * 128;
constexpr int kPSw = kPX + 2, kPSh = kPY + 2;    // new c1 values of one plane (tile + ring)
constexpr int kPSlotBytes = kPSw * kPSh * 4;

enum { PR_SELF = 0 /* c1 = f * invd (e = 0 before) */, PR_PLAIN = 1, PR_PROLONG = 2 /* ein + ec[parent] */ };

// Shared-memory layout per first-sweep mode: the prolonging pair also
// stages the coarse correction's parent plane and runs one stage fewer
// (kPMinBlocks blocks stay resident per SM).
template <int M1> struct PairCfg {
    static constexpr bool kCoarse = M1 == PR_PROLONG;
    static constexpr int kStages = kCoarse ? 5 : kPStages;
    static constexpr int kStageBytes = kPCOff + (kCoarse ? ((kPCBytes + 127) / 128) * 128 : 0);
    static constexpr int kBarOff = kStages * kStageBytes + 4 * kPSlotBytes;
    static constexpr size_t kSmem = 128 + kBarOff + kStages * 8;
    static constexpr unsigned kTx = (M1 == PR_SELF ? 0 : kPEBytes) + kPFBytes + kPGBytes + (kCoarse ? kPCBytes : 0);
    static_assert(kStageBytes % 128 == 0 && kPEBytes % 128 == 0, "TMA boxes must stay 128-byte aligned");
};

struct PairArgs {
    int d, h, w;
    float dt;
    float* eout;
    int c1;  // colour of the first half-sweep
    int tiles_x, tiles_y;
    int l2keep;  // plane loads with the L2 evict-last policy
};

template <int M1, bool RZ>
__global__ void __launch_bounds__(kPThreads, kPMinBlocks)
    k_mg_pair(const __grid_constant__ CUtensorMap emap, const __grid_constant__ CUtensorMap fmap,
              const __grid_constant__ CUtensorMap gmap, const __grid_constant__ CUtensorMap cmap, PairArgs a,
              CgState* st, double* partials) {
    typedef PairCfg<M1> Cfg;
    constexpr int kStages = Cfg::kStages, kStageBytes = Cfg::kStageBytes;
    if (st->done) return;
    extern __shared__ unsigned char pair_smem_raw[];
    __shared__ double sm[32];
    __shared__ float inv_tab[8];  // 1 / (n dt) for n open faces (0 for n = 0), as Cell<true>
    // 128-byte aligned by an offset (pointer arithmetic keeps every access
    // below in the shared window: LDS/STS, not generic loads)
    unsigned char* const base = pair_smem_raw + ((128u - (smem_u32(pair_smem_raw) & 127u)) & 127u);
    float(*const S1)[kPSh][kPSw] = (float(*)[kPSh][kPSw])(base + kStages * kStageBytes);
    uint64_t* const bars = (uint64_t*)(base + Cfg::kBarOff);
    const int tid = threadIdx.x, lane = tid & 31, ty = tid >> 5;
    const float dt = a.dt;
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
        mbar_fence_init();
        if (M1 != PR_SELF) tma_prefetch_map(&emap);
        if (Cfg::kCoarse) tma_prefetch_map(&cmap);
        tma_prefetch_map(&fmap);
        tma_prefetch_map(&gmap);
    }
    if (tid < 8) inv_tab[tid] = tid ? __frcp_rn((float)tid * dt) : 0.f;
    __syncthreads();
    const int h = a.h, w = a.w, d = a.d;
    const int per_plane = a.tiles_x * a.tiles_y;
    auto stage = [&](unsigned j) -> const unsigned char* { return base + (j % kStages) * kStageBytes; };
    auto Ev = [](const unsigned char* P, int r, int c) -> float { return ((const float*)P)[r * kPEw + c]; };
    auto Fv = [](const unsigned char* P, int r, int c) -> float {
        return ((const float*)(P + kPFOff))[r * kPFw + c];
    };
    auto Gv = [](const unsigned char* P, int r, int c) -> unsigned { return (P + kPGOff)[r * kPGw + c]; };
    // coarse correction at the parent of tile cell (yl, xl) of the staged plane
    auto Cv = [](const unsigned char* P, int yl, int xl) -> float {
        return ((const float*)(P + kPCOff))[((yl >> 1) + 1) * kPCw + (xl >> 1) + 4];
    };
    unsigned issued_end = 0;  // thread 0: one past the last plane issued
    const uint64_t keep = l2_evict_last();
    auto issue = [&](unsigned j, int plane, int x0, int y0) {
        issued_end = j + 1;
        unsigned char* dst = base + (j % kStages) * kStageBytes;
        uint64_t* bar = &bars[j % kStages];
        mbar_expect_tx(bar, Cfg::kTx);
        if (a.l2keep) {
            if (M1 != PR_SELF) tma_load_3d_hint(dst, &emap, bar, x0 - 4, y0 - 2, plane, keep);
            tma_load_3d_hint(dst + kPFOff, &fmap, bar, x0 - 4, y0 - 1, plane, keep);
            tma_load_3d_hint(dst + kPGOff, &gmap, bar, x0 - 16, y0 - 1, plane, keep);
        } else {
            if (M1 != PR_SELF) tma_load_3d(dst, &emap, bar, x0 - 4, y0 - 2, plane);
            tma_load_3d(dst + kPFOff, &fmap, bar, x0 - 4, y0 - 1, plane);
            tma_load_3d(dst + kPGOff, &gmap, bar, x0 - 16, y0 - 1, plane);
        }
        if (Cfg::kCoarse) tma_load_3d(dst + kPCOff, &cmap, bar, x0 / 2 - 4, y0 / 2 - 1, plane >> 1);
    };
    // Thread 0 alone polls the barriers; the __syncthreads that follows its
    // wait publishes the staged plane to the block.
    bool ok = true;
    auto wait = [&](unsigned j) {
        if (tid == 0 && ok) ok = mbar_wait(&bars[j % kStages], (j / kStages) & 1);
    };
    // Gauss-Seidel update from the open-face neighbour values (same
    // operation order as k_mg_smooth<true, ...>; the loads are unconditional,
    // every staged value is finite).
    auto gs = [&](unsigned fl, float fv, float vxl, float vxh, float vyl, float vyh, float vzl, float vzh) -> float {
        float s = fv;
        s = (fl & XLO) ? fmaf(dt, vxl, s) : s;
        s = (fl & XHI) ? fmaf(dt, vxh, s) : s;
        s = (fl & YLO) ? fmaf(dt, vyl, s) : s;
        s = (fl & YHI) ? fmaf(dt, vyh, s) : s;
        s = (fl & ZLO) ? fmaf(dt, vzl, s) : s;
        s = (fl & ZHI) ? fmaf(dt, vzh, s) : s;
        return s * inv_tab[__popc(fl)];
    };
    unsigned seq = 0;     // planes this block has consumed: ring slot and phase parity
    bool failed = false;  // block-uniform: a wait gave up
    Acc<float> acc, zs;   // z.r and sum(z) (RZ)
    ZWalk walk(per_plane, d);
    int t2, z0, z1;
    while (!failed && walk.next(t2, z0, z1)) {
        const int x0 = (t2 % a.tiles_x) * kPX, y0 = (t2 / a.tiles_x) * kPY;
        const int n = z1 - z0 + 4;  // planes z0 - 2 .. z1 + 1 (ring index j = plane - z0 + 2)
        if (tid == 0)
            for (int j = 0; j < min(n, kStages); ++j) issue(seq + j, z0 - 2 + j, x0, y0);
        wait(seq);
        wait(seq + 1);
        wait(seq + 2);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        for (int i = 0; i <= z1 - z0 + 1; ++i) {
            const int p = z0 - 1 + i;  // plane of this step's first half-sweep
            const unsigned char *Pm = stage(seq + i), *P0 = stage(seq + i + 1), *Pp = stage(seq + i + 2);
            // new c1 value of cell (yl, xl) of plane p, tile coordinates
            auto c1_cell = [&](int yl, int xl) -> float {
                const unsigned fl = Gv(P0, yl + 1, xl + 16);
                const float fv = Fv(P0, yl + 1, xl + 4);
                if (M1 == PR_SELF) return fv * inv_tab[__popc(fl)];
                if (M1 == PR_PROLONG)  // neighbours plus their parents' coarse correction
                    return gs(fl, fv, Ev(P0, yl + 2, xl + 3) + Cv(P0, yl, xl - 1),
                              Ev(P0, yl + 2, xl + 5) + Cv(P0, yl, xl + 1), Ev(P0, yl + 1, xl + 4) + Cv(P0, yl - 1, xl),
                              Ev(P0, yl + 3, xl + 4) + Cv(P0, yl + 1, xl), Ev(Pm, yl + 2, xl + 4) + Cv(Pm, yl, xl),
                              Ev(Pp, yl + 2, xl + 4) + Cv(Pp, yl, xl));
                return gs(fl, fv, Ev(P0, yl + 2, xl + 3), Ev(P0, yl + 2, xl + 5), Ev(P0, yl + 1, xl + 4),
                          Ev(P0, yl + 3, xl + 4), Ev(Pm, yl + 2, xl + 4), Ev(Pp, yl + 2, xl + 4));
            };
#pragma unroll
            for (int r = 0; r < kPRows; ++r) {
                const int yl = ty + r * kPWarps;
                const int xl = 2 * lane + ((a.c1 + y0 + yl + p) & 1);
                S1[p & 3][yl + 1][xl + 1] = c1_cell(yl, xl);
            }
            if (tid < 64) {  // ring rows y0 - 1 and y0 + kPY
                const int yl = tid < 32 ? -1 : kPY;
                const int xl = 2 * lane + ((a.c1 + y0 + yl + p) & 1);
                S1[p & 3][yl + 1][xl + 1] = c1_cell(yl, xl);
            } else if (tid < 64 + 2 * kPY) {  // ring columns x0 - 1 and x0 + kPX
                const int k = tid - 64;
                const int xl = k < kPY ? -1 : kPX, yl = k < kPY ? k : k - kPY;
                if (((x0 + xl + y0 + yl + p) & 1) == a.c1) S1[p & 3][yl + 1][xl + 1] = c1_cell(yl, xl);
            }
            // the next step's plane p + 2 must have landed
            if (seq + i + 3 < seq + n) wait(seq + i + 3);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            // the ring slot of plane p - 2 is free now: load kPStages planes past it
            if (tid == 0 && i >= 1 && i - 1 + kStages < n) issue(seq + i - 1 + kStages, z0 - 3 + i + kStages, x0, y0);
            if (i >= 2) {  // second half-sweep on plane q = p - 1, then store it
                const int q = p - 1;
#pragma unroll
                for (int r = 0; r < kPRows; ++r) {
                    const int yl = ty + r * kPWarps, gy = y0 + yl;
                    const int xl2 = 2 * lane + ((a.c1 + 1 + gy + q) & 1), xl1 = xl2 ^ 1;
                    const float e1 = S1[q & 3][yl + 1][xl1 + 1];
                    const float fv = Fv(Pm, yl + 1, xl2 + 4);
                    const float e2 =
                        gs(Gv(Pm, yl + 1, xl2 + 16), fv, S1[q & 3][yl + 1][xl2], S1[q & 3][yl + 1][xl2 + 2],
                           S1[q & 3][yl][xl2 + 1], S1[q & 3][yl + 2][xl2 + 1], S1[(q - 1) & 3][yl + 1][xl2 + 1],
                           S1[(q + 1) & 3][yl + 1][xl2 + 1]);
                    const int x = x0 + 2 * lane;
                    if (gy < h && x < w) {
                        const float2 v = (xl1 & 1) ? make_float2(e2, e1) : make_float2(e1, e2);
                        *(float2*)(a.eout + ((i64)q * h + gy) * w + x) = v;
                        if (RZ) {
                            acc.add(e1 * Fv(Pm, yl + 1, xl1 + 4));
                            acc.add(e2 * fv);
                            zs.add(e1);
                            zs.add(e2);
                        }
                    }
                }
            }
        }
        if (failed) break;
        __syncthreads();  // every thread is done with the ring before the next item's loads
        seq += n;
    }
    if (failed) {  // a plane never arrived: drain the copies in flight (bounded), stop the solve
        if (tid == 0) {
            const uint64_t t0 = global_ns();
            for (unsigned j = issued_end > kStages ? issued_end - kStages : 0; j < issued_end; ++j)
                while (!mbar_try_wait(&bars[j % kStages], (j / kStages) & 1) && global_ns() - t0 < kMbarWaitNs) {
                }
            st->status = PG_TIMEOUT;
            st->done = 1;
        }
        return;
    }
    if (RZ) {
        const double s = block_sum<kPThreads>(acc.value(), sm);
        const double s2 = block_sum<kPThreads>(zs.value(), sm);
        if (threadIdx.x == 0) {
            partials[blockIdx.x] = s;
            partials[kMaxBlocks + blockIdx.x] = s2;
        }
        if (last_block(&st->counter[3])) {
            const double rz = reduce_partials<false, kPThreads>(partials, gridDim.x, sm);
            const double zsum = reduce_partials<false, kPThreads>(partials + kMaxBlocks, gridDim.x, sm);
            if (threadIdx.x == 0) {
                st->counter[3] = 0;
                cg_finish_rz(st, rz, zsum);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Fine-level restriction of 3D grids with even sides, TMA-staged: a block
// owns a kQX x kQY tile of fine cells (kQX/2 x kQY/2 coarse cells, one per
// thread) and walks a range of coarse planes (ZWalk over the coarse tile
// columns); fine plane p is staged with e (one-cell halo), f and the flags
// into a kQStages-deep ring, and coarse plane Z reads the stages of fine
// planes 2Z-1 .. 2Z+2.  Each thread sums its eight children's residuals
// f - A e in the order and with the arithmetic of k_mg_restrict8<true>
// (bit-identical).  Per fine cell: 4 bytes of e (+ halo), 4 of f, 1 of flags
// in; 0.5 of the coarse right-hand side out.
constexpr int kQX = 64, kQY = 16, kQThreads = (kQX / 2) * (kQY / 2);
constexpr int kQStages = 6;
constexpr int kQEw = kQX + 8, kQEh = kQY + 2;  // e box from (x0 - 4, y0 - 1)
constexpr int kQEBytes = kQEw * kQEh * 4, kQFBytes = kQX * kQY * 4, kQGBytes = kQX * kQY;
constexpr int kQFOff = ((kQEBytes + 127) / 128) * 128, kQGOff = kQFOff + kQFBytes;
constexpr int kQStageBytes = kQGOff + ((kQGBytes + 127) / 128) * 128;
constexpr int kQBarOff = kQStages * kQStageBytes;
constexpr size_t kQSmem = 128 + kQBarOff + kQStages * 8;
constexpr unsigned kQTx = kQEBytes + kQFBytes + kQGBytes;
static_assert(kQStageBytes % 128 == 0 && kQFOff % 128 == 0 && kQGOff % 128 == 0, "TMA boxes 128-byte aligned");

struct RestrictArgs {
    int d, h, w;  // fine
    int ch, cw;   // coarse rows and columns
    float dt;
    float* fc;
    int tiles_x, tiles_y;
};

__global__ void __launch_bounds__(kQThreads)
    k_mg_restrict3p(const __grid_constant__ CUtensorMap emap, const __grid_constant__ CUtensorMap fmap,
                    const __grid_constant__ CUtensorMap gmap, RestrictArgs a, CgState* st) {
    if (st->done) return;
    extern __shared__ unsigned char rs_smem_raw[];
    unsigned char* const base = rs_smem_raw + ((128u - (smem_u32(rs_smem_raw) & 127u)) & 127u);
    uint64_t* const bars = (uint64_t*)(base + kQBarOff);
    const int tid = threadIdx.x, cx = tid % (kQX / 2), cy = tid / (kQX / 2);
    if (tid == 0) {
        for (int s = 0; s < kQStages; ++s) mbar_init(&bars[s], 1);
        mbar_fence_init();
        tma_prefetch_map(&emap);
        tma_prefetch_map(&fmap);
        tma_prefetch_map(&gmap);
    }
    __syncthreads();
    const float dt = a.dt;
    const int d = a.d;
    auto stage = [&](unsigned j) -> const unsigned char* { return base + (j % kQStages) * kQStageBytes; };
    unsigned issued_end = 0;
    auto issue = [&](unsigned j, int plane, int x0, int y0) {
        issued_end = j + 1;
        unsigned char* dst = base + (j % kQStages) * kQStageBytes;
        uint64_t* bar = &bars[j % kQStages];
        mbar_expect_tx(bar, kQTx);
        tma_load_3d(dst, &emap, bar, x0 - 4, y0 - 1, plane);
        tma_load_3d(dst + kQFOff, &fmap, bar, x0, y0, plane);
        tma_load_3d(dst + kQGOff, &gmap, bar, x0, y0, plane);
    };
    bool ok = true;
    auto wait = [&](unsigned j) {
        if (tid == 0 && ok) ok = mbar_wait(&bars[j % kQStages], (j / kQStages) & 1);
    };
    unsigned seq = 0;
    bool failed = false;
    const int cd = d / 2;
    ZWalk walk(a.tiles_x * a.tiles_y, cd);
    int t2, Z0, Z1;
    while (!failed && walk.next(t2, Z0, Z1)) {
        const int x0 = (t2 % a.tiles_x) * kQX, y0 = (t2 / a.tiles_x) * kQY;
        const int n = 2 * (Z1 - Z0) + 2;  // fine planes 2 Z0 - 1 .. 2 Z1 (ring index j = plane - 2 Z0 + 1)
        if (tid == 0)
            for (int j = 0; j < min(n, kQStages); ++j) issue(seq + j, 2 * Z0 - 1 + j, x0, y0);
        for (int i = 0; i < Z1 - Z0; ++i) {
            // coarse plane Z0 + i reads ring entries 2i .. 2i + 3
            if (i == 0) {
                wait(seq);
                wait(seq + 1);
            }
            wait(seq + 2 * i + 2);
            wait(seq + 2 * i + 3);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            float sum = 0.f;
#pragma unroll
            for (int dz = 0; dz < 2; ++dz) {
                const unsigned char *Pm = stage(seq + 2 * i + dz), *P0 = stage(seq + 2 * i + dz + 1),
                                    *Pp = stage(seq + 2 * i + dz + 2);
                const float* E0 = (const float*)P0;
                const float* Em = (const float*)Pm;
                const float* Ep = (const float*)Pp;
                const float* F0 = (const float*)(P0 + kQFOff);
                const unsigned char* G0 = P0 + kQGOff;
#pragma unroll
                for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                    for (int dx = 0; dx < 2; ++dx) {
                        const int yl = 2 * cy + dy, xl = 2 * cx + dx;
                        const int ei = (yl + 1) * kQEw + xl + 4;
                        const unsigned fl = G0[yl * kQX + xl];
                        const float ecv = E0[ei];
                        float acc = 0.f;
                        if (fl & XLO) acc = fmaf(dt, ecv - E0[ei - 1], acc);
                        if (fl & XHI) acc = fmaf(dt, ecv - E0[ei + 1], acc);
                        if (fl & YLO) acc = fmaf(dt, ecv - E0[ei - kQEw], acc);
                        if (fl & YHI) acc = fmaf(dt, ecv - E0[ei + kQEw], acc);
                        if (fl & ZLO) acc = fmaf(dt, ecv - Em[ei], acc);
                        if (fl & ZHI) acc = fmaf(dt, ecv - Ep[ei], acc);
                        sum += F0[yl * kQX + xl] - acc;
                    }
            }
            const int X = x0 / 2 + cx, Y = y0 / 2 + cy;
            if (X < a.cw && Y < a.ch) a.fc[((i64)(Z0 + i) * a.ch + Y) * a.cw + X] = sum;
            __syncthreads();  // ring entries 2i, 2i + 1 are free: refill them
            if (tid == 0) {
                if (2 * i + kQStages < n) issue(seq + 2 * i + kQStages, 2 * Z0 - 1 + 2 * i + kQStages, x0, y0);
                if (2 * i + 1 + kQStages < n) issue(seq + 2 * i + 1 + kQStages, 2 * Z0 + 2 * i + kQStages, x0, y0);
            }
        }
        if (failed) break;
        __syncthreads();
        seq += n;
    }
    if (failed) {  // a plane never arrived: drain the copies in flight (bounded), stop the solve
        if (tid == 0) {
            const uint64_t t0 = global_ns();
            for (unsigned j = issued_end > kQStages ? issued_end - kQStages : 0; j < issued_end; ++j)
                while (!mbar_try_wait(&bars[j % kQStages], (j / kQStages) & 1) && global_ns() - t0 < kMbarWaitNs) {
                }
            st->status = PG_TIMEOUT;
            st->done = 1;
        }
    }
}

static int restrict_cap(const pg_grid* g) {
    static int cap = -1;
    if (cap < 0) {
        cap = 0;
        if (cudaFuncSetAttribute(k_mg_restrict3p, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kQSmem) ==
            cudaSuccess) {
            int bps = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_mg_restrict3p, kQThreads, kQSmem) ==
                cudaSuccess)
                cap = std::min(bps * g->num_sms, kMaxBlocks);
        }
        cudaGetLastError();
    }
    return cap;
}

// Child residual f - A e of cell (z, y, x) of level v, with every neighbour
// value loaded at once (offsets of missing neighbours clamped to the cell,
// their values ignored).
template <bool L0>
__device__ __forceinline__ float child_residual(const LV& v, const float* __restrict__ e, const float* __restrict__ f,
                                                int z, int y, int x) {
    const int hw = v.h * v.w;
    const int c = (z * v.h + y) * v.w + x;
    const Cell<L0> cl(v, c, z, y, x);
    const bool d3 = v.nd == 3;
    const int ox0 = x > 0 ? -1 : 0, ox1 = x + 1 < v.w ? 1 : 0;
    const int oy0 = y > 0 ? -v.w : 0, oy1 = y + 1 < v.h ? v.w : 0;
    const int oz0 = d3 && z > 0 ? -hw : 0, oz1 = d3 && z + 1 < v.d ? hw : 0;
    const float ecv = e[c], e0 = e[c + ox0], e1 = e[c + ox1], e2 = e[c + oy0], e3 = e[c + oy1], e4 = e[c + oz0],
                e5 = e[c + oz1];
    float a = 0.f;
    if (cl.wxl != 0.f) a += cl.wxl * (ecv - e0);
    if (cl.wxh != 0.f) a += cl.wxh * (ecv - e1);
    if (cl.wyl != 0.f) a += cl.wyl * (ecv - e2);
    if (cl.wyh != 0.f) a += cl.wyh * (ecv - e3);
    if (d3) {
        if (cl.wzl != 0.f) a += cl.wzl * (ecv - e4);
        if (cl.wzh != 0.f) a += cl.wzh * (ecv - e5);
    }
    return f[c] - a;
}

// Residual of level l restricted (summed over children in (z, y, x) order)
// to level l+1, one thread per coarse cell (levels with many coarse cells).
template <bool L0>
__global__ void __launch_bounds__(kMgThreads)
    k_mg_restrict(LV v, const float* __restrict__ e, const float* __restrict__ f, float* __restrict__ fc, int cd,
                  int ch, int cw, CgState* st, FastDiv fcw, FastDiv fch) {
    if (st->done) return;
    const int nc = cd * ch * cw;
    for (int C = blockIdx.x * blockDim.x + threadIdx.x; C < nc; C += gridDim.x * blockDim.x) {
        int X, Y;
        const int CZY = split(C, cw, fcw, X);
        const int Z = split(CZY, ch, fch, Y);
        float sum = 0.f;
        const int z1 = v.nd == 3 ? min(2 * Z + 2, v.d) : 1;
        const int y1 = min(2 * Y + 2, v.h), x1 = min(2 * X + 2, v.w);
        for (int z = (v.nd == 3 ? 2 * Z : 0); z < z1; ++z)
            for (int y = 2 * Y; y < y1; ++y)
                for (int x = 2 * X; x < x1; ++x) sum += child_residual<L0>(v, e, f, z, y, x);
        fc[C] = sum;
    }
}

// The same, one thread per child (levels with few coarse cells): eight lanes
// of a warp form the eight child residuals of one coarse cell (those that
// exist), and the first of them sums them in (z, y, x) order.
template <bool L0>
__global__ void __launch_bounds__(kMgThreads)
    k_mg_restrict8(LV v, const float* __restrict__ e, const float* __restrict__ f, float* __restrict__ fc, int cd,
                   int ch, int cw, CgState* st, FastDiv fcw, FastDiv fch) {
    if (st->done) return;
    const int nc = cd * ch * cw;
    const unsigned lane = threadIdx.x & 31, grp = lane & ~7u;
    // every lane of a warp runs the same number of trips (shuffles below)
    const int n8 = (nc * 8 + 31) & ~31;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n8; t += gridDim.x * blockDim.x) {
        const int C = t >> 3, j = t & 7;
        float term = 0.f;
        bool has = false;
        if (C < nc) {
            int X, Y;
            const int CZY = split(C, cw, fcw, X);
            const int Z = split(CZY, ch, fch, Y);
            const int z = (v.nd == 3 ? 2 * Z : 0) + (j >> 2), y = 2 * Y + ((j >> 1) & 1), x = 2 * X + (j & 1);
            const int z1 = v.nd == 3 ? min(2 * Z + 2, v.d) : 1;
            if (z < z1 && y < v.h && x < v.w) {
                term = child_residual<L0>(v, e, f, z, y, x);
                has = true;
            }
        }
        const unsigned valid = __ballot_sync(0xffffffffu, has);
        float sum = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float tk = __shfl_sync(0xffffffffu, term, grp + k);
            if ((valid >> (grp + k)) & 1u) sum += tk;
        }
        if (j == 0 && C < nc) fc[C] = sum;
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
    const float* cinv;  // the coarsest level's pseudo-inverse, or null
    TailLevel L[kMaxLevels];
};

// One half-sweep by the whole block, or (WARP) by warp 0 alone.
// Every value a cell may need is loaded before any is used (a missing
// neighbour's offset is clamped to the cell itself and its value ignored),
// so a cell waits for one round of shared-memory loads; the arithmetic is
// that of k_mg_smooth.
template <int MODE, bool WARP = false>
__device__ __forceinline__ void tail_smooth(const LV& v, float* e, const float* f, const float* ec, int cw, int ch,
                                            int color) {
    const int hw = v.h * v.w, half = (v.w + 1) >> 1, total = v.d * v.h * half;
    const int t0 = WARP ? (int)(threadIdx.x & 31) : (int)threadIdx.x, dt = WARP ? 32 : (int)blockDim.x;
    const bool d3 = v.nd == 3;
    for (int i = t0; i < total; i += dt) {
        const int row = i / half, k2 = i - row * half;
        const int z = row / v.h, y = row - z * v.h;
        const int x = 2 * k2 + ((y + z + color) & 1);
        if (x >= v.w) continue;
        const int c = row * v.w + x;
        const bool hx = x + 1 < v.w, hy = y + 1 < v.h, hz = d3 && z + 1 < v.d;
        const int ox0 = x > 0 ? -1 : 0, ox1 = hx ? 1 : 0, oy0 = y > 0 ? -v.w : 0, oy1 = hy ? v.w : 0;
        const int oz0 = d3 && z > 0 ? -hw : 0, oz1 = hz ? hw : 0;
        const float wxl = v.wx[c], wxh_ = v.wx[c + ox1], wyl = v.wy[c], wyh_ = v.wy[c + oy1];
        const float wzl = d3 ? v.wz[c] : 0.f, wzh_ = v.wz[c + oz1];
        const float inv = v.invd[c];
        float s = f[c];
        if (MODE == NB_SELF) {
            e[c] = s * inv;
            continue;
        }
        const float n0 = nbval<false, MODE>(v, e, f, ec, cw, ch, c + ox0, z, y, x + (x > 0 ? -1 : 0));
        const float n1 = nbval<false, MODE>(v, e, f, ec, cw, ch, c + ox1, z, y, x + ox1);
        const float n2 = nbval<false, MODE>(v, e, f, ec, cw, ch, c + oy0, z, y + (y > 0 ? -1 : 0), x);
        const float n3 = nbval<false, MODE>(v, e, f, ec, cw, ch, c + oy1, z, y + (hy ? 1 : 0), x);
        const float n4 = nbval<false, MODE>(v, e, f, ec, cw, ch, c + oz0, z + (oz0 ? -1 : 0), y, x);
        const float n5 = nbval<false, MODE>(v, e, f, ec, cw, ch, c + oz1, z + (hz ? 1 : 0), y, x);
        const float wxh = hx ? wxh_ : 0.f, wyh = hy ? wyh_ : 0.f, wzh = hz ? wzh_ : 0.f;
        if (wxl != 0.f) s += wxl * n0;
        if (wxh != 0.f) s += wxh * n1;
        if (wyl != 0.f) s += wyl * n2;
        if (wyh != 0.f) s += wyh * n3;
        if (d3) {
            if (wzl != 0.f) s += wzl * n4;
            if (wzh != 0.f) s += wzh * n5;
        }
        e[c] = s * inv;
    }
    if (WARP)
        __syncwarp();
    else
        __syncthreads();
}

// The restriction of k_mg_restrict8 inside one block: one thread per child,
// eight lanes per coarse cell, summed by the first in (z, y, x) order.
__device__ __forceinline__ void tail_restrict(const LV& v, const float* e, const float* f, float* fc, int cd, int ch,
                                              int cw) {
    const int hw = v.h * v.w, nc = cd * ch * cw;
    const bool d3 = v.nd == 3;
    const unsigned lane = threadIdx.x & 31, grp = lane & ~7u;
    const int n8 = (nc * 8 + 31) & ~31;  // whole warps: every lane runs the same trips
    for (int t = threadIdx.x; t < n8; t += blockDim.x) {
        const int C = t >> 3, j = t & 7;
        const int CZY = C / cw, X = C - CZY * cw;
        const int Z = CZY / ch, Y = CZY - Z * ch;
        const int z = (d3 ? 2 * Z : 0) + (j >> 2), y = 2 * Y + ((j >> 1) & 1), x = 2 * X + (j & 1);
        const bool has = C < nc && z < (d3 ? v.d : 1) && y < v.h && x < v.w;
        float term = 0.f;
        if (has) {
            const int c = (z * v.h + y) * v.w + x;
            const bool hx = x + 1 < v.w, hy = y + 1 < v.h, hz = d3 && z + 1 < v.d;
            const int ox0 = x > 0 ? -1 : 0, ox1 = hx ? 1 : 0, oy0 = y > 0 ? -v.w : 0, oy1 = hy ? v.w : 0;
            const int oz0 = d3 && z > 0 ? -hw : 0, oz1 = hz ? hw : 0;
            const float wxl = v.wx[c], wxh_ = v.wx[c + ox1], wyl = v.wy[c], wyh_ = v.wy[c + oy1];
            const float wzl = d3 ? v.wz[c] : 0.f, wzh_ = v.wz[c + oz1];
            const float ecv = e[c], e0 = e[c + ox0], e1 = e[c + ox1], e2 = e[c + oy0], e3 = e[c + oy1],
                        e4 = e[c + oz0], e5 = e[c + oz1], fv = f[c];
            const float wxh = hx ? wxh_ : 0.f, wyh = hy ? wyh_ : 0.f, wzh = hz ? wzh_ : 0.f;
            float a = 0.f;
            if (wxl != 0.f) a += wxl * (ecv - e0);
            if (wxh != 0.f) a += wxh * (ecv - e1);
            if (wyl != 0.f) a += wyl * (ecv - e2);
            if (wyh != 0.f) a += wyh * (ecv - e3);
            if (d3) {
                if (wzl != 0.f) a += wzl * (ecv - e4);
                if (wzh != 0.f) a += wzh * (ecv - e5);
            }
            term = fv - a;
        }
        const unsigned valid = __ballot_sync(0xffffffffu, has);
        float sum = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float tk = __shfl_sync(0xffffffffu, term, grp + k);
            if ((valid >> (grp + k)) & 1u) sum += tk;
        }
        if (j == 0 && C < nc) fc[C] = sum;
    }
    __syncthreads();
}

// Coarsest level: symmetric red-black Gauss-Seidel from e = 0 (`pairs`
// (red, black) sweeps, then `pairs` (black, red)); a level of at most 256
// cells is swept by warp 0 alone, with warp barriers.
__device__ __forceinline__ void tail_coarsest(const LV& cv, float* e, const float* f, const float* cinv) {
    const int n = cv.d * cv.h * cv.w;
    if (cinv) {
        // e = pinv(A) f: 16 lanes per row, each summing every 16th column,
        // then a fixed butterfly over the 16 (deterministic)
        const int nr = (n * 16 + 31) & ~31;  // whole warps
        for (int t = threadIdx.x; t < nr; t += blockDim.x) {
            const int i = t >> 4, j = t & 15;
            float acc = 0.f;
            if (i < n)
                for (int k = j; k < n; k += 16) acc += cinv[i * n + k] * f[k];
#pragma unroll
            for (int m = 8; m >= 1; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
            if (j == 0 && i < n) e[i] = acc;
        }
        __syncthreads();
        return;
    }
    const int pairs = coarse_pairs(cv.d, cv.h, cv.w);
    if (n <= 256) {
        if (threadIdx.x < 32) {
            for (int c = threadIdx.x; c < n; c += 32) e[c] = 0.f;
            __syncwarp();
            for (int it = 0; it < 4 * pairs; ++it) {
                const int color = it < 2 * pairs ? (it & 1) : ((it & 1) ^ 1);
                tail_smooth<NB_PLAIN, true>(cv, e, f, nullptr, 1, 1, color);
            }
        }
        __syncthreads();
        return;
    }
    for (int c = threadIdx.x; c < n; c += blockDim.x) e[c] = 0.f;
    __syncthreads();
    for (int it = 0; it < 4 * pairs; ++it) {
        const int color = it < 2 * pairs ? (it & 1) : ((it & 1) ^ 1);
        tail_smooth<NB_PLAIN>(cv, e, f, nullptr, 1, 1, color);
    }
}

constexpr int kTailThreads = 1024;
constexpr int kTailSmemMax = 220 * 1024;

// Levels [A.lt, A.nl) by the calling block in its shared memory tsm.
__device__ __forceinline__ void tail_body(const TailArgs& A, float* tsm) {
    // Shared memory per level: wx, wy, wz, invd, e, f (n floats each).  The
    // level views are rebuilt from tsm + offset at every use, so every
    // access stays a shared-window access (a table of pointers would make
    // them generic loads).
    auto ncell = [&](int l) { return A.L[l].d * A.L[l].h * A.L[l].w; };
    auto off = [&](int l) {
        int o = 0;
        for (int k = A.lt; k < l; ++k) o += 6 * ncell(k);
        return o;
    };
    auto lv = [&](int l) -> LV {
        const TailLevel& T = A.L[l];
        const int n = ncell(l);
        float* p = tsm + off(l);
        LV v;
        v.nd = T.nd;
        v.d = T.d;
        v.h = T.h;
        v.w = T.w;
        v.flags = nullptr;
        v.wx = p;
        v.wy = p + n;
        v.wz = p + 2 * n;
        v.invd = p + 3 * n;
        v.dt = 0.f;
        return v;
    };
    auto E = [&](int l) -> float* { return tsm + off(l) + 4 * ncell(l); };
    auto F = [&](int l) -> float* { return tsm + off(l) + 5 * ncell(l); };
    for (int l = A.lt; l < A.nl; ++l) {
        const TailLevel& T = A.L[l];
        const int n = ncell(l);
        float* p = tsm + off(l);
        for (int c = threadIdx.x; c < n; c += blockDim.x) {
            p[c] = T.wx[c];
            p[n + c] = T.wy[c];
            p[2 * n + c] = T.nd == 3 ? T.wz[c] : 0.f;
            p[3 * n + c] = T.invd[c];
            if (l == A.lt) p[5 * n + c] = A.f_in[c];
        }
    }
    __syncthreads();
    const int nl = A.nl, ns = A.nsmooth;
    // down
    for (int l = A.lt; l + 1 < nl; ++l) {
        const TailLevel& c = A.L[l + 1];
        const LV v = lv(l);
        float* e = E(l);
        const float* f = F(l);
        tail_smooth<NB_FIRST>(v, e, f, nullptr, c.w, c.h, 1);
        if (ns == 1) tail_smooth<NB_SELF>(v, e, f, nullptr, c.w, c.h, 0);
        for (int k = 1; k < ns; ++k) {
            tail_smooth<NB_PLAIN>(v, e, f, nullptr, c.w, c.h, 0);
            tail_smooth<NB_PLAIN>(v, e, f, nullptr, c.w, c.h, 1);
        }
        tail_restrict(v, e, f, F(l + 1), c.d, c.h, c.w);
    }
    tail_coarsest(lv(nl - 1), E(nl - 1), F(nl - 1), A.cinv);
    // up
    for (int l = nl - 2; l >= A.lt; --l) {
        const TailLevel& c = A.L[l + 1];
        const LV v = lv(l);
        float* e = E(l);
        const float* f = F(l);
        tail_smooth<NB_PROLONG>(v, e, f, E(l + 1), c.w, c.h, 1);
        for (int k = 0; k < ns; ++k) {
            if (k > 0) tail_smooth<NB_PLAIN>(v, e, f, nullptr, c.w, c.h, 1);
            tail_smooth<NB_PLAIN>(v, e, f, nullptr, c.w, c.h, 0);
        }
    }
    const int n0 = ncell(A.lt);
    const float* e0 = E(A.lt);
    for (int c = threadIdx.x; c < n0; c += blockDim.x) A.e_out[c] = e0[c];
}

__global__ void __launch_bounds__(kTailThreads) k_mg_tail(TailArgs A, CgState* st) {
    if (st->done) return;
    extern __shared__ float tsm[];
    tail_body(A, tsm);
}

// ---------------------------------------------------------------------------
// Cluster tail (3D): the levels from the first one of at most kCtCells cells
// down to the coarsest, in ONE thread-block cluster of R blocks (16 where the
// device allows it, else 8).  Levels larger than kCtLocal cells are cut into
// z slabs of ppc = ceil(d / R) planes, one per rank, each rank holding its
// slab of wx, wy, wz, 1/diag, e and f in shared memory; a rank updates its own
// cells and reads the neighbouring planes of other ranks through distributed
// shared memory, with a cluster barrier between half-sweeps.  Smaller levels
// live in rank 0 alone and run the single-block tail's phases with block
// barriers.  Every cell is computed by the same formula, in the same order of
// operations, as k_mg_smooth / k_mg_restrict8 / the single-block tail, so the
// V-cycle is bit-identical to the per-level kernels plus k_mg_tail.

constexpr int kCtThreads = 1024;
constexpr int kCtCells = 32768;  // first level of the cluster tail: at most this many cells
constexpr int kCtLocal = 512;    // levels at most this large live in rank 0 alone
constexpr int kCtMaxRanks = 16;
constexpr int kCtSmemMax = 200 * 1024;

struct CtLevel {
    int d, h, w;
    int ppc;  // planes per rank (d: the level lives in rank 0)
    int off;  // offset (floats) of the level's block [wx | wy | wz | invd | e | f] in shared memory
    int P;    // floats per array of the block: ppc * h * w
    FastDiv fhalf, fh, fw, fhw, fppc;  // invariant divisors (w + 1) / 2, h, w, h * w, ppc
    const float* wx;
    const float* wy;
    const float* wz;
    const float* invd;
};

struct CtArgs {
    int lt, ls, nl, nsmooth, ranks;
    float* e_out;       // global e of level lt
    const float* f_in;  // global f of level lt
    const float* cinv;  // the coarsest level's pseudo-inverse, or null
    CtLevel L[kMaxLevels];
};

__device__ __forceinline__ unsigned ct_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ float* ct_map(float* p, unsigned rank) {
    unsigned long long r;
    asm volatile("mapa.u64 %0, %1, %2;" : "=l"(r) : "l"(p), "r"(rank));
    return (float*)r;
}

__device__ __forceinline__ void ct_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Array 0 (wx) of level L at plane z, on the rank that owns it.
__device__ __forceinline__ float* ct_plane(float* const* peer, const CtLevel& L, int z) {
    int zl;
    const int r = split(z, L.ppc, L.fppc, zl);
    return peer[r] + L.off + zl * L.h * L.w;
}

// Neighbour value of the smoother at the cell whose array-0 entry is q
// (z, y, x): e, f / diag (first half-sweep from e = 0) or e + the coarse
// correction of its parent (first post-smoothing half-sweep).
template <int MODE>
__device__ __forceinline__ float ct_nb(float* const* peer, const float* q, int P, const CtLevel* Lc, int z, int y,
                                       int x) {
    if (MODE == NB_FIRST) return q[5 * P] * q[3 * P];
    if (MODE == NB_PROLONG) {
        const float* pc = ct_plane(peer, *Lc, z >> 1) + 4 * Lc->P + (y >> 1) * Lc->w + (x >> 1);
        return q[4 * P] + *pc;
    }
    return q[4 * P];
}

// One half-sweep of a distributed level over the calling rank's planes.
// Every value a cell may need is loaded before any is used (a missing
// neighbour's offset is clamped to the cell itself and its value ignored),
// so a cell waits for one round of shared and distributed-shared loads.
template <int MODE>
__device__ void ct_smooth(float* const* peer, const CtLevel& L, const CtLevel* Lc, int rank, int color) {
    const int h = L.h, w = L.w, P = L.P;
    const int z0 = rank * L.ppc, nz = max(0, min(L.ppc, L.d - z0));
    const int half = (w + 1) >> 1, total = nz * h * half;
    float* B = peer[rank] + L.off;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        int k2, y;
        const int row = split(i, half, L.fhalf, k2);
        const int zl = split(row, h, L.fh, y), z = z0 + zl;
        const int x = 2 * k2 + ((y + z + color) & 1);
        if (x >= w) continue;
        const int c = row * w + x;
        const float* q = B + c;
        const bool hx = x + 1 < w, hy = y + 1 < h, hz = z + 1 < L.d;
        const int ox0 = x > 0 ? -1 : 0, ox1 = hx ? 1 : 0, oy0 = y > 0 ? -w : 0, oy1 = hy ? w : 0;
        const float* qd = z > 0 ? (zl > 0 ? q - h * w : ct_plane(peer, L, z - 1) + y * w + x) : q;
        const float* qu = hz ? (zl + 1 < L.ppc ? q + h * w : ct_plane(peer, L, z + 1) + y * w + x) : q;
        const float wxl = q[0], wxh_ = q[ox1], wyl = q[P], wyh_ = q[P + oy1], wzl = q[2 * P], wzh_ = qu[2 * P];
        const float inv = q[3 * P];
        float s = q[5 * P];
        if (MODE == NB_SELF) {
            B[4 * P + c] = s * inv;
            continue;
        }
        const float n0 = ct_nb<MODE>(peer, q + ox0, P, Lc, z, y, x + (x > 0 ? -1 : 0));
        const float n1 = ct_nb<MODE>(peer, q + ox1, P, Lc, z, y, x + ox1);
        const float n2 = ct_nb<MODE>(peer, q + oy0, P, Lc, z, y + (y > 0 ? -1 : 0), x);
        const float n3 = ct_nb<MODE>(peer, q + oy1, P, Lc, z, y + (hy ? 1 : 0), x);
        const float n4 = ct_nb<MODE>(peer, qd, P, Lc, z > 0 ? z - 1 : z, y, x);
        const float n5 = ct_nb<MODE>(peer, qu, P, Lc, hz ? z + 1 : z, y, x);
        const float wxh = hx ? wxh_ : 0.f, wyh = hy ? wyh_ : 0.f, wzh = hz ? wzh_ : 0.f;
        if (wxl != 0.f) s += wxl * n0;
        if (wxh != 0.f) s += wxh * n1;
        if (wyl != 0.f) s += wyl * n2;
        if (wyh != 0.f) s += wyh * n3;
        if (wzl != 0.f) s += wzl * n4;
        if (wzh != 0.f) s += wzh * n5;
        B[4 * P + c] = s * inv;
    }
}

// Residual of distributed level L summed over children into f of level Lc,
// one thread per child (eight lanes per coarse cell, summed by the first in
// (z, y, x) order as k_mg_restrict8 does).  Coarse plane Z is computed by the
// rank owning fine plane 2Z.
__device__ void ct_restrict(float* const* peer, const CtLevel& L, const CtLevel& Lc, int rank) {
    const int h = L.h, w = L.w, P = L.P;
    const int ch = Lc.h, cw = Lc.w, chw = ch * cw;
    // coarse planes Z with 2Z in [rank * ppc, (rank + 1) * ppc)
    const int Z0 = (rank * L.ppc + 1) / 2, Z1 = min(Lc.d, ((rank + 1) * L.ppc + 1) / 2);
    const int total = max(0, Z1 - Z0) * chw;
    const unsigned lane = threadIdx.x & 31, grp = lane & ~7u;
    const int n8 = (total * 8 + 31) & ~31;  // whole warps: every lane runs the same trips
    for (int t = threadIdx.x; t < n8; t += blockDim.x) {
        const int i = t >> 3, j = t & 7;
        int YX, X;
        const int Z = Z0 + split(i, chw, Lc.fhw, YX);
        const int Y = split(YX, cw, Lc.fw, X);
        const int z = 2 * Z + (j >> 2), y = 2 * Y + ((j >> 1) & 1), x = 2 * X + (j & 1);
        const bool has = i < total && z < L.d && y < h && x < w;
        float term = 0.f;
        if (has) {
            const int k = y * w + x;
            const float* q = ct_plane(peer, L, z) + k;
            const bool hx = x + 1 < w, hy = y + 1 < h, hz = z + 1 < L.d;
            const int ox0 = x > 0 ? -1 : 0, ox1 = hx ? 1 : 0, oy0 = y > 0 ? -w : 0, oy1 = hy ? w : 0;
            const float* pd = z > 0 ? ct_plane(peer, L, z - 1) + k : q;
            const float* pu = hz ? ct_plane(peer, L, z + 1) + k : q;
            const float wxl = q[0], wxh_ = q[ox1], wyl = q[P], wyh_ = q[P + oy1], wzl = q[2 * P], wzh_ = pu[2 * P];
            const float ecv = q[4 * P], e0 = q[4 * P + ox0], e1 = q[4 * P + ox1], e2 = q[4 * P + oy0],
                        e3 = q[4 * P + oy1], e4 = pd[4 * P], e5 = pu[4 * P], fv = q[5 * P];
            const float wxh = hx ? wxh_ : 0.f, wyh = hy ? wyh_ : 0.f, wzh = hz ? wzh_ : 0.f;
            float a = 0.f;
            if (wxl != 0.f) a += wxl * (ecv - e0);
            if (wxh != 0.f) a += wxh * (ecv - e1);
            if (wyl != 0.f) a += wyl * (ecv - e2);
            if (wyh != 0.f) a += wyh * (ecv - e3);
            if (wzl != 0.f) a += wzl * (ecv - e4);
            if (wzh != 0.f) a += wzh * (ecv - e5);
            term = fv - a;
        }
        const unsigned valid = __ballot_sync(0xffffffffu, has);
        float sum = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float tk = __shfl_sync(0xffffffffu, term, grp + k);
            if ((valid >> (grp + k)) & 1u) sum += tk;
        }
        if (j == 0 && i < total) ct_plane(peer, Lc, Z)[5 * Lc.P + YX] = sum;
    }
}

__global__ void __launch_bounds__(kCtThreads) k_mg_ctail(CtArgs A, CgState* st) {
    if (st->done) return;  // the same value in every block of the cluster
    extern __shared__ float csm[];
    __shared__ float* peer[kCtMaxRanks];
    const int rank = (int)ct_rank();
    if (threadIdx.x < A.ranks) peer[threadIdx.x] = ct_map(csm, threadIdx.x);
    __syncthreads();
    const int lt = A.lt, ls = A.ls, nl = A.nl, ns = A.nsmooth;
    // load: the distributed levels' slabs, and rank 0's levels
    for (int l = lt; l < nl; ++l) {
        const CtLevel& L = A.L[l];
        const int z0 = l < ls ? rank * L.ppc : 0;
        const int nz = l < ls ? max(0, min(L.ppc, L.d - z0)) : (rank == 0 ? L.d : 0);
        const int n = nz * L.h * L.w, g0 = z0 * L.h * L.w;
        float* B = csm + L.off;
        for (int c = threadIdx.x; c < n; c += blockDim.x) {
            B[c] = L.wx[g0 + c];
            B[L.P + c] = L.wy[g0 + c];
            B[2 * L.P + c] = L.wz[g0 + c];
            B[3 * L.P + c] = L.invd[g0 + c];
            if (l == lt) B[5 * L.P + c] = A.f_in[g0 + c];
        }
    }
    ct_sync();
    // down through the distributed levels
    for (int l = lt; l < ls; ++l) {
        const CtLevel& L = A.L[l];
        ct_smooth<NB_FIRST>(peer, L, nullptr, rank, 1);
        ct_sync();
        if (ns == 1) {
            ct_smooth<NB_SELF>(peer, L, nullptr, rank, 0);
            ct_sync();
        }
        for (int k = 1; k < ns; ++k) {
            ct_smooth<NB_PLAIN>(peer, L, nullptr, rank, 0);
            ct_sync();
            ct_smooth<NB_PLAIN>(peer, L, nullptr, rank, 1);
            ct_sync();
        }
        ct_restrict(peer, L, A.L[l + 1], rank);
        ct_sync();
    }
    // rank 0: levels [ls, nl) as in the single-block tail
    if (rank == 0) {
        auto lv = [&](int l) -> LV {
            const CtLevel& T = A.L[l];
            float* p = csm + T.off;
            LV v;
            v.nd = 3;
            v.d = T.d;
            v.h = T.h;
            v.w = T.w;
            v.flags = nullptr;
            v.wx = p;
            v.wy = p + T.P;
            v.wz = p + 2 * T.P;
            v.invd = p + 3 * T.P;
            v.dt = 0.f;
            return v;
        };
        auto E = [&](int l) -> float* { return csm + A.L[l].off + 4 * A.L[l].P; };
        auto F = [&](int l) -> float* { return csm + A.L[l].off + 5 * A.L[l].P; };
        for (int l = ls; l + 1 < nl; ++l) {
            const CtLevel& c = A.L[l + 1];
            const LV v = lv(l);
            float* e = E(l);
            const float* f = F(l);
            tail_smooth<NB_FIRST>(v, e, f, nullptr, c.w, c.h, 1);
            if (ns == 1) tail_smooth<NB_SELF>(v, e, f, nullptr, c.w, c.h, 0);
            for (int k = 1; k < ns; ++k) {
                tail_smooth<NB_PLAIN>(v, e, f, nullptr, c.w, c.h, 0);
                tail_smooth<NB_PLAIN>(v, e, f, nullptr, c.w, c.h, 1);
            }
            tail_restrict(v, e, f, F(l + 1), c.d, c.h, c.w);
        }
        tail_coarsest(lv(nl - 1), E(nl - 1), F(nl - 1), A.cinv);
        for (int l = nl - 2; l >= ls; --l) {
            const CtLevel& c = A.L[l + 1];
            const LV v = lv(l);
            float* e = E(l);
            const float* f = F(l);
            tail_smooth<NB_PROLONG>(v, e, f, E(l + 1), c.w, c.h, 1);
            for (int k = 0; k < ns; ++k) {
                if (k > 0) tail_smooth<NB_PLAIN>(v, e, f, nullptr, c.w, c.h, 1);
                tail_smooth<NB_PLAIN>(v, e, f, nullptr, c.w, c.h, 0);
            }
        }
    }
    ct_sync();
    // up through the distributed levels
    for (int l = ls - 1; l >= lt; --l) {
        const CtLevel& L = A.L[l];
        ct_smooth<NB_PROLONG>(peer, L, &A.L[l + 1], rank, 1);
        ct_sync();
        for (int k = 0; k < ns; ++k) {
            if (k > 0) {
                ct_smooth<NB_PLAIN>(peer, L, nullptr, rank, 1);
                ct_sync();
            }
            ct_smooth<NB_PLAIN>(peer, L, nullptr, rank, 0);
            ct_sync();
        }
    }
    // level lt's correction to global memory (own slab, own shared memory)
    const CtLevel& L = A.L[lt];
    const int z0 = rank * L.ppc, nz = max(0, min(L.ppc, L.d - z0));
    const float* Eo = csm + L.off + 4 * L.P;
    for (int c = threadIdx.x; c < nz * L.h * L.w; c += blockDim.x) A.e_out[z0 * L.h * L.w + c] = Eo[c];
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
        cudaFree(ex->mg->e0b);
        cudaFree(ex->mg->cinv);
        delete ex->mg;
        ex->mg = nullptr;
    }
}

static int blocks_for(const pg_grid* g, i64 n) { return grid_blocks(g, n, kMgThreads, 8); }

static int pair_setup(pg_grid* g, MgHierarchy* H);
static void ctail_setup(MgHierarchy* H);

// Moore-Penrose pseudo-inverse of the symmetric n x n matrix a (row-major,
// overwritten) by cyclic Jacobi rotations in double; eigenvalues below
// 1e-10 of the largest count as zero (the constant mode of every closed
// fluid component, and cells without open faces).
static void sym_pinv(int n, std::vector<double>& a) {
    std::vector<double> v((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
    auto A = [&](int i, int j) -> double& { return a[(size_t)i * n + j]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) (i == j ? tot : off) += A(i, j) * A(i, j);
        if (off <= 1e-30 * (tot + off)) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A(p, q);
                if (apq == 0.0) continue;
                const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < n; ++k) {  // columns p, q
                    const double akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - sn * akq;
                    A(k, q) = sn * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {  // rows p, q
                    const double apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - sn * aqk;
                    A(q, k) = sn * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
                    v[(size_t)k * n + p] = c * vkp - sn * vkq;
                    v[(size_t)k * n + q] = sn * vkp + c * vkq;
                }
            }
    }
    double lmax = 0.0;
    for (int i = 0; i < n; ++i) lmax = std::max(lmax, std::fabs(A(i, i)));
    std::vector<double> lam(n);
    for (int i = 0; i < n; ++i) lam[i] = A(i, i);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double sum = 0.0;
            for (int k = 0; k < n; ++k)
                if (lam[k] > 1e-10 * lmax) sum += v[(size_t)i * n + k] * v[(size_t)j * n + k] / lam[k];
            A(i, j) = sum;
        }
}

// The coarsest level's operator (its face weights; the diagonal is their
// sum, as 1/diag is) and its pseudo-inverse on the device, when the level
// has at most kCinvCells cells (PG_MG_CINV=0 keeps the Gauss-Seidel sweeps;
// a diagnostic switch read per build).
static int coarsest_pinv(pg_grid* g, MgHierarchy* H) {
    const int nl = H->nlev;
    const char* env = getenv("PG_MG_CINV");
    if (nl < 2 || (env && env[0] == '0')) return PG_OK;
    const MgLevel& L = H->lv[nl - 1];
    const int n = (int)L.D.nc(), d = (int)L.D.d, h = (int)L.D.h, w = (int)L.D.w;
    if (n > kCinvCells) return PG_OK;
    std::vector<float> wx(n), wy(n), wz(n, 0.f);
    PG_CUDA(cudaMemcpyAsync(wx.data(), L.wx, sizeof(float) * n, cudaMemcpyDeviceToHost, g->stream));
    PG_CUDA(cudaMemcpyAsync(wy.data(), L.wy, sizeof(float) * n, cudaMemcpyDeviceToHost, g->stream));
    if (L.D.nd == 3) PG_CUDA(cudaMemcpyAsync(wz.data(), L.wz, sizeof(float) * n, cudaMemcpyDeviceToHost, g->stream));
    PG_CUDA(cudaStreamSynchronize(g->stream));
    std::vector<double> a((size_t)n * n, 0.0);
    auto link = [&](int c, int k, float wt) {  // face between cells c and k
        if (wt == 0.f) return;
        a[(size_t)c * n + c] += wt;
        a[(size_t)k * n + k] += wt;
        a[(size_t)c * n + k] -= wt;
        a[(size_t)k * n + c] -= wt;
    };
    for (int z = 0; z < d; ++z)
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const int c = (z * h + y) * w + x;
                if (x > 0) link(c, c - 1, wx[c]);
                if (y > 0) link(c, c - w, wy[c]);
                if (z > 0) link(c, c - h * w, wz[c]);
            }
    sym_pinv(n, a);
    std::vector<float> m((size_t)n * n);
    for (size_t i = 0; i < m.size(); ++i) m[i] = (float)a[i];
    PG_CUDA(cudaMalloc(&H->cinv, sizeof(float) * m.size()));
    PG_CUDA(cudaMemcpyAsync(H->cinv, m.data(), sizeof(float) * m.size(), cudaMemcpyHostToDevice, g->stream));
    PG_CUDA(cudaStreamSynchronize(g->stream));
    return PG_OK;
}

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
    // Fused fine-level pairs: 3D, rows of a multiple of 16 cells (the flags'
    // TMA row stride), the flags' map encodable; PG_MG_PAIRS=0 keeps the
    // separate half-sweeps (a diagnostic switch read per build).
    {
        const char* env = getenv("PG_MG_PAIRS");
        const bool want = !(env && env[0] == '0');
        const Dims& D0 = g->dims;
        if (want && D0.nd == 3 && nl > 1 && D0.w % 16 == 0 &&
            encode_map_3d(&H->gmap, H->flags, 1, D0.w, D0.h, D0.d, kPGw, kPGh)) {
            err = cudaMalloc(&H->e0b, sizeof(float) * (size_t)D0.nc());
            if (err != cudaSuccess) return cuda_fail(err, "cudaMalloc(mg fine scratch)");
            const int prc = pair_setup(g, H);
            if (prc) return prc;
            H->pairs = H->pair_cap > 0;
            const char* keep = getenv("PG_MG_L2KEEP");
            H->l2keep = !(keep && keep[0] == '0');
        }
    }
    // fluid components of the mask (host labelling, once per mask)
    {
        std::vector<uint8_t> hf((size_t)g->dims.nc());
        PG_CUDA(cudaMemcpy(hf.data(), g->flags, hf.size(), cudaMemcpyDeviceToHost));
        i64 nf = 0;
        for (uint8_t f : hf) nf += f != 0;
        H->nfluid = (double)nf;
        std::vector<i64> cells;
        std::vector<int> start;
        find_pockets(hf.data(), g->dims.nd, g->dims.d, g->dims.h, g->dims.w, 0, cells, start);
        int prc = upload_pockets(cells, start, &H->pockets);
        if (prc) return prc;
    }
    ctail_setup(H);
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
    if (const int crc = coarsest_pinv(g, H)) return crc;
    *out = H;
    return PG_OK;
}

int set_stage_wait_polls_mg(unsigned polls) {
    PG_CUDA(cudaMemcpyToSymbol(c_stage_wait_polls, &polls, sizeof(polls)));
    return PG_OK;
}

// ---------------------------------------------------------------------------
// Fused fine-level pairs: launch setup.

template <int M1, bool RZ>
static int pair_attr() {
    return (int)cudaFuncSetAttribute(k_mg_pair<M1, RZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)PairCfg<M1>::kSmem);
}

// Opt every instantiation into its shared memory and size the grid by the
// resident block count (outside any stream capture).
static int pair_setup(pg_grid* g, MgHierarchy* H) {
    int e = pair_attr<PR_SELF, false>() | pair_attr<PR_PLAIN, false>() | pair_attr<PR_PROLONG, false>() |
            pair_attr<PR_PLAIN, true>() | pair_attr<PR_PROLONG, true>();
    if (e) return cuda_fail((cudaError_t)e, "cudaFuncSetAttribute(k_mg_pair)");
    int bps[5] = {};
    PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps[0], k_mg_pair<PR_PLAIN, false>, kPThreads,
                                                          PairCfg<PR_PLAIN>::kSmem));
    PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps[1], k_mg_pair<PR_PLAIN, true>, kPThreads,
                                                          PairCfg<PR_PLAIN>::kSmem));
    PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps[2], k_mg_pair<PR_SELF, false>, kPThreads,
                                                          PairCfg<PR_SELF>::kSmem));
    PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps[3], k_mg_pair<PR_PROLONG, false>, kPThreads,
                                                          PairCfg<PR_PROLONG>::kSmem));
    PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps[4], k_mg_pair<PR_PROLONG, true>, kPThreads,
                                                          PairCfg<PR_PROLONG>::kSmem));
    const int plain = std::min(bps[0], std::min(bps[1], bps[2]));
    H->pair_cap_plain = std::min(plain * g->num_sms, kMaxBlocks);
    H->pair_cap = std::min(std::min(plain, std::min(bps[3], bps[4])) * g->num_sms, kMaxBlocks);
    const MgLevel& C = H->lv[1];
    if (!encode_map_3d(&H->cmap, C.e, 4, C.D.w, C.D.h, C.D.d, kPCw, kPCh)) H->pair_cap = 0;
    // TMA-staged fine restriction (PG_MG_RESTRICT_TMA=0 keeps the plain kernel; a diagnostic switch read
    // per build)
    const Dims& D0 = H->D0;
    const char* env = getenv("PG_MG_RESTRICT_TMA");
    H->restrict_tma = !(env && env[0] == '0') && D0.d % 2 == 0 && D0.h % 2 == 0 && D0.w % 2 == 0 &&
                      restrict_cap(g) > 0 && encode_map_3d(&H->rgmap, H->flags, 1, D0.w, D0.h, D0.d, kQX, kQY);
    return PG_OK;
}

// Tensor map of a fine-level float vector with a box of kPEw x by, encoded
// once per (pointer, box); nullptr when the vector cannot be mapped.
static const CUtensorMap* vec_map(const MgHierarchy& H, const float* p, int by, int bx = kPEw) {
    for (auto& m : H.maps)
        if (m.p == p && m.by == by && m.bx == bx) return &m.m;
    MgHierarchy::MapEnt& m = H.maps[H.next_map];
    const Dims& D = H.D0;
    if (!encode_map_3d(&m.m, p, 4, D.w, D.h, D.d, bx, by)) return nullptr;
    H.next_map = (H.next_map + 1) % 8;
    m.p = p;
    m.bx = bx;
    m.by = by;
    return &m.m;
}

struct PairLaunch {
    const CUtensorMap* fm;  // f (the residual r)
    PairArgs a;
    int nb_plain, nb_prolong;  // blocks of the launches without / with the coarse correction
};

// Geometry of the pair launches of one V-cycle; false when a vector cannot
// be mapped (the V-cycle then uses the half-sweeps).
static bool pair_plan(const MgHierarchy& H, const float* r, const float* z, PairLaunch* P) {
    if (!H.pairs || !vec_map(H, z, kPEh) || !vec_map(H, H.e0b, kPEh) || !(P->fm = vec_map(H, r, kPFh)))
        return false;
    const Dims& D = H.D0;
    PairArgs& a = P->a;
    a.d = (int)D.d;
    a.h = (int)D.h;
    a.w = (int)D.w;
    a.dt = (float)H.dt;
    a.tiles_x = (a.w + kPX - 1) / kPX;
    a.tiles_y = (a.h + kPY - 1) / kPY;
    a.l2keep = H.l2keep;
    // every resident block, each with an equal share of the plane-tiles
    P->nb_plain = zwalk_blocks(a.tiles_x * a.tiles_y, a.d, H.pair_cap_plain);
    P->nb_prolong = zwalk_blocks(a.tiles_x * a.tiles_y, a.d, H.pair_cap);
    return true;
}

template <int M1, bool RZ>
static void pair_t(pg_grid* g, const MgHierarchy& H, const CUtensorMap* em, const PairLaunch& P, const PairArgs& a) {
    cudaStream_t s = g->stream;
    const int nb = M1 == PR_PROLONG ? P.nb_prolong : P.nb_plain;
    PG_LAUNCH(KK_MG_PAIR, s,
              k_mg_pair<M1, RZ><<<nb, kPThreads, PairCfg<M1>::kSmem, s>>>(*em, *P.fm, H.gmap, H.cmap, a,
                                                                          g->ws.state, g->ws.partials));
}

// One fused pair: first half-sweep over colour c1 in `mode` from ein
// (unused for PR_SELF; PR_PROLONG adds the level-1 correction), second
// over the other colour; both into eout.
static void pair(pg_grid* g, const MgHierarchy& H, const PairLaunch& P, int mode, int c1, bool rz, const float* ein,
                 float* eout) {
    PairArgs a = P.a;
    a.eout = eout;
    a.c1 = c1;
    const CUtensorMap* em = vec_map(H, ein ? ein : H.e0b, kPEh);  // cached by pair_plan
    if (mode == PR_SELF) pair_t<PR_SELF, false>(g, H, em, P, a);
    else if (mode == PR_PROLONG && rz) pair_t<PR_PROLONG, true>(g, H, em, P, a);
    else if (mode == PR_PROLONG) pair_t<PR_PROLONG, false>(g, H, em, P, a);
    else if (rz) pair_t<PR_PLAIN, true>(g, H, em, P, a);
    else pair_t<PR_PLAIN, false>(g, H, em, P, a);
}

// The fine restriction of 3D grids with even sides by k_mg_restrict3p;
// false (nothing launched) when it does not apply.
static bool restrict_tma(pg_grid* g, const MgHierarchy& H, const float* e, const float* f, float* fc) {
    if (!H.restrict_tma) return false;
    const CUtensorMap* em = vec_map(H, e, kQEh, kQEw);
    const CUtensorMap* fm = em ? vec_map(H, f, kQY, kQX) : nullptr;
    if (!fm) return false;
    const Dims& D = H.D0;
    RestrictArgs a;
    a.d = (int)D.d;
    a.h = (int)D.h;
    a.w = (int)D.w;
    a.ch = (int)H.lv[1].D.h;
    a.cw = (int)H.lv[1].D.w;
    a.dt = (float)H.dt;
    a.fc = fc;
    a.tiles_x = (a.w + kQX - 1) / kQX;
    a.tiles_y = (a.h + kQY - 1) / kQY;
    const int nb = zwalk_blocks(a.tiles_x * a.tiles_y, a.d / 2, restrict_cap(g));
    cudaStream_t s = g->stream;
    PG_LAUNCH(KK_MG_RESTRICT, s, k_mg_restrict3p<<<nb, kQThreads, kQSmem, s>>>(*em, *fm, H.rgmap, a, g->ws.state));
    return true;
}

// ---------------------------------------------------------------------------
// Tail launch.

static size_t tail_smem(const MgHierarchy& H) {
    size_t smem = 0;
    for (int l = H.tail; l < H.nlev; ++l) smem += 6 * sizeof(float) * (size_t)H.lv[l].D.nc();
    return smem;
}

static TailArgs tail_args(const MgHierarchy& H, int nsmooth) {
    TailArgs A;
    A.lt = H.tail;
    A.nl = H.nlev;
    A.nsmooth = nsmooth;
    A.e_out = H.lv[H.tail].e;
    A.f_in = H.lv[H.tail].f;
    A.cinv = H.cinv;
    for (int l = H.tail; l < H.nlev; ++l) {
        const MgLevel& L = H.lv[l];
        A.L[l] = TailLevel{L.D.nd, (int)L.D.d, (int)L.D.h, (int)L.D.w, L.wx, L.wy, L.wz, L.invd};
    }
    return A;
}

// The single-block tail: levels [H.tail, nl).
static int launch_tail(pg_grid* g, const MgHierarchy& H, int nsmooth) {
    const TailArgs A = tail_args(H, nsmooth);
    const size_t smem = tail_smem(H);
    static bool attr = false;
    if (!attr) {
        PG_CUDA(cudaFuncSetAttribute(k_mg_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmemMax));
        attr = true;
    }
    if (smem > (size_t)kTailSmemMax) return bad_arg("PG_PRECOND_MG: multigrid tail does not fit in shared memory");
    PG_LAUNCH(KK_MG_COARSE, g->stream, k_mg_tail<<<1, kTailThreads, smem, g->stream>>>(A, g->ws.state));
    return PG_OK;
}

// Shared-memory layout of the cluster tail with R ranks; 0 when it does not
// fit.
static size_t ctail_layout(const MgHierarchy& H, int lt, int ls, int R, CtArgs* A) {
    size_t off = 0;
    for (int l = lt; l < H.nlev; ++l) {
        const Dims& D = H.lv[l].D;
        CtLevel& L = A->L[l];
        L.d = (int)D.d;
        L.h = (int)D.h;
        L.w = (int)D.w;
        L.ppc = l < ls ? (int)((D.d + R - 1) / R) : (int)D.d;
        L.P = (int)(((size_t)L.ppc * D.h * D.w + 3) & ~(size_t)3);
        L.fhalf = fast_div((unsigned)((D.w + 1) / 2));
        L.fh = fast_div((unsigned)D.h);
        L.fw = fast_div((unsigned)D.w);
        L.fhw = fast_div((unsigned)(D.h * D.w));
        L.fppc = fast_div((unsigned)L.ppc);
        L.off = (int)off;
        L.wx = H.lv[l].wx;
        L.wy = H.lv[l].wy;
        L.wz = H.lv[l].wz;
        L.invd = H.lv[l].invd;
        off += 6 * (size_t)L.P;
    }
    const size_t bytes = off * sizeof(float);
    return bytes <= (size_t)kCtSmemMax ? bytes : 0;
}

static cudaLaunchConfig_t ctail_config(int R, size_t smem, cudaStream_t s, cudaLaunchAttribute* at) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(R, 1, 1);
    cfg.blockDim = dim3(kCtThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = R;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cfg;
}

// Cluster tail for 3D hierarchies: a level of at most kCtCells cells above
// the rank-0 levels, 16 or 8 ranks that fit and can be resident together;
// PG_MG_CTAIL=0 keeps the per-level kernels and the single-block tail (a
// diagnostic switch read per build).
static void ctail_setup(MgHierarchy* H) {
    H->ct_lt = 0;
    const char* env = getenv("PG_MG_CTAIL");
    if ((env && env[0] == '0') || H->D0.nd != 3) return;
    const int nl = H->nlev;
    int lt = 0, ls = 0;
    for (int l = 1; l < nl; ++l)
        if (H->lv[l].D.nc() <= kCtCells) {
            lt = l;
            break;
        }
    if (lt == 0) return;
    for (int l = lt; l < nl; ++l)
        if (H->lv[l].D.nc() <= kCtLocal) {
            ls = l;
            break;
        }
    if (ls <= lt || ls > nl - 1) return;
    for (int R : {16, 8}) {
        CtArgs A{};
        const size_t smem = ctail_layout(*H, lt, ls, R, &A);
        if (smem == 0) continue;
        if (cudaFuncSetAttribute(k_mg_ctail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
            (R > 8 && cudaFuncSetAttribute(k_mg_ctail, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                          cudaSuccess)) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchAttribute at[1];
        const cudaLaunchConfig_t cfg = ctail_config(R, smem, nullptr, at);
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, k_mg_ctail, &cfg) != cudaSuccess || nclusters < 1) {
            cudaGetLastError();
            continue;
        }
        H->ct_lt = lt;
        H->ct_ls = ls;
        H->ct_ranks = R;
        H->ct_smem = smem;
        return;
    }
}

static int launch_ctail(pg_grid* g, const MgHierarchy& H, int nsmooth) {
    CtArgs A{};
    ctail_layout(H, H.ct_lt, H.ct_ls, H.ct_ranks, &A);
    A.lt = H.ct_lt;
    A.ls = H.ct_ls;
    A.nl = H.nlev;
    A.nsmooth = nsmooth;
    A.ranks = H.ct_ranks;
    A.e_out = H.lv[H.ct_lt].e;
    A.f_in = H.lv[H.ct_lt].f;
    A.cinv = H.cinv;
    cudaLaunchAttribute at[1];
    const cudaLaunchConfig_t cfg = ctail_config(H.ct_ranks, H.ct_smem, g->stream, at);
    cudaError_t err = cudaSuccess;
    PG_LAUNCH(KK_MG_COARSE, g->stream, err = cudaLaunchKernelEx(&cfg, k_mg_ctail, A, g->ws.state));
    if (err != cudaSuccess) return cuda_fail(err, "cluster tail launch");
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
              k_mg_smooth<L0, MODE, RZ><<<blocks_for(g, n), kMgThreads, 0, s>>>(
                  v, e, f, ec, cw, ch, color, g->ws.state, g->ws.partials, fast_div((unsigned)((v.w + 1) >> 1)),
                  fast_div((unsigned)v.h)));
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
static int vcycle(pg_grid* g, const MgHierarchy& H, const float* r, float* z, int nsmooth, int l0 = 0);

// z = P V(P r): P removes the mean of every fluid component when there are
// several (pg_pocket.cu); r is projected in place (the CG's recursive
// residual then measures the consistent part).
static int vcycle_projected(pg_grid* g, const MgHierarchy& H, float* r, float* z, int nsmooth) {
    pocket_project(g->stream, r, H.pockets);
    const int rc = vcycle(g, H, r, z, nsmooth);
    pocket_project(g->stream, z, H.pockets);
    return rc;
}

// l0 = 1: only the coarse part, from level 1's f (already restricted) to
// its correction e.
static int vcycle(pg_grid* g, const MgHierarchy& H, const float* r, float* z, int nsmooth, int l0) {
    cudaStream_t s = g->stream;
    const int nl = H.nlev;
    auto E = [&](int l) -> float* { return l == 0 ? z : H.lv[l].e; };
    auto F = [&](int l) -> const float* { return l == 0 ? r : H.lv[l].f; };
    if (l0 > 0 && nl == 1) return bad_arg("vcycle: no coarse levels");
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
    const bool ctail = H.ct_lt > 0;
    const bool tail = ctail || H.tail < nl;
    const int top = ctail ? H.ct_lt : tail ? H.tail : nl - 1;
    // Fine level of 3D grids as fused pairs: 2 * nsmooth of them alternate
    // between the scratch and z (pair k writes pout[k & 1]), so the last one
    // lands in z; the pre-smoothed correction is pout[(nsmooth - 1) & 1].
    PairLaunch P;
    const bool pairs = l0 == 0 && pair_plan(H, r, z, &P);
    float* const pout[2] = {H.e0b, z};
    // down
    for (int l = l0; l < top; ++l) {
        float* e = E(l);
        const float* f = F(l);
        if (l == 0 && pairs) {
            pair(g, H, P, PR_SELF, 0, false, nullptr, pout[0]);
            for (int k = 1; k < nsmooth; ++k) pair(g, H, P, PR_PLAIN, 0, false, pout[(k - 1) & 1], pout[k & 1]);
            e = pout[(nsmooth - 1) & 1];
        } else {
            // pre-smoothing: (red, black) x nsmooth from e = 0; the first red is implicit
            smooth_lv(g, H, l, e, f, nullptr, 1, NB_FIRST);
            if (nsmooth == 1) smooth_lv(g, H, l, e, f, nullptr, 0, NB_SELF);  // store the implicit red values
            for (int k = 1; k < nsmooth; ++k) {
                smooth_lv(g, H, l, e, f, nullptr, 0, NB_PLAIN);
                smooth_lv(g, H, l, e, f, nullptr, 1, NB_PLAIN);
            }
        }
        const LV v = view(H, l);
        const MgLevel& C = H.lv[l + 1];
        const i64 nc = C.D.nc();
        if (l == 0 && pairs && restrict_tma(g, H, e, f, C.f)) {
        } else {
            // one thread per child where there are few coarse cells, else
            // one per coarse cell (a thread per child measured 10.7 -> 5.3 us
            // for 32^3 coarse cells but 14 -> 19 us for 64^3)
            const int kind = l == 0 ? KK_MG_RESTRICT : KK_MG_RESTRICT_C;
            const int cd = (int)C.D.d, ch = (int)C.D.h, cw = (int)C.D.w;
            const FastDiv fcw = fast_div((unsigned)cw), fch = fast_div((unsigned)ch);
            cudaStream_t ss = s;
            if (nc <= kRestrictPerChild) {
                if (l == 0)
                    PG_LAUNCH(kind, ss, k_mg_restrict8<true><<<blocks_for(g, 8 * nc), kMgThreads, 0, ss>>>(v, e, f, C.f, cd, ch, cw, g->ws.state, fcw, fch));
                else
                    PG_LAUNCH(kind, ss, k_mg_restrict8<false><<<blocks_for(g, 8 * nc), kMgThreads, 0, ss>>>(v, e, f, C.f, cd, ch, cw, g->ws.state, fcw, fch));
            } else {
                if (l == 0)
                    PG_LAUNCH(kind, ss, k_mg_restrict<true><<<blocks_for(g, nc), kMgThreads, 0, ss>>>(v, e, f, C.f, cd, ch, cw, g->ws.state, fcw, fch));
                else
                    PG_LAUNCH(kind, ss, k_mg_restrict<false><<<blocks_for(g, nc), kMgThreads, 0, ss>>>(v, e, f, C.f, cd, ch, cw, g->ws.state, fcw, fch));
            }
        }
    }
    if (tail) {
        const int rc = ctail ? launch_ctail(g, H, nsmooth) : launch_tail(g, H, nsmooth);
        if (rc) return rc;
    } else {
        const LV v = view(H, nl - 1);
        PG_LAUNCH(KK_MG_COARSE, s,
                  k_mg_coarse<<<1, kCoarseThreads, 0, s>>>(v, H.lv[nl - 1].e, H.lv[nl - 1].f, g->ws.state));
    }
    // up
    for (int l = top - 1; l >= l0; --l) {
        float* e = E(l);
        const float* f = F(l);
        const float* ec = H.lv[l + 1].e;
        if (l == 0 && pairs) {
            for (int k = nsmooth; k < 2 * nsmooth; ++k)
                pair(g, H, P, k == nsmooth ? PR_PROLONG : PR_PLAIN, 1, k == 2 * nsmooth - 1, pout[(k - 1) & 1],
                     pout[k & 1]);
            continue;
        }
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
    bool writes_input() const override { return H->pockets.ncomp > 1; }
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
    // One fluid component: z's constant mode on it is removed lazily inside
    // the CG kernels (the coarse sweeps amplify the constant part that FP32
    // rounding leaves in r; unremoved, it swamps A p near tight tolerances).
    // Several components are projected explicitly around the V-cycle.
    CgConfig c2 = cfg;
    c2.nfluid = H->pockets.ncomp > 1 ? 0.0 : H->nfluid;
    return run_cg<T>(g, c2, buf, st, &hook);
}

template int solve_mgpcg<float>(pg_grid*, const pg_solver_params*, const CgConfig&, CgBuffers<float>, pg_pcg_stats*);
template int solve_mgpcg<double>(pg_grid*, const pg_solver_params*, const CgConfig&, CgBuffers<double>,
                                 pg_pcg_stats*);

}  // namespace pg

using namespace pg;

// The coarsest level's pseudo-inverse routine on a caller's symmetric matrix
// (host only; for tests).
extern "C" int pg_debug_sym_pinv(int n, double* a) {
    if (n < 1 || n > 4096 || !a) return bad_arg("pg_debug_sym_pinv: bad argument");
    std::vector<double> m(a, a + (size_t)n * n);
    sym_pinv(n, m);
    std::copy(m.begin(), m.end(), a);
    return PG_OK;
}

// Device time of one V-cycle and of its coarse part (levels >= 1), each
// captured once into a CUDA graph and replayed `reps` times between two
// events on a private stream; r = 0 (the kernels' work does not depend on
// the values).  Diagnostic: the coarse levels' kernels are too short to time
// one by one without the timing itself dominating.
extern "C" int pg_debug_mg_vcycle_ms(pg_grid* g, double dt, int nsmooth, int reps, double* full_ms,
                                     double* coarse_ms) {
    if (!g || !full_ms || !coarse_ms || reps < 1 || nsmooth < 1) return bad_arg("pg_debug_mg_vcycle_ms: bad argument");
    MgHierarchy* H = nullptr;
    int rc = ensure_mg(g, dt, &H);
    if (rc) return rc;
    if (H->nlev < 2) return bad_arg("pg_debug_mg_vcycle_ms: no coarse levels");
    if ((rc = ensure_workspace(g))) return rc;
    const size_t bytes = sizeof(float) * (size_t)g->dims.nc();
    float *r = nullptr, *z = nullptr;
    PG_CUDA(cudaMalloc(&r, bytes));
    cudaError_t err = cudaMalloc(&z, bytes);
    if (err != cudaSuccess) {
        cudaFree(r);
        return cuda_fail(err, "cudaMalloc(vcycle timing)");
    }
    cudaStream_t cs = nullptr, saved = g->stream;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    double out[2] = {0.0, 0.0};
    err = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreate(&ev[0]);
    if (err == cudaSuccess) err = cudaEventCreate(&ev[1]);
    if (err == cudaSuccess) err = cudaMemsetAsync(r, 0, bytes, cs);
    if (err == cudaSuccess) err = cudaMemsetAsync(z, 0, bytes, cs);
    if (err == cudaSuccess) err = cudaMemsetAsync(g->ws.state, 0, sizeof(CgState), cs);
    for (int k = 0; k < 2 && err == cudaSuccess && rc == PG_OK; ++k) {
        g->stream = cs;
        prof_capture_begin();
        err = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (err == cudaSuccess) {
            rc = vcycle(g, *H, r, z, nsmooth, k);
            const cudaError_t e2 = cudaStreamEndCapture(cs, &graph[k]);
            if (err == cudaSuccess) err = e2;
        }
        prof_capture_end();
        g->stream = saved;
        if (err == cudaSuccess && rc == PG_OK) err = cudaGraphInstantiate(&exec[k], graph[k], 0);
        for (int i = 0; i < 3 && err == cudaSuccess && rc == PG_OK; ++i) err = cudaGraphLaunch(exec[k], cs);
        if (err == cudaSuccess && rc == PG_OK) err = cudaEventRecord(ev[0], cs);
        for (int i = 0; i < reps && err == cudaSuccess && rc == PG_OK; ++i) err = cudaGraphLaunch(exec[k], cs);
        if (err == cudaSuccess && rc == PG_OK) err = cudaEventRecord(ev[1], cs);
        if (err == cudaSuccess && rc == PG_OK) err = cudaEventSynchronize(ev[1]);
        float ms = 0.f;
        if (err == cudaSuccess && rc == PG_OK) err = cudaEventElapsedTime(&ms, ev[0], ev[1]);
        out[k] = (double)ms / reps;
    }
    for (int k = 0; k < 2; ++k) {
        if (exec[k]) cudaGraphExecDestroy(exec[k]);
        if (graph[k]) cudaGraphDestroy(graph[k]);
    }
    if (cs) cudaStreamSynchronize(cs);
    for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
    if (cs) cudaStreamDestroy(cs);
    cudaFree(r);
    cudaFree(z);
    if (rc) return rc;
    if (err != cudaSuccess) return cuda_fail(err, "pg_debug_mg_vcycle_ms");
    *full_ms = out[0];
    *coarse_ms = out[1];
    return PG_OK;
}
