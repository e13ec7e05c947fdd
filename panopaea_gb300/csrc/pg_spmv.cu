// pg_spmv.cu -- TMA-staged z-marching kernels of the 3D solve: the fused
// SpMV of the CG (p = z + beta p, Ap, p.Ap; pcg.rs:52-53, 77 with the
// masked Laplacian of grid.rs) for every preconditioner, and the
// double-float residual b - A x of the refinement.
//
// A block owns a kSX x kSY column tile and walks a chunk of z planes.  TMA
// stages every plane of the source vector and p_old (one-cell halo) and of
// the face flags (tile and halo) into a kSStages-deep shared-memory ring; for
// plane q+1 the block computes p_new = z + beta p_old on the tile and its
// one-cell ring into a 4-slot plane ring (and stores the tile's values), then
// A p_new of plane q from the slots of planes q-1, q and q+1.  A staged plane
// is free as soon as its p_new and its flags have been used, so most of the
// ring is in flight.  Per cell: 4 bytes of the source, 4 of p_old, 1 of flags
// in; 4 of p_new and 4 of Ap out.  The source is z itself (multigrid writes
// it), or r with z = r (identity, pcg.rs:8-12) or z = r / diag computed from
// the staged flags once per cell and plane (Jacobi).  Same per-cell
// arithmetic as k_cg_spmv3t<float, PM> (the p.Ap reduction runs in a
// different order).
#include <mutex>

#include "pg_cg.cuh"
#include "pg_tma.cuh"

namespace pg {

namespace {

constexpr int kSX = 64, kSWarps = 8, kSRows = 2, kSY = kSWarps * kSRows;
constexpr int kSThreads = 32 * kSWarps;
constexpr int kSStages = 7;
constexpr int kSVw = kSX + 8, kSVh = kSY + 2;  // z / p_old boxes from (x0 - 4, y0 - 1)
constexpr int kSGw = kSX + 32, kSGh = kSY + 2;  // flags box from (x0 - 16, y0 - 1)
constexpr int kSVBytes = kSVw * kSVh * 4;
constexpr int kSGBytes = kSGw * kSGh;
constexpr int kSVPad = ((kSVBytes + 127) / 128) * 128;
constexpr int kSPOff = kSVPad, kSGOff = 2 * kSVPad;
constexpr int kSStageBytes = kSGOff + ((kSGBytes + 127) / 128) * 128;
constexpr int kSSw = kSX + 2, kSSh = kSY + 2;  // p_new of one plane (tile + ring)
constexpr int kSSlotBytes = kSSw * kSSh * 4;
constexpr int kSBarOff = kSStages * kSStageBytes + 4 * kSSlotBytes;
constexpr size_t kSSmem = 128 + kSBarOff + kSStages * 8;
constexpr unsigned kSTx = 2 * kSVBytes + kSGBytes;
static_assert(kSStageBytes % 128 == 0, "TMA boxes must stay 128-byte aligned");

struct SpmvArgs {
    int d, h, w;
    float dt;
    float* p0;
    float* p1;
    float* ap;
    int tiles_x, tiles_y;
};

template <int PM>
__global__ void __launch_bounds__(kSThreads, 2)
    k_cg_spmv3p(const __grid_constant__ CUtensorMap zmap, const __grid_constant__ CUtensorMap pmap0,
                const __grid_constant__ CUtensorMap pmap1, const __grid_constant__ CUtensorMap gmap, SpmvArgs a,
                CgState* st, double* partials) {
    if (st->done) return;
    extern __shared__ unsigned char spmv_smem_raw[];
    __shared__ double sm[32];
    unsigned char* const base = spmv_smem_raw + ((128u - (smem_u32(spmv_smem_raw) & 127u)) & 127u);
    float(*const S)[kSSh][kSSw] = (float(*)[kSSh][kSSw])(base + kSStages * kSStageBytes);
    uint64_t* const bars = (uint64_t*)(base + kSBarOff);
    const int tid = threadIdx.x, lane = tid & 31, ty = tid >> 5;
    const i64 kit = *(volatile const i64*)&st->iter;
    const CUtensorMap* pmap = (kit & 1) ? &pmap1 : &pmap0;  // p_old
    float* const p_new = (kit & 1) ? a.p0 : a.p1;
    const int first = st->first;
    const float beta = first ? 0.f : (float)st->beta;
    // Jacobi: 1 / (n dt) for n open faces, computed as in zval (0 for n = 0)
    __shared__ float inv_diag[8];
    if (PM == PM_JACOBI && tid < 8) inv_diag[tid] = tid ? __frcp_rn((float)tid * a.dt) : 0.f;
    if (tid == 0) {
        for (int s = 0; s < kSStages; ++s) mbar_init(&bars[s], 1);
        mbar_fence_init();
        tma_prefetch_map(&zmap);
        tma_prefetch_map(pmap);
        tma_prefetch_map(&gmap);
    }
    __syncthreads();
    const float dt = a.dt;
    const int h = a.h, w = a.w, d = a.d;
    const int per_plane = a.tiles_x * a.tiles_y;
    auto stage = [&](unsigned j) -> const unsigned char* { return base + (j % kSStages) * kSStageBytes; };
    auto Zv = [](const unsigned char* P, int r, int c) -> float { return ((const float*)P)[r * kSVw + c]; };
    auto Pv = [](const unsigned char* P, int r, int c) -> float {
        return ((const float*)(P + kSPOff))[r * kSVw + c];
    };
    auto Gv = [](const unsigned char* P, int r, int c) -> unsigned { return (P + kSGOff)[r * kSGw + c]; };
    unsigned issued_end = 0;
    auto issue = [&](unsigned j, int plane, int x0, int y0) {
        issued_end = j + 1;
        unsigned char* dst = base + (j % kSStages) * kSStageBytes;
        uint64_t* bar = &bars[j % kSStages];
        mbar_expect_tx(bar, kSTx);
        tma_load_3d(dst, &zmap, bar, x0 - 4, y0 - 1, plane);
        tma_load_3d(dst + kSPOff, pmap, bar, x0 - 4, y0 - 1, plane);
        tma_load_3d(dst + kSGOff, &gmap, bar, x0 - 16, y0 - 1, plane);
    };
    bool ok = true;
    auto wait = [&](unsigned j) {
        if (tid == 0 && ok) ok = mbar_wait(&bars[j % kSStages], (j / kSStages) & 1);
    };
    // p_new of cell (yl, xl) of the staged plane P (tile coordinates), with
    // z projected lazily on the fluid cells (zm = 0 when off)
    const float zm = (PM == PM_ZBUF && st->nfluid > 0.0) ? (float)st->zmean : 0.f;
    auto pn = [&](const unsigned char* P, int yl, int xl) -> float {
        const float z0 = Zv(P, yl + 1, xl + 4);
        float z = z0;
        if (PM == PM_ZBUF) {
            z = Gv(P, yl + 1, xl + 16) ? z0 - zm : z0;
        } else if (PM == PM_JACOBI) {
            const unsigned f = Gv(P, yl + 1, xl + 16);
            z = f ? z0 * inv_diag[__popc(f)] : 0.f;
        }
        return first ? z : fmaf(beta, Pv(P, yl + 1, xl + 4), z);
    };
    unsigned seq = 0;
    bool failed = false;
    Acc<float> acc;
    ZWalk walk(per_plane, d);
    int t2, z0, z1;
    while (!failed && walk.next(t2, z0, z1)) {
        const int x0 = (t2 % a.tiles_x) * kSX, y0 = (t2 / a.tiles_x) * kSY;
        const int n = z1 - z0 + 2;  // planes z0 - 1 .. z1 (ring index j = plane - z0 + 1)
        if (tid == 0)
            for (int j = 0; j < min(n, kSStages); ++j) issue(seq + j, z0 - 1 + j, x0, y0);
        // p_new of plane x (tile and ring) into its slot; the tile's values
        // are stored when x is one of this chunk's planes
        auto fill = [&](const unsigned char* P, int x) {
            float(*const D)[kSSw] = S[x & 3];
#pragma unroll
            for (int r = 0; r < kSRows; ++r) {
                const int yl = ty + r * kSWarps, xl = 2 * lane;
                const float v0 = pn(P, yl, xl), v1 = pn(P, yl, xl + 1);
                D[yl + 1][xl + 1] = v0;
                D[yl + 1][xl + 2] = v1;
                const int gy = y0 + yl, gx = x0 + xl;
                if (x >= z0 && x < z1 && gy < h && gx < w)
                    *(float2*)(p_new + ((i64)x * h + gy) * w + gx) = make_float2(v0, v1);
            }
            if (tid < 64) {  // ring rows y0 - 1 and y0 + kSY
                const int yl = tid < 32 ? -1 : kSY, xl = 2 * lane;
                D[yl + 1][xl + 1] = pn(P, yl, xl);
                D[yl + 1][xl + 2] = pn(P, yl, xl + 1);
            } else if (tid < 64 + 2 * kSY) {  // ring columns x0 - 1 and x0 + kSX
                const int k = tid - 64;
                const int xl = k < kSY ? -1 : kSX, yl = k < kSY ? k : k - kSY;
                D[yl + 1][xl + 1] = pn(P, yl, xl);
            }
        };
        wait(seq);
        wait(seq + 1);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        fill(stage(seq), z0 - 1);
        for (int i = 0; i <= z1 - z0; ++i) {
            const int q = z0 - 1 + i;  // Ap of plane q after p_new of plane q + 1
            fill(stage(seq + i + 1), q + 1);
            if (i + 2 < n) wait(seq + i + 2);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            // plane q - 1's stage has served its p_new and its flags
            if (tid == 0 && i >= 1 && i - 1 + kSStages < n) issue(seq + i - 1 + kSStages, z0 - 2 + i + kSStages, x0, y0);
            if (i >= 1) {
                const unsigned char* P = stage(seq + i);
#pragma unroll
                for (int r = 0; r < kSRows; ++r) {
                    const int yl = ty + r * kSWarps, gy = y0 + yl;
                    float out[2];
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const int xl = 2 * lane + u;
                        const unsigned f = Gv(P, yl + 1, xl + 16);
                        const float pc = S[q & 3][yl + 1][xl + 1];
                        const float gy_lo = (f & YLO) ? -sub_rn(pc, S[q & 3][yl][xl + 1]) : 0.f;
                        const float gy_hi = (f & YHI) ? -sub_rn(S[q & 3][yl + 2][xl + 1], pc) : 0.f;
                        const float gx_lo = (f & XLO) ? sub_rn(S[q & 3][yl + 1][xl], pc) : 0.f;
                        const float gx_hi = (f & XHI) ? sub_rn(pc, S[q & 3][yl + 1][xl + 2]) : 0.f;
                        float v = add_rn(sub_rn(sub_rn(gy_hi, gy_lo), gx_lo), gx_hi);
                        const float gz_lo = (f & ZLO) ? -sub_rn(pc, S[(q - 1) & 3][yl + 1][xl + 1]) : 0.f;
                        const float gz_hi = (f & ZHI) ? -sub_rn(S[(q + 1) & 3][yl + 1][xl + 1], pc) : 0.f;
                        v = add_rn(sub_rn(v, gz_lo), gz_hi);
                        out[u] = mul_rn(v, dt);
                    }
                    const int gx = x0 + 2 * lane;
                    if (gy < h && gx < w) {
                        *(float2*)(a.ap + ((i64)q * h + gy) * w + gx) = make_float2(out[0], out[1]);
                        acc.add(S[q & 3][yl + 1][2 * lane + 1] * out[0]);
                        acc.add(S[q & 3][yl + 1][2 * lane + 2] * out[1]);
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
            for (unsigned j = issued_end > kSStages ? issued_end - kSStages : 0; j < issued_end; ++j)
                while (!mbar_try_wait(&bars[j % kSStages], (j / kSStages) & 1) && global_ns() - t0 < kMbarWaitNs) {
                }
            st->status = PG_TIMEOUT;
            st->done = 1;
        }
        return;
    }
    const double s = block_sum<kSThreads>(acc.value(), sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    if (!last_block(&st->counter[1])) return;
    const double pap = reduce_partials<false, kSThreads>(partials, gridDim.x, sm);
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

// ---------------------------------------------------------------------------
// Double-float residual r = b - A (xh + xl), ||r||inf (the refinement's outer
// residual).  Stages per plane: xh and xl with a one-cell halo, b and the
// flags on the tile; plane p's residual reads the stages of planes p-1, p,
// p+1 (its z neighbours are the halo boxes' centres), so a stage is refilled
// once plane p+1 is done with it.  Same arithmetic as k_residual_df3t.
constexpr int kRX = 64, kRWarps = 8, kRRows = 2, kRY = kRWarps * kRRows;
constexpr int kRThreads = 32 * kRWarps;
constexpr int kRStages = 6;
constexpr int kRVw = kRX + 8, kRVh = kRY + 2;  // xh / xl boxes from (x0 - 4, y0 - 1)
constexpr int kRBw = kRX, kRBh = kRY;          // b box from (x0, y0)
constexpr int kRGw = kRX + 32, kRGh = kRY;     // flags box from (x0 - 16, y0)
constexpr int kRVBytes = kRVw * kRVh * 4, kRBBytes = kRBw * kRBh * 4, kRGBytes = kRGw * kRGh;
constexpr int kRVPad = ((kRVBytes + 127) / 128) * 128;
constexpr int kRLOff = kRVPad, kRBOff = 2 * kRVPad, kRGOff = kRBOff + ((kRBBytes + 127) / 128) * 128;
constexpr int kRStageBytes = kRGOff + ((kRGBytes + 127) / 128) * 128;
constexpr int kRBarOff = kRStages * kRStageBytes;
constexpr size_t kRSmem = 128 + kRBarOff + kRStages * 8;
constexpr unsigned kRTx = 2 * kRVBytes + kRBBytes + kRGBytes;
static_assert(kRStageBytes % 128 == 0, "TMA boxes must stay 128-byte aligned");

__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

struct ResArgs {
    int d, h, w;
    float dt;
    float* r;
    int tiles_x, tiles_y;
};

__global__ void __launch_bounds__(kRThreads, 2)
    k_residual_df3p(const __grid_constant__ CUtensorMap hmap, const __grid_constant__ CUtensorMap lmap,
                    const __grid_constant__ CUtensorMap bmap, const __grid_constant__ CUtensorMap gmap, ResArgs a,
                    double* partials, unsigned int* counter, double* out, CgState* st) {
    extern __shared__ unsigned char res_smem_raw[];
    __shared__ double sm[32];
    unsigned char* const base = res_smem_raw + ((128u - (smem_u32(res_smem_raw) & 127u)) & 127u);
    uint64_t* const bars = (uint64_t*)(base + kRBarOff);
    const int tid = threadIdx.x, lane = tid & 31, ty = tid >> 5;
    if (tid == 0) {
        for (int s = 0; s < kRStages; ++s) mbar_init(&bars[s], 1);
        mbar_fence_init();
        tma_prefetch_map(&hmap);
        tma_prefetch_map(&lmap);
        tma_prefetch_map(&bmap);
        tma_prefetch_map(&gmap);
    }
    __syncthreads();
    const float dt = a.dt;
    const int h = a.h, w = a.w, d = a.d;
    const int per_plane = a.tiles_x * a.tiles_y;
    auto stage = [&](unsigned j) -> const unsigned char* { return base + (j % kRStages) * kRStageBytes; };
    auto H = [](const unsigned char* P, int r, int c) -> float { return ((const float*)P)[r * kRVw + c]; };
    auto L = [](const unsigned char* P, int r, int c) -> float { return ((const float*)(P + kRLOff))[r * kRVw + c]; };
    auto Bv = [](const unsigned char* P, int r, int c) -> float { return ((const float*)(P + kRBOff))[r * kRBw + c]; };
    auto Gv = [](const unsigned char* P, int r, int c) -> unsigned { return (P + kRGOff)[r * kRGw + c]; };
    unsigned issued_end = 0;
    auto issue = [&](unsigned j, int plane, int x0, int y0) {
        issued_end = j + 1;
        unsigned char* dst = base + (j % kRStages) * kRStageBytes;
        uint64_t* bar = &bars[j % kRStages];
        mbar_expect_tx(bar, kRTx);
        tma_load_3d(dst, &hmap, bar, x0 - 4, y0 - 1, plane);
        tma_load_3d(dst + kRLOff, &lmap, bar, x0 - 4, y0 - 1, plane);
        tma_load_3d(dst + kRBOff, &bmap, bar, x0, y0, plane);
        tma_load_3d(dst + kRGOff, &gmap, bar, x0 - 16, y0, plane);
    };
    bool ok = true;
    auto wait = [&](unsigned j) {
        if (tid == 0 && ok) ok = mbar_wait(&bars[j % kRStages], (j / kRStages) & 1);
    };
    unsigned seq = 0;
    bool failed = false;
    float m = 0.f;
    ZWalk walk(per_plane, d);
    int t2, z0, z1;
    while (!failed && walk.next(t2, z0, z1)) {
        const int x0 = (t2 % a.tiles_x) * kRX, y0 = (t2 / a.tiles_x) * kRY;
        const int n = z1 - z0 + 2;  // planes z0 - 1 .. z1 (ring index j = plane - z0 + 1)
        if (tid == 0)
            for (int j = 0; j < min(n, kRStages); ++j) issue(seq + j, z0 - 1 + j, x0, y0);
        wait(seq);
        wait(seq + 1);
        wait(seq + 2);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        for (int i = 0; i < z1 - z0; ++i) {
            const int p = z0 + i;
            const unsigned char *Pm = stage(seq + i), *P0 = stage(seq + i + 1), *Pp = stage(seq + i + 2);
#pragma unroll
            for (int rr = 0; rr < kRRows; ++rr) {
                const int yl = ty + rr * kRWarps, gy = y0 + yl;
                float out2[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int xl = 2 * lane + u;
                    const unsigned f = Gv(P0, yl, xl + 16);
                    const float ch = H(P0, yl + 1, xl + 4), cl = L(P0, yl + 1, xl + 4);
                    float sh = 0.f, sl = 0.f;
                    auto face = [&](float nh, float nl) {
                        float dh, de, t, te;
                        df_two_sum(ch, -nh, dh, de);
                        df_two_sum(sh, dh, t, te);
                        sh = t;
                        sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(te, de), __fsub_rn(cl, nl)));
                    };
                    if (f & XLO) face(H(P0, yl + 1, xl + 3), L(P0, yl + 1, xl + 3));
                    if (f & XHI) face(H(P0, yl + 1, xl + 5), L(P0, yl + 1, xl + 5));
                    if (f & YLO) face(H(P0, yl, xl + 4), L(P0, yl, xl + 4));
                    if (f & YHI) face(H(P0, yl + 2, xl + 4), L(P0, yl + 2, xl + 4));
                    if (f & ZLO) face(H(Pm, yl + 1, xl + 4), L(Pm, yl + 1, xl + 4));
                    if (f & ZHI) face(H(Pp, yl + 1, xl + 4), L(Pp, yl + 1, xl + 4));
                    const float ph = __fmul_rn(dt, sh);
                    const float pl = __fadd_rn(__fmaf_rn(dt, sh, -ph), __fmul_rn(dt, sl));
                    float rh, re;
                    df_two_sum(Bv(P0, yl, xl), -ph, rh, re);
                    out2[u] = __fadd_rn(rh, __fsub_rn(re, pl));
                }
                const int gx = x0 + 2 * lane;
                if (gy < h && gx < w) {
                    *(float2*)(a.r + ((i64)p * h + gy) * w + gx) = make_float2(out2[0], out2[1]);
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        m = fmaxf(m, fabsf(out2[u]));
                        if (out2[u] != out2[u]) m = __int_as_float(0x7f800000);
                    }
                }
            }
            if (i + 3 < n) wait(seq + i + 3);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            // plane p - 1's stage has served its last z neighbour
            if (tid == 0 && i + kRStages < n) issue(seq + i + kRStages, z0 - 1 + i + kRStages, x0, y0);
        }
        if (failed) break;
        __syncthreads();
        seq += n;
    }
    if (failed) {  // a plane never arrived: drain the copies in flight (bounded), report NaN
        if (tid == 0) {
            const uint64_t t0 = global_ns();
            for (unsigned j = issued_end > kRStages ? issued_end - kRStages : 0; j < issued_end; ++j)
                while (!mbar_try_wait(&bars[j % kRStages], (j / kRStages) & 1) && global_ns() - t0 < kMbarWaitNs) {
                }
            st->status = PG_TIMEOUT;
        }
        m = __int_as_float(0x7fc00000);
    }
    const double bm = block_max<kRThreads>((double)m, sm);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bm;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    double v = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) v = fmax(v, __ldcg(partials + i));
    v = block_max<kRThreads>(v, sm);
    if (threadIdx.x == 0) {
        *out = v;
        *counter = 0;
    }
}

// Tensor maps by (pointer, element size, box), shared by every grid.
struct MapCache {
    std::mutex m;
    struct E {
        const void* p = nullptr;
        Dims D{};
        int elem = 0, bx = 0, by = 0;
        CUtensorMap map;
    } e[16];
    int next = 0;
};

MapCache& map_cache() {
    static MapCache c;
    return c;
}

bool cached_map(const void* p, int elem, const Dims& D, int bx, int by, CUtensorMap* out) {
    MapCache& c = map_cache();
    std::lock_guard<std::mutex> lk(c.m);
    for (auto& e : c.e)
        if (e.p == p && e.elem == elem && e.bx == bx && e.by == by && e.D.d == D.d && e.D.h == D.h && e.D.w == D.w) {
            *out = e.map;
            return true;
        }
    MapCache::E& e = c.e[c.next];
    if (!encode_map_3d(&e.map, p, elem, D.w, D.h, D.d, bx, by)) return false;
    c.next = (c.next + 1) % 16;
    e.p = p;
    e.D = D;
    e.elem = elem;
    e.bx = bx;
    e.by = by;
    *out = e.map;
    return true;
}

template <int PM> static int spmv_cap(int num_sms) {
    static int cap = -1;
    if (cap < 0) {
        cap = 0;
        if (cudaFuncSetAttribute(k_cg_spmv3p<PM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSSmem) ==
            cudaSuccess) {
            int bps = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_cg_spmv3p<PM>, kSThreads, kSSmem) ==
                cudaSuccess)
                cap = std::min(bps * num_sms, kMaxBlocks);
        }
        cudaGetLastError();
    }
    return cap;
}

}  // namespace

int set_stage_wait_polls_spmv(unsigned polls) {
    PG_CUDA(cudaMemcpyToSymbol(c_stage_wait_polls, &polls, sizeof(polls)));
    return PG_OK;
}

bool spmv_tma_launch(cudaStream_t s, int num_sms, int pm, const float* zb, float* p0, float* p1, float* ap,
                     const uint8_t* flags, const Dims& D, float dt, CgState* st, double* partials) {
    if (pm != PM_NONE && pm != PM_JACOBI && pm != PM_ZBUF) return false;
    const int cap = pm == PM_ZBUF ? spmv_cap<PM_ZBUF>(num_sms)
                                  : (pm == PM_JACOBI ? spmv_cap<PM_JACOBI>(num_sms) : spmv_cap<PM_NONE>(num_sms));
    if (cap <= 0 || D.nd != 3 || D.w % 16 != 0 || D.nc() >= ((i64)1 << 31)) return false;
    if (((uintptr_t)ap & 7) || ((uintptr_t)p0 & 7) || ((uintptr_t)p1 & 7)) return false;
    CUtensorMap zm, pm0, pm1, gm;
    if (!cached_map(zb, 4, D, kSVw, kSVh, &zm) || !cached_map(p0, 4, D, kSVw, kSVh, &pm0) ||
        !cached_map(p1, 4, D, kSVw, kSVh, &pm1) || !cached_map(flags, 1, D, kSGw, kSGh, &gm))
        return false;
    SpmvArgs a;
    a.d = (int)D.d;
    a.h = (int)D.h;
    a.w = (int)D.w;
    a.dt = dt;
    a.p0 = p0;
    a.p1 = p1;
    a.ap = ap;
    a.tiles_x = (a.w + kSX - 1) / kSX;
    a.tiles_y = (a.h + kSY - 1) / kSY;
    const int nb = zwalk_blocks(a.tiles_x * a.tiles_y, a.d, cap);
    if (pm == PM_ZBUF)
        k_cg_spmv3p<PM_ZBUF><<<nb, kSThreads, kSSmem, s>>>(zm, pm0, pm1, gm, a, st, partials);
    else if (pm == PM_JACOBI)
        k_cg_spmv3p<PM_JACOBI><<<nb, kSThreads, kSSmem, s>>>(zm, pm0, pm1, gm, a, st, partials);
    else
        k_cg_spmv3p<PM_NONE><<<nb, kSThreads, kSSmem, s>>>(zm, pm0, pm1, gm, a, st, partials);
    return true;
}

bool residual_df_tma_launch(cudaStream_t s, int num_sms, const float* b, const float* xh, const float* xl,
                            const uint8_t* flags, const Dims& D, float dt, float* r, double* partials,
                            unsigned int* counter, double* out, CgState* st) {
    static int cap = -1;
    if (cap < 0) {
        cap = 0;
        if (cudaFuncSetAttribute(k_residual_df3p, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRSmem) ==
            cudaSuccess) {
            int bps = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_residual_df3p, kRThreads, kRSmem) == cudaSuccess)
                cap = std::min(bps * num_sms, kMaxBlocks);
        }
        cudaGetLastError();
    }
    if (cap <= 0 || D.nd != 3 || D.w % 16 != 0 || D.nc() >= ((i64)1 << 31) || ((uintptr_t)r & 7)) return false;
    CUtensorMap hm, lm, bm, gm;
    if (!cached_map(xh, 4, D, kRVw, kRVh, &hm) || !cached_map(xl, 4, D, kRVw, kRVh, &lm) ||
        !cached_map(b, 4, D, kRBw, kRBh, &bm) || !cached_map(flags, 1, D, kRGw, kRGh, &gm))
        return false;
    ResArgs a;
    a.d = (int)D.d;
    a.h = (int)D.h;
    a.w = (int)D.w;
    a.dt = dt;
    a.r = r;
    a.tiles_x = (a.w + kRX - 1) / kRX;
    a.tiles_y = (a.h + kRY - 1) / kRY;
    const int nb = zwalk_blocks(a.tiles_x * a.tiles_y, a.d, cap);
    k_residual_df3p<<<nb, kRThreads, kRSmem, s>>>(hm, lm, bm, gm, a, partials, counter, out, st);
    return true;
}

}  // namespace pg
