// pg_batch.cuh -- shared definitions of the batched 2D grids (pg_batch.cu)
// and their batched multigrid preconditioner (pg_batch_mg.cu).
#pragma once
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "pg_cg.cuh"
#include "pg_ops2d.cuh"

namespace pg {

struct GInfo {
    int h, w;
    i64 coff, foff;     // first cell / first face of the grid in the packed fields
    int t0, t1;         // cell-tile range [t0, t1)
    float hix, hiy;     // n - 1.00001 rounded to float, per axis (advect clamp)
};

struct Tile {
    int grid, y0, x0;
};

struct BState {
    double sigma, pap, alpha, beta, rmax, bmax, thr;
    // MG: z is used as z - zmean on the grid's fluid cells (lazy projection
    // of the constant mode; nfluid = 0: off), rsum = sum of the residual
    double nfluid, zmean, rsum;
    // alpha, beta and the applied zmean rounded to float, as every cell
    // uses them (written by the per-grid finalisers)
    float falpha, fbeta, fzm;
    int iter, max_iter, done, status, first, nan_seen;
};

struct BatchMg;

}  // namespace pg

struct pg_batch {
    int n = 0;
    std::vector<int> h, w;
    std::vector<pg::i64> coff, foff;  // n + 1 entries
    pg::i64 ncells = 0, nfaces = 0;
    cudaStream_t stream = nullptr;
    int device = 0, num_sms = 0;
    // device data
    pg::GInfo* ginfo = nullptr;
    uint8_t* flags = nullptr;       // packed cells: face-open bits
    uint8_t* face_solid = nullptr;  // packed faces (optional)
    pg::BState* state = nullptr;
    int* active = nullptr;          // grids still iterating (written by the finaliser)
    double* partials = nullptr;     // 2 per tile
    double* nfluid = nullptr;       // per grid: cells with an open face
    float *r = nullptr, *ap = nullptr, *p0 = nullptr, *p1 = nullptr, *b = nullptr, *tmp = nullptr;
    float* vtmp = nullptr;
    // tiling (cells) -- extended tiles cover the (h+1) x (w+1) face index box
    int tx = 32, ty = 8, fused = 1;
    int ntiles = 0, ntiles_ext = 0;
    pg::Tile* tiles = nullptr;
    pg::Tile* tiles_ext = nullptr;
    std::vector<pg::GInfo> host_info;
    // graph of the CG loop
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_tx = 0, graph_ty = 0, graph_fused = -1, graph_pm = -1;
    float graph_dt = 0.f;
    float* graph_x = nullptr;
    uint64_t graph_mg = 0;
    // batched multigrid (PG_PRECOND_MG)
    unsigned long long mask_version = 0;  // bumped by pg_batch_set_solid_cells
    pg::BatchMg* mg = nullptr;
    float* z = nullptr;  // preconditioned residual, packed cells
};

namespace pg {

constexpr int kBMaxThreads = 256;

// Block reductions for a runtime block size (a multiple of 32, <= 256).
__device__ __forceinline__ double bsum(double v, double* sm) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    v = (threadIdx.x < nw) ? sm[threadIdx.x] : 0.0;
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double bmaxr(double v, double* sm) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    v = (threadIdx.x < nw) ? sm[threadIdx.x] : 0.0;
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Per-tile block reductions in FP32 arithmetic alone.  They run once per
// tile (a few hundred cells) and GB300 executes FP64 at a small fraction of
// its FP32 rate, so a double-precision shuffle tree would dominate the
// kernels.  A sum travels as a double-float pair (hi + lo, about 44
// significant bits), two pairs added by TwoSum on the high parts with the
// low parts and the rounding error folded in; a maximum is exact in FP32.
// The block's result is a double in thread 0 only.
struct F2 {
    float hi, lo;
};

__device__ __forceinline__ F2 f2_of(const Acc<float>& a) { return F2{a.s, -a.c}; }

__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float v = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v)), __fadd_rn(a.lo, b.lo));
    const float h = __fadd_rn(s, e);
    return F2{h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ F2 f2_warp(F2 v) {
    for (int o = 16; o > 0; o >>= 1)
        v = f2_add(v, F2{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)});
    return v;
}

// sm: 32 pairs.
__device__ __forceinline__ double tsum(F2 v, F2* sm) {
    v = f2_warp(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    double out = 0.0;
    if (wid == 0) {
        v = f2_warp(lane < nw ? sm[lane] : F2{0.f, 0.f});
        if (lane == 0) out = (double)v.hi + (double)v.lo;
    }
    return out;
}

// Two sums in one pass (sm: 64 pairs).
__device__ __forceinline__ void tsum2(F2 a, F2 b, F2* sm, double* oa, double* ob) {
    a = f2_warp(a);
    b = f2_warp(b);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) {
        sm[wid] = a;
        sm[32 + wid] = b;
    }
    __syncthreads();
    *oa = *ob = 0.0;
    if (wid == 0) {
        a = f2_warp(lane < nw ? sm[lane] : F2{0.f, 0.f});
        b = f2_warp(lane < nw ? sm[32 + lane] : F2{0.f, 0.f});
        if (lane == 0) {
            *oa = (double)a.hi + (double)a.lo;
            *ob = (double)b.hi + (double)b.lo;
        }
    }
}

// Maximum and sum in one pass (sm: 64 pairs).
__device__ __forceinline__ void tmaxsum(float m, F2 v, F2* sm, double* om, double* os) {
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    v = f2_warp(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float* smm = reinterpret_cast<float*>(sm + 32);
    __syncthreads();
    if (lane == 0) {
        sm[wid] = v;
        smm[wid] = m;
    }
    __syncthreads();
    *om = *os = 0.0;
    if (wid == 0) {
        m = lane < nw ? smm[lane] : 0.f;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        v = f2_warp(lane < nw ? sm[lane] : F2{0.f, 0.f});
        if (lane == 0) {
            *om = (double)m;
            *os = (double)v.hi + (double)v.lo;
        }
    }
}

#define FOR_TILES(list, count) for (int ti = blockIdx.x; ti < (count); ti += gridDim.x)

// Batched multigrid (pg_batch_mg.cu).
// (Re)build the hierarchy of every grid for the batch's mask and dt.
int bmg_ensure(pg_batch* B, float dt);
// Enqueue z = V(r) for every grid still iterating; the last fine
// half-sweep writes per-tile z.r partials.
void bmg_vcycle(pg_batch* B, cudaStream_t s, int nsmooth);
// Fold the z.r partials per grid: first = 1 sets sigma; else beta and sigma.
void bmg_rz_finalize(pg_batch* B, cudaStream_t s, int first);
uint64_t bmg_id(const pg_batch* B);
void bmg_release(pg_batch* B);

}  // namespace pg
