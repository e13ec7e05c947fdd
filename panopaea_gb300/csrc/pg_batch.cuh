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
