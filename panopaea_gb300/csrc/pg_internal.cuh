// pg_internal.cuh -- shared definitions of the sm_103a grid-fluid library.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "panopaea_gpu.h"

namespace pg {

typedef int64_t i64;

// Face-open bits of a cell for the Laplacian (interior and not solid).
enum : uint8_t { XLO = 1, XHI = 2, YLO = 4, YHI = 8, ZLO = 16, ZHI = 32 };

// Grid shape.  2D grids are stored with d = 1 and no z faces, so the face
// buffer is [vy (h+1)w | vx h(w+1)] exactly as dec/grid.rs:36-73; 3D grids
// prepend the vz part.
struct Dims {
    int nd;
    i64 d, h, w;
    __host__ __device__ i64 nc() const { return d * h * w; }
    __host__ __device__ i64 nfz() const { return nd == 3 ? (d + 1) * h * w : 0; }
    __host__ __device__ i64 nfy() const { return d * (h + 1) * w; }
    __host__ __device__ i64 nfx() const { return d * h * (w + 1); }
    __host__ __device__ i64 nf() const { return nfz() + nfy() + nfx(); }
    __host__ __device__ i64 offy() const { return nfz(); }
    __host__ __device__ i64 offx() const { return nfz() + nfy(); }
    __host__ __device__ i64 cell(i64 z, i64 y, i64 x) const { return (z * h + y) * w + x; }
    __host__ __device__ i64 fz(i64 z, i64 y, i64 x) const { return (z * h + y) * w + x; }
    __host__ __device__ i64 fy(i64 z, i64 y, i64 x) const { return offy() + (z * (h + 1) + y) * w + x; }
    __host__ __device__ i64 fx(i64 z, i64 y, i64 x) const { return offx() + (z * h + y) * (w + 1) + x; }
};

// ---------------------------------------------------------------------------
// Round-to-nearest arithmetic that the compiler may not fuse into FMA, so
// the operator kernels reproduce the reference's operation order exactly.
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
// x / 2 and x / 4 as multiplications by the exact reciprocals: both round
// the same real number, so the result is the IEEE quotient bit for bit, in
// one instruction instead of a division sequence.
template <class T> __device__ __forceinline__ T half_rn(T x) { return mul_rn(x, T(0.5)); }
template <class T> __device__ __forceinline__ T quarter_rn(T x) { return mul_rn(x, T(0.25)); }

// Index splitting by a divisor fixed for the launch: the quotient of a 32-bit
// n by d >= 2 with one multiply-high instead of an integer division sequence
// (Granlund and Montgomery, "Division by invariant integers using
// multiplication", 1994, the round-up method): l = ceil(log2 d),
// m = floor(2^32 (2^l - d) / d) + 1, t = umulhi(m, n),
// n / d = (t + ((n - t) >> 1)) >> (l - 1), exact for every 32-bit n.
// m >= 1 for every d >= 2; m = 0 stands for d = 1.
struct FastDiv {
    unsigned m = 0, s = 0;
};
inline FastDiv fast_div(unsigned d) {
    FastDiv f;
    if (d < 2) return f;
    unsigned l = 0;
    while ((1ull << l) < d) ++l;
    f.m = (unsigned)((((unsigned long long)1 << 32) * ((1ull << l) - d)) / d + 1);
    f.s = l - 1;
    return f;
}
__device__ __forceinline__ unsigned fdiv(unsigned n, FastDiv f) {
    const unsigned t = __umulhi(n, f.m);
    return f.m ? (t + ((n - t) >> 1)) >> f.s : n;
}
// (i / d, i % d) of a flat index; fd = fast_div(d), used when I is 32-bit
// (indices below 2^31).
template <class I> __device__ __forceinline__ I split(I i, I d, FastDiv fd, I& rem) {
    const I q = sizeof(I) == 4 ? (I)fdiv((unsigned)i, fd) : i / d;
    rem = i - q * d;
    return q;
}
// fast_div for a launch whose index type is I (nothing to do for 64-bit).
template <class I> inline FastDiv fast_div_for(i64 d) { return sizeof(I) == 4 ? fast_div((unsigned)d) : FastDiv{}; }

// math/interp.rs:7-12: a0*(1-s) + a1*s
template <class T> __device__ __forceinline__ T lerp_ref(T a0, T a1, T s) {
    return add_rn(mul_rn(a0, sub_rn(T(1), s)), mul_rn(a1, s));
}

// Symmetric red-black Gauss-Seidel sweep pairs of a multigrid coarsest
// level: Gauss-Seidel contracts the smoothest error by about 1 - c / s^2
// per sweep on a level whose longest side is s, so s^2 / 2 pairs (at least
// 4, at most 32) reduce it far below what the V-cycle needs.
__host__ __device__ inline int coarse_pairs(int d, int h, int w) {
    const int s = d > h ? (d > w ? d : w) : (h > w ? h : w);
    const int p = (s * s + 1) / 2;
    return p < 4 ? 4 : (p > 32 ? 32 : p);
}

// ---------------------------------------------------------------------------
// Block reductions in FP64 (deterministic for a fixed launch shape).
template <int NT> __device__ __forceinline__ double block_sum(double v, double* sm) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    v = (threadIdx.x < NT / 32) ? sm[threadIdx.x] : 0.0;
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;  // valid in thread 0
}

template <int NT> __device__ __forceinline__ double block_max(double v, double* sm) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    v = (threadIdx.x < NT / 32) ? sm[threadIdx.x] : 0.0;
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// ---------------------------------------------------------------------------
// Device-resident state of one CG run.  Written only by the last block of
// each reduction kernel; read by every block at kernel entry.
struct CgState {
    double sigma;      // z.r of the current search direction
    double pap;        // p.Ap
    double alpha, beta;
    double rmax;       // ||r||inf after the last update
    double bmax;       // ||b||inf
    double threshold;  // absolute stop threshold
    double rz_new;
    i64 iter;          // operator applications done
    i64 max_iter;
    // MG on one fluid component: z is used as z - mean(z) over the fluid
    // cells (the constant mode the coarse sweeps amplify), applied lazily
    double nfluid;     // fluid cells (0: no projection)
    double zmean;      // mean of the current z over the fluid cells
    double rsum;       // sum of the current residual
    int done;          // 1: stop issuing work
    int status;        // pg_status
    int first;         // next p-update is p = z
    int nan_seen;
    unsigned int counter[4];  // last-block tickets
};

// Host view of the workspace owned by a grid.
struct Workspace {
    double* partials = nullptr;  // per-block reduction partials (4 x kMaxBlocks: two reductions of two kernels)
    CgState* state = nullptr;    // device
    CgState* state_host = nullptr;  // pinned mirror (see ensure_workspace)
    void* vec = nullptr;         // extra CG vectors (lazily sized)
    size_t vec_bytes = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    void* graphs = nullptr;      // cached CG-loop graphs (pg_cg.cu)
};

constexpr int kMaxBlocks = 4096;

}  // namespace pg

struct pg_grid {
    pg::Dims dims;
    cudaStream_t stream = nullptr;
    int device = 0;
    int num_sms = 0;
    uint8_t* flags = nullptr;       // device, per cell: Laplacian face-open bits
    uint8_t* face_solid = nullptr;  // device, per face (1 = solid) or null
    unsigned long long mask_version = 0;  // bumped on every mask upload
    pg::Workspace ws;
    void* extras = nullptr;         // solver state owned by pg_solve.cu (MG levels, graphs)
};

namespace pg {

// Thread-local error text.
void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define PG_CUDA(call)                                              \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return ::pg::cuda_fail(e_, #call);  \
    } while (0)

#define PG_CHECK_LAUNCH() PG_CUDA(cudaGetLastError())

inline int bad_arg(const char* msg) {
    set_error(msg);
    return PG_BAD_ARG;
}

// Index type for per-element kernels: 32-bit when every face index fits.
inline bool idx32(const pg_grid* g) { return g->dims.nf() < ((i64)1 << 31); }
#define PG_IDX(g, ...)              \
    do {                            \
        if (::pg::idx32(g)) {       \
            typedef int I;          \
            __VA_ARGS__;            \
        } else {                    \
            typedef ::pg::i64 I;    \
            __VA_ARGS__;            \
        }                           \
    } while (0)

// Blocks for a grid-stride kernel over n items.
inline int grid_blocks(const pg_grid* g, i64 n, int threads, int per_sm = 8) {
    i64 b = (n + threads - 1) / threads;
    i64 cap = (i64)g->num_sms * per_sm;
    if (cap > kMaxBlocks) cap = kMaxBlocks;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

// Kernel kinds for launch counting and event timing (pg_prof.cu).
enum KernelKind {
    KK_CG_INIT, KK_CG_SPMV, KK_CG_UPDATE, KK_CG_TAIL, KK_ADVECT, KK_ADVECT_MAC, KK_RHS, KK_PROJECT, KK_DEC_OP,
    KK_RESIDUAL64, KK_REFINE_UPDATE, KK_MG_SMOOTH, KK_MG_RESTRICT, KK_MG_SMOOTH_C, KK_MG_RESTRICT_C, KK_MG_COARSE,
    KK_MG_SETUP, KK_STEP_MISC, KK_UNET_CONV, KK_UNET_WGRAD, KK_UNET_MISC, KK_MG_PAIR, KK_COUNT
};
void prof_begin(cudaStream_t s, int kind);
void prof_end(cudaStream_t s, int kind);
// Stream capture into a graph: launches are counted separately (as graph
// nodes) and get no timing events; graph executions add their kernels later.
int64_t prof_capture_begin();
int64_t prof_capture_end();
void prof_add_launches(int64_t n);
// Device-side graph loops are used unless per-kernel profiling is on or
// PG_NO_GRAPHS=1 is set in the environment.
bool graphs_enabled();
void release_cg_graphs(pg_grid* g);

// Every kernel launch of the library goes through this macro.
#define PG_LAUNCH(kind, stream, ...)        \
    do {                                    \
        ::pg::prof_begin((stream), (kind)); \
        __VA_ARGS__;                        \
        ::pg::prof_end((stream), (kind));   \
    } while (0)

// Disconnected fluid components (pg_pocket.cu): on grids with more than one,
// the cells of every component grouped by component and cut into chunks.
struct Pockets {
    int* cells = nullptr;
    int* start = nullptr;        // ncomp + 1 offsets into cells
    int* chunk_start = nullptr;  // nchunk + 1 offsets into cells
    int* chunk_comp = nullptr;   // component of each chunk
    int* comp_chunk = nullptr;   // ncomp + 1 offsets into the chunks
    double* partials = nullptr;  // nchunk partial sums, then ncomp means
    int ncomp = 0, nchunk = 0;
};
void find_pockets(const uint8_t* flags, int nd, i64 d, i64 h, i64 w, i64 base, std::vector<i64>& cells,
                  std::vector<int>& start);
int upload_pockets(const std::vector<i64>& cells, const std::vector<int>& start, Pockets* pk);
void release_pockets(Pockets* pk);
// a -= its mean over each component (stream-ordered; nothing for connected fluid)
void pocket_project(cudaStream_t s, float* a, const Pockets& pk);

int ensure_workspace(pg_grid* g);

// Small results for the host are written into pinned host memory by a
// one-block kernel at the end of the stream's work instead of copied by the
// copy engine, whose queue may hold a caller's large transfers on other
// streams.
__global__ void k_words_out(const unsigned* __restrict__ src, unsigned* dst, int nwords);
inline double* host_scalar(Workspace& ws) { return (double*)(ws.state_host + 3); }
void release_extras(pg_grid* g);
int ensure_vec(pg_grid* g, size_t bytes);

}  // namespace pg
