// pg_cg.cuh -- the CG engine shared by pg_pcg_* and the pressure solver.
#pragma once
#include "pg_internal.cuh"

namespace pg {

// How z = M^-1 r is obtained inside the CG kernels.
enum PrecMode { PM_NONE = 0, PM_JACOBI = 1, PM_ZBUF = 2 /* z stored by an outer preconditioner (MG) */ };

// Buffers of one CG run.  p[0], p[1] ping-pong: the SpMV of iteration k
// reads p[k & 1] and writes p[(k + 1) & 1], so the search direction of the
// latest iteration is p[iter & 1].
template <class T> struct CgBuffers {
    T* x;
    const T* b;
    T* r;
    T* ap;
    T* p[2];
    T* z = nullptr;   // PM_ZBUF only
    T* xl = nullptr;  // PM_ZBUF, float, n % 4 == 0: x held as the double-float pair (x, xl)
                      // and started from 0 (see run_cg_pm)
};

struct CgConfig {
    int precond;        // PG_PRECOND_NONE / JACOBI / MG
    i64 max_iter;
    double threshold;   // absolute: stop when ||r||inf < threshold
    double rel_tol;     // > 0: threshold = rel_tol * ||b||inf (set on device)
    double dt;
    int check_every;    // 0 = auto
    int zero_x;         // 1: x = 0 first (pcg.rs:32)
    double nfluid = 0;  // MG on one fluid component: fluid cells (lazy projection of z); 0 = off
};

// Per-thread partial sums: compensated FP32 (float fields) or plain FP64
// (double fields); the cross-thread/-block tree is FP64 in both cases.
template <class T> struct Acc;
template <> struct Acc<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};
template <> struct Acc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double v) { s += v; }
    __device__ __forceinline__ double value() const { return s; }
};

// The fused SpMV on 3D float grids, TMA-staged (pg_spmv.cu), for the
// preconditioner mode pm (PrecMode): src is z (PM_ZBUF) or r (PM_NONE,
// PM_JACOBI).  False when it does not apply (2D, rows not a multiple of 16
// cells, a vector that cannot be mapped) and nothing was launched.
bool spmv_tma_launch(cudaStream_t s, int num_sms, int pm, const float* src, float* p0, float* p1, float* ap,
                     const uint8_t* flags, const Dims& D, float dt, CgState* st, double* partials);

// The double-float residual r = b - A (xh + xl) and ||r||inf (to *out) of the
// refinement on 3D grids, TMA-staged (pg_spmv.cu); false when it does not
// apply and nothing was launched.
bool residual_df_tma_launch(cudaStream_t s, int num_sms, const float* b, const float* xh, const float* xl,
                            const uint8_t* flags, const Dims& D, float dt, float* r, double* partials,
                            unsigned int* counter, double* out, CgState* st);

// Hooks for an outer preconditioner that produces z between the update
// and the next SpMV (multigrid).  The last V-cycle kernel reduces z.r and
// calls cg_finish_rz on the device state.
struct ZHook {
    // Enqueue z = M^-1 r on the grid's stream; must end with a kernel that
    // publishes z.r through cg_finish_rz.
    virtual int apply(pg_grid* g, const void* r, void* z) = 0;
    // Identity of the kernel sequence apply() enqueues (graph cache key).
    virtual uintptr_t key() const = 0;
    // The CG's A p vector (read by flexible-CG hooks for beta), given before
    // the first apply().
    virtual void bind(const void* ap) { (void)ap; }
    // Whether apply() writes r (an in-place projection): the CG then cannot
    // hand it the right-hand side itself for the first application.
    virtual bool writes_input() const { return true; }
    virtual ~ZHook() {}
};

// Runs CG on the grid's stream and synchronises at the end.  Returns a
// pg_status for launch/CUDA failures; the solve outcome is in *stats.
template <class T>
int run_cg(pg_grid* g, const CgConfig& cfg, CgBuffers<T> buf, pg_pcg_stats* stats, ZHook* hook = nullptr);

// Whether run_cg with MG preconditioning can carry x as the double-float pair
// (buf.x, buf.xl): float4-aligned buffers and flags, cells a multiple of 4.
// PG_CG_DFX=0 turns it off (a diagnostic switch).
bool cg_dfx_supported(const pg_grid* g, const CgBuffers<float>& buf);

// Device side: fold a freshly reduced z.r into the CG state.  Right after
// init (iter == 0) it is sigma; afterwards beta = z.r / sigma (pcg.rs:67-68).
// With the lazy projection on (nfluid > 0) z stands for z - m on the fluid
// cells, m = sum(z) / nfluid: (z - m).r = z.r - m sum(r) (r is 0 off the
// fluid cells).
__device__ __forceinline__ void cg_finish_rz(CgState* st, double rz, double zsum = 0.0) {
    if (st->done) return;
    if (st->nfluid > 0.0) {
        const double m = zsum / st->nfluid;
        st->zmean = m;
        rz -= m * st->rsum;
    }
    if (!isfinite(rz)) {
        st->status = PG_NAN_DETECTED;
        st->done = 1;
        return;
    }
    if (st->iter == 0) {
        st->sigma = rz;
    } else {
        st->beta = rz / st->sigma;
        st->sigma = rz;
        st->first = 0;
    }
}

// Last-block ticket: true in every thread of the block that finished last.
// Per-block partials must be written (by thread 0) before the call.
__device__ __forceinline__ bool last_block(unsigned int* counter) {
    __shared__ bool am_last;
    __threadfence();
    if (threadIdx.x == 0) {
        const unsigned int t = atomicAdd(counter, 1u);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return am_last;
}

// Deterministic sum (or max) of n per-block partials, by one block of NT.
template <bool MAX, int NT> __device__ __forceinline__ double reduce_partials(const double* partials, int n, double* sm) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double pv = __ldcg(partials + i);
        v = MAX ? fmax(v, pv) : v + pv;
    }
    return MAX ? block_max<NT>(v, sm) : block_sum<NT>(v, sm);
}

}  // namespace pg
