// pg_solve.cu -- pressure solve (plain PCG or FP64 residual refinement) and
// the fluid step of examples/dec_fluid.rs:46-141.
#include <algorithm>
#include <cmath>

#include "pg_cg.cuh"
#include "pg_solve.cuh"

namespace pg {

// Launchers defined in pg_dec.cu / pg_advect.cu.
template <class T> int launch_copy(const pg_grid* g, T* out, const T* in, i64 n);
template <class T> int launch_rhs(const pg_grid* g, T* b, const T* vel);
// Projection into vel from the velocity src (src == vel: in place).
template <class T>
int launch_project(const pg_grid* g, T* vel, const T* p, double dt, int zero_solid, const T* src);
int launch_project_p64(const pg_grid* g, float* vel, const double* p, double dt, int zero_solid, const float* src);
int launch_project_df(const pg_grid* g, float* vel, const float* ph, const float* pl, double dt, int zero_solid,
                      const float* src, float* pout);
template <class T> int launch_walls(const pg_grid* g, T* vel);
template <class T> int launch_source_box(const pg_grid* g, T* rho, T* vel, const pg_step_params* prm);
template <class T> int launch_source_field(const pg_grid* g, T* rho, const T* src);
template <class T> int launch_buoyancy(const pg_grid* g, T* vel, const T* rho, double dt, double beta);
template <class T> int launch_advect(const pg_grid* g, T* dst, const T* src, double dt, const T* vel);
template <class T> int launch_advect_mac(const pg_grid* g, T* dst, const T* src, double dt, const T* vel);
template <class T>
int launch_advect2(const pg_grid* g, T* dst, const T* src, double dt, const T* vel, int scheme, T* t1, T* t2);
int launch_advect_bf16(const pg_grid* g, uint16_t* dst, const uint16_t* src, double dt, const float* vel);
int launch_source_box_bf16(const pg_grid* g, uint16_t* rho, float* vel, const pg_step_params* prm);
int launch_source_field_bf16(const pg_grid* g, uint16_t* rho, const float* src);
int launch_buoyancy_bf16(const pg_grid* g, float* vel, const uint16_t* rho, double dt, double beta);

// Second-order scalar advection with library-owned scratch.
template <class T> static int advect2(pg_grid* g, T* dst, const T* src, double dt, const T* vel, int scheme) {
    if (scheme != 1 && scheme != 2) return bad_arg("advect scheme must be 1 (MacCormack) or 2 (BFECC)");
    const Dims& D = g->dims;
    if (D.h < 2 || D.w < 2 || (D.nd == 3 && D.d < 2)) return bad_arg("pg_advect2: every dimension must be >= 2");
    Extras* ex = extras_of(g);
    void *t1, *t2;
    int rc;
    if ((rc = ex->buffer(Extras::kAdv1, sizeof(T) * (size_t)D.nc(), &t1)) ||
        (rc = ex->buffer(Extras::kAdv2, sizeof(T) * (size_t)D.nc(), &t2)))
        return rc;
    return launch_advect2<T>(g, dst, src, dt, vel, scheme, (T*)t1, (T*)t2);
}

Extras* extras_of(pg_grid* g) {
    if (!g->extras) g->extras = new Extras();
    return (Extras*)g->extras;
}

int Extras::buffer(int slot, size_t bytes, void** out) {
    if (bytes_[slot] < bytes) {
        if (buf_[slot]) {
            PG_CUDA(cudaDeviceSynchronize());
            PG_CUDA(cudaFree(buf_[slot]));
            buf_[slot] = nullptr;
            bytes_[slot] = 0;
        }
        PG_CUDA(cudaMalloc(&buf_[slot], bytes));
        bytes_[slot] = bytes;
    }
    *out = buf_[slot];
    return PG_OK;
}

Extras::~Extras() {
    for (int i = 0; i < kSlots; ++i) cudaFree(buf_[i]);
    release_mg(this);
}

void release_extras(pg_grid* g) {
    delete (Extras*)g->extras;
    g->extras = nullptr;
}

// ---------------------------------------------------------------------------
// FP64 residual r = b - A x for x held in FP64 (refinement), written as T,
// with ||r||inf reduced to *out (device double).
constexpr int kThreads = 256;

template <int ND>
__global__ void __launch_bounds__(kThreads)
    k_residual64(const float* __restrict__ b, const double* __restrict__ x, const uint8_t* __restrict__ flags, Dims D,
                 double dt, float* __restrict__ r, double* partials, unsigned int* counter, double* out) {
    __shared__ double sm[32];
    const i64 n = D.nc(), w = D.w, hw = D.h * D.w;
    double m = 0.0;
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x) {
        const uint8_t f = flags[c];
        const double xc = x[c];
        double s = 0.0;
        if (f & XLO) s += xc - x[c - 1];
        if (f & XHI) s += xc - x[c + 1];
        if (f & YLO) s += xc - x[c - w];
        if (f & YHI) s += xc - x[c + w];
        if (ND == 3) {
            if (f & ZLO) s += xc - x[c - hw];
            if (f & ZHI) s += xc - x[c + hw];
        }
        const double rv = (double)b[c] - dt * s;
        r[c] = (float)rv;
        m = fmax(m, fabs(rv));
    }
    const double bm = block_max<kThreads>(m, sm);
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
    v = block_max<kThreads>(v, sm);
    if (threadIdx.x == 0) {
        *out = v;
        *counter = 0;
    }
}

__global__ void k_x64_add(double* __restrict__ x, const float* __restrict__ d, i64 n) {
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x)
        x[c] += (double)d[c];
}

// x = 0 + d: k_x64_add onto a zeroed x without reading (or zeroing) it.
__global__ void k_x64_set(double* __restrict__ x, const float* __restrict__ d, i64 n) {
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x)
        x[c] = 0.0 + (double)d[c];
}

__global__ void k_x64_store(float* __restrict__ out, const double* __restrict__ x, i64 n) {
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x)
        out[c] = (float)x[c];
}

// ---------------------------------------------------------------------------
// The same three operations in double-float: x = xh + xl held as two FP32
// arrays (|xl| <= ulp(xh)/2), error-free transformations on the FP32 pipes
// (TwoSum, TwoProduct by fma).  The differences x_c - x_nb, where the
// refinement's cancellation happens, are formed exactly in the high parts.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

template <int ND>
__global__ void __launch_bounds__(kThreads)
    k_residual_df(const float* __restrict__ b, const float* __restrict__ xh, const float* __restrict__ xl,
                  const uint8_t* __restrict__ flags, Dims D, float dt, float* __restrict__ r, double* partials,
                  unsigned int* counter, double* out) {
    __shared__ double sm[32];
    const i64 n = D.nc(), w = D.w, hw = D.h * D.w;
    float m = 0.f;
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x) {
        const uint8_t f = flags[c];
        const float hc = xh[c], lc = xl[c];
        float sh = 0.f, sl = 0.f;  // sum over open faces of (x_c - x_nb)
        auto face = [&](i64 k) {
            float dh, de, t, te;
            two_sum(hc, -xh[k], dh, de);
            two_sum(sh, dh, t, te);
            sh = t;
            sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(te, de), __fsub_rn(lc, xl[k])));
        };
        if (f & XLO) face(c - 1);
        if (f & XHI) face(c + 1);
        if (f & YLO) face(c - w);
        if (f & YHI) face(c + w);
        if (ND == 3) {
            if (f & ZLO) face(c - hw);
            if (f & ZHI) face(c + hw);
        }
        const float ph = __fmul_rn(dt, sh);
        const float pl = __fadd_rn(__fmaf_rn(dt, sh, -ph), __fmul_rn(dt, sl));  // dt * (sh + sl) - ph
        float rh, re;
        two_sum(b[c], -ph, rh, re);
        const float rv = __fadd_rn(rh, __fsub_rn(re, pl));
        r[c] = rv;
        m = fmaxf(m, fabsf(rv));
        if (rv != rv) m = __int_as_float(0x7f800000);  // NaN reported as inf
    }
    const double bm = block_max<kThreads>((double)m, sm);
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
    v = block_max<kThreads>(v, sm);
    if (threadIdx.x == 0) {
        *out = v;
        *counter = 0;
    }
}

// k_residual_df for 3D grids as a z-marching 2.5D tile (32 x 8 columns; x/y
// neighbours from shared memory, z neighbours from registers), so each cell's
// (xh, xl) is loaded once.  Same arithmetic as k_residual_df.
constexpr int kRTX = 32, kRTY = 8;

__global__ void __launch_bounds__(kRTX * kRTY)
    k_residual_df3t(const float* __restrict__ b, const float* __restrict__ xh, const float* __restrict__ xl,
                    const uint8_t* __restrict__ flags, Dims D, float dt, float* __restrict__ r, double* partials,
                    unsigned int* counter, double* out, int tiles_x, int tiles_y, int zc, int nwork) {
    __shared__ float SH[kRTY + 2][kRTX + 2], SL[kRTY + 2][kRTX + 2];
    __shared__ double sm[32];
    const int tx = threadIdx.x % kRTX, ty = threadIdx.x / kRTX;
    const int w = (int)D.w, h = (int)D.h, d = (int)D.d;
    const i64 hw = (i64)h * w;
    const int per_plane = tiles_x * tiles_y;
    float m = 0.f;
    for (int item = blockIdx.x; item < nwork; item += gridDim.x) {
        const int tz = item / per_plane, t2 = item - tz * per_plane;
        const int x = (t2 % tiles_x) * kRTX + tx, y = (t2 / tiles_x) * kRTY + ty;
        const int z0 = tz * zc, z1 = min(z0 + zc, d);
        const bool inside = x < w && y < h;
        const i64 col = (i64)y * w + x;
        float bh = 0.f, bl = 0.f, ch = 0.f, cl = 0.f, ah = 0.f, al = 0.f;  // below / current / above
        if (inside) {
            if (z0 > 0) {
                bh = xh[(i64)(z0 - 1) * hw + col];
                bl = xl[(i64)(z0 - 1) * hw + col];
            }
            ch = xh[(i64)z0 * hw + col];
            cl = xl[(i64)z0 * hw + col];
            if (z0 + 1 < d) {
                ah = xh[(i64)(z0 + 1) * hw + col];
                al = xl[(i64)(z0 + 1) * hw + col];
            }
        }
        for (int z = z0; z < z1; ++z) {
            const i64 c = (i64)z * hw + col;
            // plane z + 2 is loaded one step ahead of its use
            float nh = 0.f, nl = 0.f;
            if (inside && z + 2 < d && z + 1 < z1) {
                nh = xh[c + 2 * hw];
                nl = xl[c + 2 * hw];
            }
            SH[ty + 1][tx + 1] = ch;
            SL[ty + 1][tx + 1] = cl;
            if (inside) {
                if (tx == 0 && x > 0) { SH[ty + 1][0] = xh[c - 1]; SL[ty + 1][0] = xl[c - 1]; }
                if (tx == kRTX - 1 && x + 1 < w) { SH[ty + 1][kRTX + 1] = xh[c + 1]; SL[ty + 1][kRTX + 1] = xl[c + 1]; }
                if (ty == 0 && y > 0) { SH[0][tx + 1] = xh[c - w]; SL[0][tx + 1] = xl[c - w]; }
                if (ty == kRTY - 1 && y + 1 < h) { SH[kRTY + 1][tx + 1] = xh[c + w]; SL[kRTY + 1][tx + 1] = xl[c + w]; }
            }
            __syncthreads();
            if (inside) {
                const uint8_t f = flags[c];
                float sh = 0.f, sl = 0.f;
                auto face = [&](float nh, float nl) {
                    float dh, de, t, te;
                    two_sum(ch, -nh, dh, de);
                    two_sum(sh, dh, t, te);
                    sh = t;
                    sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(te, de), __fsub_rn(cl, nl)));
                };
                if (f & XLO) face(SH[ty + 1][tx], SL[ty + 1][tx]);
                if (f & XHI) face(SH[ty + 1][tx + 2], SL[ty + 1][tx + 2]);
                if (f & YLO) face(SH[ty][tx + 1], SL[ty][tx + 1]);
                if (f & YHI) face(SH[ty + 2][tx + 1], SL[ty + 2][tx + 1]);
                if (f & ZLO) face(bh, bl);
                if (f & ZHI) face(ah, al);
                const float ph = __fmul_rn(dt, sh);
                const float pl = __fadd_rn(__fmaf_rn(dt, sh, -ph), __fmul_rn(dt, sl));
                float rh, re;
                two_sum(b[c], -ph, rh, re);
                const float rv = __fadd_rn(rh, __fsub_rn(re, pl));
                r[c] = rv;
                m = fmaxf(m, fabsf(rv));
                if (rv != rv) m = __int_as_float(0x7f800000);
            }
            __syncthreads();
            bh = ch;
            bl = cl;
            ch = ah;
            cl = al;
            ah = nh;
            al = nl;
        }
    }
    const double bm = block_max<kRTX * kRTY>((double)m, sm);
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
    v = block_max<kRTX * kRTY>(v, sm);
    if (threadIdx.x == 0) {
        *out = v;
        *counter = 0;
    }
}

// (xh, xl) += d, renormalised.
__global__ void k_xdf_add(float* __restrict__ xh, float* __restrict__ xl, const float* __restrict__ d, i64 n) {
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x) {
        float s, e;
        two_sum(xh[c], d[c], s, e);
        const float lo = __fadd_rn(xl[c], e);
        const float h2 = __fadd_rn(s, lo);
        xh[c] = h2;
        xl[c] = __fsub_rn(lo, __fsub_rn(h2, s));
    }
}

// x = 0 + d: the arithmetic of k_xdf_add with xh = xl = 0, without reading
// (or zeroing) them -- the same bits for every d, -0 and NaN included.
__global__ void k_xdf_set(float* __restrict__ xh, float* __restrict__ xl, const float* __restrict__ d, i64 n) {
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x) {
        float s, e;
        two_sum(0.f, d[c], s, e);
        const float lo = __fadd_rn(0.f, e);
        const float h2 = __fadd_rn(s, lo);
        xh[c] = h2;
        xl[c] = __fsub_rn(lo, __fsub_rn(h2, s));
    }
}

__global__ void k_xdf_store(float* __restrict__ out, const float* __restrict__ xh, const float* __restrict__ xl, i64 n) {
    for (i64 c = (i64)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (i64)gridDim.x * blockDim.x)
        out[c] = __fadd_rn(xh[c], xl[c]);
}

// One FP64-class residual evaluation; returns ||b - A x||inf on the host.
// x64 is a double array (native) or the [xh | xl] pair (double-float).
static int residual64(pg_grid* g, const float* b, const void* x64, bool native, double dt, float* r,
                      double* rmax_host) {
    if (const int rc = ensure_workspace(g)) return rc;
    Extras* ex = extras_of(g);
    const Dims& D = g->dims;
    const int nb = grid_blocks(g, D.nc(), kThreads, 8);
    double* dev_out = (double*)ex->small;
    unsigned int* counter = (unsigned int*)(dev_out + 1);
    cudaStream_t s = g->stream;
    const double* x = (const double*)x64;
    const float* xh = (const float*)x64;
    const float* xl = xh + D.nc();
    if (native) {
        if (D.nd == 2)
            PG_LAUNCH(KK_RESIDUAL64, s, k_residual64<2><<<nb, kThreads, 0, s>>>(b, x, g->flags, D, dt, r, g->ws.partials, counter, dev_out));
        else
            PG_LAUNCH(KK_RESIDUAL64, s, k_residual64<3><<<nb, kThreads, 0, s>>>(b, x, g->flags, D, dt, r, g->ws.partials, counter, dev_out));
    } else {
        bool done = false;
        if (D.nd == 3)
            PG_LAUNCH(KK_RESIDUAL64, s,
                      done = residual_df_tma_launch(s, g->num_sms, b, xh, xl, g->flags, D, (float)dt, r,
                                                    g->ws.partials, counter, dev_out, g->ws.state));
        if (done) {
        } else if (D.nd == 2) {
            PG_LAUNCH(KK_RESIDUAL64, s, k_residual_df<2><<<nb, kThreads, 0, s>>>(b, xh, xl, g->flags, D, (float)dt, r, g->ws.partials, counter, dev_out));
        } else {
            const int tiles_x = (int)((D.w + kRTX - 1) / kRTX), tiles_y = (int)((D.h + kRTY - 1) / kRTY);
            const int cap = std::min(g->num_sms * 8, kMaxBlocks);
            const i64 want = std::max<i64>(1, (2 * (i64)cap + tiles_x * tiles_y - 1) / ((i64)tiles_x * tiles_y));
            const int zc = (int)std::max<i64>(4, (D.d + want - 1) / want);
            const int nwork = tiles_x * tiles_y * (int)((D.d + zc - 1) / zc);
            const int nbt = std::max(1, std::min(nwork, cap));
            PG_LAUNCH(KK_RESIDUAL64, s,
                      k_residual_df3t<<<nbt, kRTX * kRTY, 0, s>>>(b, xh, xl, g->flags, D, (float)dt, r, g->ws.partials,
                                                                  counter, dev_out, tiles_x, tiles_y, zc, nwork));
        }
    }
    PG_CHECK_LAUNCH();
    double* hs = host_scalar(g->ws);
    k_words_out<<<1, 32, 0, g->stream>>>((const unsigned*)dev_out, (unsigned*)hs, 2);
    PG_CHECK_LAUNCH();
    PG_CUDA(cudaStreamSynchronize(g->stream));
    *rmax_host = *hs;
    return PG_OK;
}

int ensure_small(pg_grid* g) {
    Extras* ex = extras_of(g);
    if (!ex->small) {
        PG_CUDA(cudaMalloc(&ex->small, 256));
        PG_CUDA(cudaMemset(ex->small, 0, 256));
    }
    return PG_OK;
}

// One CG run with z from an outer hook (the grid's z buffer; no lazy
// projection of z's mean).
static int run_hooked(pg_grid* g, CgConfig cfg, CgBuffers<float> buf, ZHook* hook, pg_pcg_stats* st) {
    void* z;
    int rc;
    if ((rc = extras_of(g)->buffer(Extras::kZ, sizeof(float) * (size_t)g->dims.nc(), &z))) return rc;
    buf.z = (float*)z;
    cfg.precond = PG_PRECOND_MG;  // the z-buffer form of the CG kernels
    cfg.nfluid = 0.0;
    return run_cg<float>(g, cfg, buf, st, hook);
}

// Plain CG (the reference algorithm) with library-owned work vectors.
template <class T>
static int solve_plain(pg_grid* g, const pg_solver_params* prm, T* x, const T* b, double dt, pg_pcg_stats* st,
                       ZHook* hook = nullptr) {
    Extras* ex = extras_of(g);
    const size_t n = (size_t)g->dims.nc();
    void *r, *ap, *p0, *p1;
    int rc;
    if ((rc = ex->buffer(Extras::kR, sizeof(T) * n, &r)) || (rc = ex->buffer(Extras::kAp, sizeof(T) * n, &ap)) ||
        (rc = ex->buffer(Extras::kP0, sizeof(T) * n, &p0)) || (rc = ex->buffer(Extras::kP1, sizeof(T) * n, &p1)))
        return rc;
    CgBuffers<T> buf{x, b, (T*)r, (T*)ap, {(T*)p0, (T*)p1}};
    CgConfig cfg{prm->precond, prm->max_iter, prm->threshold, prm->rel_stop ? prm->rel_tol : 0.0, dt,
                 prm->check_every, 1};
    if (hook) {
        if (sizeof(T) != 4) return bad_arg("solver: an outer preconditioner needs f32 fields");
        return run_hooked(g, cfg, *reinterpret_cast<CgBuffers<float>*>(&buf), hook, st);
    }
    if (prm->precond == PG_PRECOND_MG) return solve_mgpcg<T>(g, prm, cfg, buf, st);
    return run_cg<T>(g, cfg, buf, st);
}

// FP32 CG rounds inside FP64 residual refinement.
// store_x = false leaves x to the caller (the step's projection writes it
// from the double-float x it reads anyway); the FP64-class x stays in the
// grid's kX64 buffer either way.
static int solve_refined(pg_grid* g, const pg_solver_params* prm, float* x, const float* b, double dt,
                         pg_pcg_stats* st, ZHook* hook = nullptr, bool store_x = true) {
    Extras* ex = extras_of(g);
    const i64 n = g->dims.nc();
    int rc;
    if ((rc = ensure_small(g))) return rc;
    void *x64, *rr, *d, *ap, *p0, *p1;
    if ((rc = ex->buffer(Extras::kX64, sizeof(double) * n, &x64)) || (rc = ex->buffer(Extras::kR, 4 * n, &rr)) ||
        (rc = ex->buffer(Extras::kD, 4 * n, &d)) || (rc = ex->buffer(Extras::kAp, 4 * n, &ap)) ||
        (rc = ex->buffer(Extras::kP0, 4 * n, &p0)) || (rc = ex->buffer(Extras::kP1, 4 * n, &p1)))
        return rc;
    void* rin;
    if ((rc = ex->buffer(Extras::kRin, 4 * n, &rin))) return rc;
    const int nb = grid_blocks(g, n, kThreads, 8);
    const bool native = prm->fp64_native != 0;
    float* xh = (float*)x64;
    float* xl = xh + n;
    double rmax = 0.0, bmax = 0.0, target = 0.0;
    pg_pcg_stats out{};
    out.status = PG_NOT_CONVERGED;
    i64 iters = 0;
    int rounds = 0;
    const bool guess = prm->initial_guess != 0;
    bool done = false;
    // x = 0: zeroed here only when a guess is added to it; otherwise the
    // first round's correction is stored into it (k_*_set), and a solve
    // that ends before storing any (b = 0, NaN, breakdown) zeroes it at the
    // end.
    bool x_set = guess;
    if (guess) PG_CUDA(cudaMemsetAsync(x64, 0, sizeof(double) * n, g->stream));
    if (guess) {
        // ||b||inf from the residual of x = 0, then the residual of the guess.
        if ((rc = residual64(g, b, x64, native, dt, (float*)rin, &bmax))) return rc;
        target = prm->rel_stop ? prm->rel_tol * bmax : prm->threshold;
        rmax = bmax;
        if (bmax == 0.0 || !std::isfinite(bmax)) {
            out.status = bmax == 0.0 ? PG_OK : PG_NAN_DETECTED;
            done = true;
        } else {
            if (native)
                PG_LAUNCH(KK_REFINE_UPDATE, g->stream, k_x64_add<<<nb, kThreads, 0, g->stream>>>((double*)x64, x, n));
            else
                PG_LAUNCH(KK_REFINE_UPDATE, g->stream, k_xdf_add<<<nb, kThreads, 0, g->stream>>>(xh, xl, x, n));
            PG_CHECK_LAUNCH();
            if ((rc = residual64(g, b, x64, native, dt, (float*)rin, &rmax))) return rc;
            if (!std::isfinite(rmax)) {
                out.status = PG_NAN_DETECTED;
                done = true;
            } else if (rmax <= target) {
                out.status = PG_OK;
                done = true;
            }
        }
    }
    while (!done && rounds < prm->refine) {
        // Round 0 without a guess solves A d = b itself (x = 0, so the
        // residual is b exactly and no residual kernel is needed); other
        // rounds solve for the correction of the FP64-class residual
        // r = b - A x.
        const bool from_b = rounds == 0 && !guess;
        CgBuffers<float> buf{(float*)d, from_b ? b : (const float*)rin, (float*)rr, (float*)ap,
                             {(float*)p0, (float*)p1}};
        // The first refinement round of the MG path accumulates x = 0 +
        // sum(alpha p) straight into the double-float iterate (no
        // k_xdf_set).  An FP32 iterate floors the true residual near 2e-6 of
        // ||b|| (the FP32 sum of a few long steps), so FP32 rounds are asked
        // for no more than 1e-5 and a second round follows; the double-float
        // one is asked for the target itself and usually ends the solve.
        bool dfx = false;
        if (from_b && !native && !hook && prm->precond == PG_PRECOND_MG) {
            CgBuffers<float> b2 = buf;
            b2.x = xh;
            b2.xl = xl;
            if (cg_dfx_supported(g, b2)) {
                buf = b2;
                dfx = true;
            }
        }
        CgConfig cfg{prm->precond, prm->max_iter, 0.0, 0.0, dt, prm->check_every, 1};
        if (from_b && !prm->rel_stop) {
            cfg.threshold = 0.5 * prm->threshold;
        } else {
            // Automatic: reach half the outer target, but never ask FP32 CG
            // for more than ~1e-5 relative per round.  An explicit
            // inner_rel_tol is taken as given.
            if (prm->inner_rel_tol > 0) {
                cfg.rel_tol = std::min(prm->inner_rel_tol, 0.5);
            } else {
                const double inner = from_b ? 0.5 * prm->rel_tol : 0.5 * target / rmax;
                cfg.rel_tol = std::min(std::max(inner, dfx ? 0.0 : 1e-5), 0.5);
            }
        }
        pg_pcg_stats s{};
        if (hook)
            rc = run_hooked(g, cfg, buf, hook, &s);
        else if (prm->precond == PG_PRECOND_MG)
            rc = solve_mgpcg<float>(g, prm, cfg, buf, &s);
        else
            rc = run_cg<float>(g, cfg, buf, &s);
        if (rc) return rc;
        iters += s.iterations;
        ++rounds;
        if (rounds == 1 && !guess) {
            bmax = s.b_max;
            target = prm->rel_stop ? prm->rel_tol * bmax : prm->threshold;
            rmax = bmax;
            if (bmax == 0.0) {  // x = 0 is exact
                out.status = PG_OK;
                break;
            }
        }
        if (s.status == PG_NAN_DETECTED || s.status == PG_BREAKDOWN) {
            out.status = s.status;
            break;
        }
        if (dfx) {
            // x holds the round's iterate -- written by its first update, so
            // a round that made none leaves it to be zeroed here
            if (s.iterations == 0) PG_CUDA(cudaMemsetAsync(x64, 0, sizeof(double) * n, g->stream));
        } else if (from_b) {  // x was 0: x = d
            if (native)
                PG_LAUNCH(KK_REFINE_UPDATE, g->stream, k_x64_set<<<nb, kThreads, 0, g->stream>>>((double*)x64, (const float*)d, n));
            else
                PG_LAUNCH(KK_REFINE_UPDATE, g->stream, k_xdf_set<<<nb, kThreads, 0, g->stream>>>(xh, xl, (const float*)d, n));
        } else if (native) {
            PG_LAUNCH(KK_REFINE_UPDATE, g->stream, k_x64_add<<<nb, kThreads, 0, g->stream>>>((double*)x64, (const float*)d, n));
        } else {
            PG_LAUNCH(KK_REFINE_UPDATE, g->stream, k_xdf_add<<<nb, kThreads, 0, g->stream>>>(xh, xl, (const float*)d, n));
        }
        PG_CHECK_LAUNCH();
        x_set = true;
        if ((rc = residual64(g, b, x64, native, dt, (float*)rin, &rmax))) return rc;
        if (!std::isfinite(rmax)) {
            out.status = PG_NAN_DETECTED;
            break;
        }
        if (rmax <= target) {
            out.status = PG_OK;
            break;
        }
        if (iters >= prm->max_iter * (i64)prm->refine) break;
    }
    out.b_max = bmax;
    out.threshold = target;
    if (!x_set) PG_CUDA(cudaMemsetAsync(x64, 0, sizeof(double) * n, g->stream));
    if (native)
        PG_LAUNCH(KK_REFINE_UPDATE, g->stream, k_x64_store<<<nb, kThreads, 0, g->stream>>>(x, (const double*)x64, n));
    else if (store_x)
        PG_LAUNCH(KK_REFINE_UPDATE, g->stream, k_xdf_store<<<nb, kThreads, 0, g->stream>>>(x, xh, xl, n));
    PG_CHECK_LAUNCH();
    PG_CUDA(cudaStreamSynchronize(g->stream));
    out.iterations = iters;
    out.refinements = rounds;
    out.residual_max = rmax;
    out.true_residual_max = rmax;
    if (st) *st = out;
    return PG_OK;
}

int solve_pressure_hooked(pg_grid* g, const pg_solver_params* prm, float* x, const float* b, double dt, ZHook* hook,
                          pg_pcg_stats* st) {
    if (prm->max_iter < 0) return bad_arg("solver: max_iter < 0");
    if (prm->refine > 0) return solve_refined(g, prm, x, b, dt, st, hook);
    if (prm->initial_guess) return bad_arg("solver: initial_guess needs refine > 0");
    return solve_plain<float>(g, prm, x, b, dt, st, hook);
}

template <class T>
int solve_pressure(pg_grid* g, const pg_solver_params* prm, T* x, const T* b, double dt, pg_pcg_stats* st) {
    if (prm->precond < PG_PRECOND_NONE || prm->precond > PG_PRECOND_MG) return bad_arg("solver: unknown precond");
    if (prm->max_iter < 0) return bad_arg("solver: max_iter < 0");
    if (prm->initial_guess && prm->refine <= 0) return bad_arg("solver: initial_guess needs refine > 0");
    if (prm->refine > 0) {
        if (sizeof(T) != 4) return bad_arg("solver: refinement is for f32 fields");
        return solve_refined(g, prm, (float*)x, (const float*)b, dt, st);
    }
    return solve_plain<T>(g, prm, x, b, dt, st);
}

// ---------------------------------------------------------------------------
// The step (examples/dec_fluid.rs:46-141).  The density is stored as T or,
// with R = uint16_t, as BF16 (pg_bf16.cu).

// density stages for R = T
template <class T> static int density_source_box(pg_grid* g, T* rho, T* vel, const pg_step_params* prm) {
    return launch_source_box<T>(g, rho, vel, prm);
}
template <class T> static int density_source_field(pg_grid* g, T* rho, const void* src) {
    return launch_source_field<T>(g, rho, (const T*)src);
}
template <class T> static int density_advect(pg_grid* g, T* dst, const T* rho, double dt, const T* vel, int scheme) {
    return scheme == 0 ? launch_advect<T>(g, dst, rho, dt, vel) : advect2<T>(g, dst, rho, dt, vel, scheme);
}
template <class T> static int density_buoyancy(pg_grid* g, T* vel, const T* rho, double dt, double beta) {
    return launch_buoyancy<T>(g, vel, rho, dt, beta);
}
// density stages for BF16 storage (FP32 velocity)
static int density_source_box(pg_grid* g, uint16_t* rho, float* vel, const pg_step_params* prm) {
    return launch_source_box_bf16(g, rho, vel, prm);
}
static int density_source_field(pg_grid* g, uint16_t* rho, const void* src) {
    return launch_source_field_bf16(g, rho, (const float*)src);
}
static int density_advect(pg_grid* g, uint16_t* dst, const uint16_t* rho, double dt, const float* vel, int scheme) {
    if (scheme != 0) return bad_arg("BF16 density: only the reference's advection (advect_scheme 0)");
    return launch_advect_bf16(g, dst, rho, dt, vel);
}
static int density_buoyancy(pg_grid* g, float* vel, const uint16_t* rho, double dt, double beta) {
    return launch_buoyancy_bf16(g, vel, rho, dt, beta);
}

template <class T, class R>
int step(pg_grid* g, const pg_step_params* prm, T* vel, R* rho, T* pressure, pg_pcg_stats* st) {
    const Dims& D = g->dims;
    Extras* ex = extras_of(g);
    const size_t nc = (size_t)D.nc(), nf = (size_t)D.nf();
    void *temp, *vtemp, *b;
    int rc;
    if ((rc = ex->buffer(Extras::kTemp, sizeof(T) * nc, &temp)) ||
        (rc = ex->buffer(Extras::kVelTemp, sizeof(T) * nf, &vtemp)) || (rc = ex->buffer(Extras::kB, sizeof(T) * nc, &b)))
        return rc;
    const double dt = prm->dt;
    // inflow (dec_fluid.rs:48-57)
    if (prm->source_enabled && (rc = density_source_box(g, rho, vel, prm))) return rc;
    if (prm->source_field && (rc = density_source_field(g, rho, prm->source_field))) return rc;
    // advection with the old velocity (dec_fluid.rs:59-66)
    if ((rc = density_advect(g, (R*)temp, rho, dt, vel, prm->advect_scheme))) return rc;
    // The advected velocity stays in the scratch buffer `av` until the
    // projection writes the step's result into vel.
    T* av = (T*)vtemp;
    if ((rc = launch_advect_mac<T>(g, av, vel, dt, vel))) return rc;
    PG_CUDA(cudaMemcpyAsync(rho, temp, sizeof(R) * nc, cudaMemcpyDeviceToDevice, g->stream));
    if (prm->walls_after_advect && (rc = launch_walls<T>(g, av))) return rc;
    if (prm->buoyancy != 0.0 && (rc = density_buoyancy(g, av, rho, dt, prm->buoyancy))) return rc;
    // -div (dec_fluid.rs:68-83)
    if ((rc = launch_rhs<T>(g, (T*)b, av))) return rc;
    // pressure solve (dec_fluid.rs:87-121)
    pg_pcg_stats s{};
    // double-float refinement: the projection below also stores the pressure
    const bool df = sizeof(T) == 4 && prm->solver.refine > 0 && !prm->solver.fp64_native;
    if (df) {
        const pg_solver_params* sp = &prm->solver;
        if (sp->precond < PG_PRECOND_NONE || sp->precond > PG_PRECOND_MG) return bad_arg("solver: unknown precond");
        if (sp->max_iter < 0) return bad_arg("solver: max_iter < 0");
        rc = solve_refined(g, sp, (float*)pressure, (const float*)b, dt, &s, nullptr, false);
    } else {
        rc = solve_pressure<T>(g, &prm->solver, pressure, (const T*)b, dt, &s);
    }
    if (rc) return rc;
    // projection + walls (dec_fluid.rs:123-141); after a refined solve the
    // gradient is taken from the FP64 pressure it accumulated.
    if (sizeof(T) == 4 && prm->solver.refine > 0) {
        void* x64;
        if ((rc = ex->buffer(Extras::kX64, sizeof(double) * nc, &x64))) return rc;
        if (prm->solver.fp64_native)
            rc = launch_project_p64(g, (float*)vel, (const double*)x64, dt, prm->zero_solid_after_project,
                                    (const float*)av);
        else
            rc = launch_project_df(g, (float*)vel, (const float*)x64, (const float*)x64 + nc, dt,
                                   prm->zero_solid_after_project, (const float*)av, (float*)pressure);
        if (rc) return rc;
    } else if ((rc = launch_project<T>(g, vel, pressure, dt, prm->zero_solid_after_project, av))) {
        return rc;
    }
    PG_CUDA(cudaStreamSynchronize(g->stream));
    if (st) *st = s;
    return s.status;
}

}  // namespace pg

using namespace pg;

extern "C" int pg_solve_pressure_f32(const pg_grid* g, const pg_solver_params* prm, float* x, const float* b,
                                     double dt, pg_pcg_stats* st) {
    if (!g || !prm || !x || !b) return bad_arg("pg_solve_pressure: NULL argument");
    pg_pcg_stats s{};
    int rc = solve_pressure<float>(const_cast<pg_grid*>(g), prm, x, b, dt, &s);
    if (rc) return rc;
    if (st) *st = s;
    return s.status;
}

#define PG_ADV2_ABI(T, SFX)                                                                                     \
    extern "C" int pg_advect2_##SFX(const pg_grid* g, T* dst, const T* src, double dt, const T* vel, int scheme) { \
        if (!g || !dst || !src || !vel) return bad_arg("pg_advect2: NULL argument");                           \
        if (dst == src) return bad_arg("pg_advect2: dst must not alias src");                                  \
        return advect2<T>(const_cast<pg_grid*>(g), dst, src, dt, vel, scheme);                                 \
    }
PG_ADV2_ABI(float, f32)
PG_ADV2_ABI(double, f64)

#define PG_STEP_ABI(T, SFX)                                                                                     \
    extern "C" int pg_step_##SFX(const pg_grid* g, const pg_step_params* prm, T* vel, T* rho, T* pressure,     \
                                 pg_pcg_stats* st) {                                                           \
        if (!g || !prm || !vel || !rho || !pressure) return bad_arg("pg_step: NULL argument");                 \
        return step<T, T>(const_cast<pg_grid*>(g), prm, vel, rho, pressure, st);                               \
    }

PG_STEP_ABI(float, f32)
PG_STEP_ABI(double, f64)

extern "C" int pg_step_bf16rho_f32(const pg_grid* g, const pg_step_params* prm, float* vel, uint16_t* rho,
                                   float* pressure, pg_pcg_stats* st) {
    if (!g || !prm || !vel || !rho || !pressure) return bad_arg("pg_step_bf16rho_f32: NULL argument");
    return step<float, uint16_t>(const_cast<pg_grid*>(g), prm, vel, rho, pressure, st);
}
