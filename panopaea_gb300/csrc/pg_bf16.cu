// pg_bf16.cu -- BF16-stored density for the fluid step (an extension: the
// reference's density is a Simplex2<f64>, examples/dec_fluid.rs:34-37).
//
// The advected scalar is the step's only cell field that is streamed by
// advection alone; storing it in BF16 halves its bytes.  Every kernel that
// touches it reads BF16 values exactly into FP32, computes in FP32 with the
// same operation order as the FP32 kernels (advection: dec_fluid.rs:173-211,
// trilinear in 3D; source: :48-57; buoyancy) and rounds to nearest even on
// store, so a step equals the FP32 step with the density rounded to BF16
// after every write.  Velocity, pressure and the solve stay FP32 (+ FP64
// refinement).
#include <cuda_bf16.h>

#include "pg_ops2d.cuh"

namespace pg {

namespace {

constexpr int kThreads = 256;
#define GRID_STRIDE_B(i, n) for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (I)gridDim.x * blockDim.x)

__device__ __forceinline__ float ld(const uint16_t* p, i64 k) {
    return __uint_as_float((unsigned)p[k] << 16);
}
__device__ __forceinline__ uint16_t st_bf16(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }

template <class I>
__global__ void k_advect_bf16_2d(uint16_t* __restrict__ dst, const uint16_t* __restrict__ q,
                                 const float* __restrict__ vel, I h, I w, float ndt, float hix, float hiy) {
    const float* vy = vel;
    const float* vx = vel + (h + 1) * w;
    GRID_STRIDE_B(i, h * w) {
        const I y = i / w, x = i - y * w;
        const float vcx = half_rn(add_rn(vx[y * (w + 1) + x], vx[y * (w + 1) + x + 1]));
        const float vcy = half_rn(add_rn(vy[y * w + x], vy[(y + 1) * w + x]));
        I ix, iy;
        float u, v;
        cell_coord(back(add_rn((float)x, 0.5f), ndt, vcx), w, hix, ix, u);
        cell_coord(back(add_rn((float)y, 0.5f), ndt, vcy), h, hiy, iy, v);
        const I k = iy * w + ix;
        dst[i] = st_bf16(bilerp(ld(q, k), ld(q, k + 1), ld(q, k + w), ld(q, k + w + 1), u, v));
    }
}

template <class I>
__global__ void k_advect_bf16_3d(uint16_t* __restrict__ dst, const uint16_t* __restrict__ q,
                                 const float* __restrict__ vel, Dims D, float ndt, float hix, float hiy, float hiz) {
    const I d = (I)D.d, h = (I)D.h, w = (I)D.w, hw = h * w;
    const I offy = (I)D.offy(), offx = (I)D.offx();
    GRID_STRIDE_B(i, d * hw) {
        const I zy = i / w, x = i - zy * w;
        const I z = zy / h, y = zy - z * h;
        const float vcx = half_rn(add_rn(vel[offx + (z * h + y) * (w + 1) + x], vel[offx + (z * h + y) * (w + 1) + x + 1]));
        const float vcy = half_rn(add_rn(vel[offy + (z * (h + 1) + y) * w + x], vel[offy + (z * (h + 1) + y + 1) * w + x]));
        const float vcz = half_rn(add_rn(vel[(z * h + y) * w + x], vel[((z + 1) * h + y) * w + x]));
        I ix, iy, iz;
        float s, t, u;
        cell_coord(back(add_rn((float)x, 0.5f), ndt, vcx), w, hix, ix, s);
        cell_coord(back(add_rn((float)y, 0.5f), ndt, vcy), h, hiy, iy, t);
        cell_coord(back(add_rn((float)z, 0.5f), ndt, vcz), d, hiz, iz, u);
        const I k0 = iz * hw + iy * w + ix, k1 = k0 + hw;
        const float b0 = bilerp(ld(q, k0), ld(q, k0 + 1), ld(q, k0 + w), ld(q, k0 + w + 1), s, t);
        const float b1 = bilerp(ld(q, k1), ld(q, k1 + 1), ld(q, k1 + w), ld(q, k1 + w + 1), s, t);
        dst[i] = st_bf16(lerp_ref(b0, b1, u));
    }
}

template <class I>
__global__ void k_source_box_bf16(uint16_t* __restrict__ rho, float* __restrict__ vel, Dims D, I z0, I y0, I x0, I bz,
                                  I by, I bx, float sd, float sv) {
    GRID_STRIDE_B(i, bz * by * bx) {
        const I zy = i / bx, x = x0 + (i - zy * bx);
        const I z = z0 + zy / by, y = y0 + zy % by;
        rho[(I)D.cell(z, y, x)] = st_bf16(sd);
        vel[(I)D.fy(z, y, x)] = sv;
    }
}

__global__ void k_source_field_bf16(uint16_t* __restrict__ rho, const float* __restrict__ src, i64 n) {
    typedef i64 I;
    GRID_STRIDE_B(i, n) rho[i] = st_bf16(fmax(ld(rho, i), src[i]));
}

template <class I>
__global__ void k_buoyancy_bf16(float* __restrict__ vel, const uint16_t* __restrict__ rho, Dims D, float coef) {
    const I h = D.h, w = D.w;
    GRID_STRIDE_B(j, (I)D.nfy()) {
        const I zy = j / w, x = j - zy * w;
        const I z = zy / (h + 1), y = zy - z * (h + 1);
        if (y == 0 || y == h) continue;
        const I c = (z * h + y) * w + x;
        const I f = (I)D.offy() + j;
        vel[f] = add_rn(vel[f], mul_rn(coef, mul_rn(0.5f, add_rn(ld(rho, c - w), ld(rho, c)))));
    }
}

}  // namespace

int launch_advect_bf16(const pg_grid* g, uint16_t* dst, const uint16_t* src, double dt, const float* vel) {
    const Dims& D = g->dims;
    if (D.h < 2 || D.w < 2 || (D.nd == 3 && D.d < 2))
        return bad_arg("pg_advect_bf16: every dimension must be >= 2 (the reference indexes the +1 neighbour)");
    const float ndt = -(float)dt;
    const float hix = (float)((double)D.w - 1.00001), hiy = (float)((double)D.h - 1.00001),
                hiz = (float)((double)D.d - 1.00001);
    const int nb = grid_blocks(g, D.nc(), kThreads);
    cudaStream_t s = g->stream;
    PG_IDX(g, {
        if (D.nd == 2)
            PG_LAUNCH(KK_ADVECT, s, k_advect_bf16_2d<I><<<nb, kThreads, 0, s>>>(dst, src, vel, (I)D.h, (I)D.w, ndt, hix, hiy));
        else
            PG_LAUNCH(KK_ADVECT, s, k_advect_bf16_3d<I><<<nb, kThreads, 0, s>>>(dst, src, vel, D, ndt, hix, hiy, hiz));
    });
    PG_CHECK_LAUNCH();
    return PG_OK;
}

int launch_source_box_bf16(const pg_grid* g, uint16_t* rho, float* vel, const pg_step_params* prm) {
    const Dims& D = g->dims;
    i64 lo[3], hi[3];
    const i64 ext[3] = {D.d, D.h, D.w};
    for (int a = 0; a < 3; ++a) {  // the FP32 source's rule
        lo[a] = prm->source_lo[a];
        hi[a] = prm->source_hi[a];
        if (D.nd == 2 && a == 0) {
            lo[a] = 0;
            hi[a] = 1;
        }
        if (lo[a] < 0 || hi[a] > ext[a] || lo[a] > hi[a]) return bad_arg("source box outside the grid");
    }
    const i64 n = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
    if (n == 0) return PG_OK;
    PG_IDX(g, PG_LAUNCH(KK_STEP_MISC, g->stream,
                        k_source_box_bf16<I><<<grid_blocks(g, n, kThreads), kThreads, 0, g->stream>>>(
                            rho, vel, D, (I)lo[0], (I)lo[1], (I)lo[2], (I)(hi[0] - lo[0]), (I)(hi[1] - lo[1]),
                            (I)(hi[2] - lo[2]), (float)prm->source_density, (float)prm->source_vy)));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

int launch_source_field_bf16(const pg_grid* g, uint16_t* rho, const float* src) {
    const i64 n = g->dims.nc();
    PG_LAUNCH(KK_STEP_MISC, g->stream, k_source_field_bf16<<<grid_blocks(g, n, kThreads), kThreads, 0, g->stream>>>(rho, src, n));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

int launch_buoyancy_bf16(const pg_grid* g, float* vel, const uint16_t* rho, double dt, double beta) {
    const Dims& D = g->dims;
    PG_IDX(g, PG_LAUNCH(KK_STEP_MISC, g->stream,
                        k_buoyancy_bf16<I><<<grid_blocks(g, D.nfy(), kThreads), kThreads, 0, g->stream>>>(
                            vel, rho, D, (float)(dt * beta))));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

}  // namespace pg

using namespace pg;

extern "C" int pg_advect_bf16(const pg_grid* g, uint16_t* dst, const uint16_t* src, double dt, const float* vel) {
    if (!g || !dst || !src || !vel) return bad_arg("pg_advect_bf16: NULL argument");
    if (dst == src) return bad_arg("pg_advect_bf16: dst must not alias src");
    return launch_advect_bf16(g, dst, src, dt, vel);
}
