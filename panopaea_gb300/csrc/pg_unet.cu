// pg_unet.cu -- the learned pressure guess: a 3-level 3D conv U-Net with 16
// base channels, BF16 weights and activations, FP32 accumulation on the
// tensor cores (mma.sync m16n8k16), trained on the device by its own
// forward and backward kernels.  No reference counterpart (panopaea has no
// learned component).
//
// Network (channels-last tensors [voxel][channel], level l = dims >> l):
//   X0 = (b / rms(b), n_open / 6, 0 x 14)
//   L0 16->16, L1 16->16 (skip0), P0 = avgpool(L1)
//   L2 16->32, L3 32->32 (skip1), P1 = avgpool(L3)
//   L4 32->64, L5 64->64
//   C1 = [up(L5) | L3] (96), L6 96->32, L7 32->32
//   C0 = [up(L7) | L1] (48), L8 48->16, L9 16->16
//   q = L9 . wh (FP32), 0 on solid cells; guess = q * rms(b) * out_scale / dt
// Every conv is 3x3x3, zero padded, followed by ReLU.
//
// Kernels:
//   k_conv   implicit-GEMM conv: M = voxels of a CTA tile, N = C_out,
//            K = 27 taps x C_in.  The input brick (tile + 1-voxel halo, one
//            16-channel chunk at a time) is staged in shared memory with a
//            48-byte voxel stride (conflict-free ldmatrix rows); B fragments
//            come pre-permuted from global memory (L1-resident weights).  The
//            backward-data pass is the same kernel with the transposed,
//            tap-mirrored weights and a ReLU-gate epilogue.
//   k_wgrad  dW[tap] = X(shifted)^T dZ: one CTA per (tap, voxel slab), the
//            chunk of X and dZ staged in shared memory and fed to the tensor
//            cores with ldmatrix.trans; per-slab partials summed in fixed
//            order (deterministic).
//   small elementwise kernels: input, pooling, upsample+concat and their
//            backward forms, the output layer + loss, Adam, weight layouts.

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "pg_internal.cuh"
#include "pg_solve.cuh"
#include "pg_tma.cuh"

namespace pg {
template <class T> int launch_laplacian(const pg_grid* g, T* out, const T* p, double dt);
}

namespace pg {
namespace unet {

typedef __nv_bfloat16 bf16;

constexpr int kL = 10;
constexpr int kCin[kL] = {16, 16, 16, 32, 32, 64, 96, 32, 48, 16};
constexpr int kCout[kL] = {16, 16, 32, 32, 64, 64, 32, 32, 16, 16};
constexpr int kLevel[kL] = {0, 0, 1, 1, 2, 2, 1, 1, 0, 0};

inline i64 param_offset(int k) {
    i64 o = 0;
    for (int j = 0; j < k; ++j) o += 27LL * kCin[j] * kCout[j];
    return o;
}
inline i64 num_params() { return param_offset(kL) + 16; }

// ---------------------------------------------------------------------------
// Tensor-core primitives (inline PTX).

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t& r0, uint32_t& r1, uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(addr));
}
// D += A (16x16, row) * B (16x8, col), bf16 inputs, f32 accumulators.
__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    uint32_t u;
    memcpy(&u, &h, 4);
    return u;
}

// ---------------------------------------------------------------------------
// Implicit-GEMM 3x3x3 convolution.

enum { EPI_RELU = 0, EPI_NONE = 1, EPI_GATE = 2 };
constexpr int kConvThreads = 256;
constexpr int kRowBytes = 48;  // one brick voxel, one 16-channel chunk: 32 B + 16 B pad

struct ConvGeom {
    int D, H, W;
    int TX, TY, TZ;
    int BX, BY;  // brick extent (tile + 2) in x and y
    int tiles_x, tiles_y;
};

// out[v][co] = epi(sum_tap sum_ci in[v + off(tap)][ci] * w[tap][ci][co]).
// wf: fragments [tap][CIN/16][COUT/8][lane] of the B operand.
template <int CIN, int COUT, int MT>
__global__ void __launch_bounds__(kConvThreads) k_conv(const bf16* __restrict__ in, const uint2* __restrict__ wf,
                                                       bf16* __restrict__ out, const bf16* __restrict__ gate,
                                                       ConvGeom G, int epi) {
    extern __shared__ __align__(16) unsigned char brick[];
    constexpr int NT = COUT / 8, KC = CIN / 16;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int t = blockIdx.x;
    const int tx0 = (t % G.tiles_x) * G.TX;
    t /= G.tiles_x;
    const int ty0 = (t % G.tiles_y) * G.TY;
    const int tz0 = (t / G.tiles_y) * G.TZ;
    const int nbrick = G.BX * G.BY * (G.TZ + 2);
    const uint32_t sbase = smem_addr(brick);

    // ldmatrix row address of this lane for each m-tile: voxel (lane & 15)
    // of the tile, channel half (lane >> 4) of the 16-channel chunk.
    uint32_t arow[MT];
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
        const int v = (warp * MT + mt) * 16 + (lane & 15);
        const int x = v % G.TX, y = (v / G.TX) % G.TY, z = v / (G.TX * G.TY);
        arow[mt] = sbase + ((z * G.BY + y) * G.BX + x) * kRowBytes + (lane >> 4) * 16;
    }
    float acc[MT][NT][4];
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[mt][nt][j] = 0.f;

    for (int kc = 0; kc < KC; ++kc) {
        if (kc) __syncthreads();
        for (int i = threadIdx.x; i < nbrick * 2; i += kConvThreads) {
            const int bv = i >> 1, hf = i & 1;
            const int bx = bv % G.BX, r = bv / G.BX;
            const int by = r % G.BY, bz = r / G.BY;
            const int gx = tx0 + bx - 1, gy = ty0 + by - 1, gz = tz0 + bz - 1;
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if ((unsigned)gx < (unsigned)G.W && (unsigned)gy < (unsigned)G.H && (unsigned)gz < (unsigned)G.D)
                val = __ldg(reinterpret_cast<const uint4*>(in + (((size_t)gz * G.H + gy) * G.W + gx) * CIN + kc * 16 +
                                                           hf * 8));
            *reinterpret_cast<uint4*>(brick + bv * kRowBytes + hf * 16) = val;
        }
        __syncthreads();
#pragma unroll 1
        for (int tap = 0; tap < 27; ++tap) {
            const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
            const uint32_t toff = (uint32_t)(((dz * G.BY + dy) * G.BX + dx) * kRowBytes);
            uint32_t a[MT][4];
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) ldsm_x4(a[mt], arow[mt] + toff);
            const uint2* wp = wf + ((size_t)(tap * KC + kc) * NT) * 32 + lane;
#pragma unroll
            for (int nt = 0; nt < NT; ++nt) {
                const uint2 b = __ldg(wp + nt * 32);
#pragma unroll
                for (int mt = 0; mt < MT; ++mt) mma_bf16(acc[mt][nt], a[mt], b.x, b.y);
            }
        }
    }

#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
            const int v = (warp * MT + mt) * 16 + (lane >> 2) + hf * 8;
            const int x = tx0 + v % G.TX, y = ty0 + (v / G.TX) % G.TY, z = tz0 + v / (G.TX * G.TY);
            if (x >= G.W || y >= G.H || z >= G.D) continue;
            const size_t o = (((size_t)z * G.H + y) * G.W + x) * COUT + (lane & 3) * 2;
#pragma unroll
            for (int nt = 0; nt < NT; ++nt) {
                float v0 = acc[mt][nt][hf * 2], v1 = acc[mt][nt][hf * 2 + 1];
                if (epi == EPI_RELU) {
                    v0 = v0 > 0.f ? v0 : 0.f;
                    v1 = v1 > 0.f ? v1 : 0.f;
                } else if (epi == EPI_GATE) {
                    const __nv_bfloat162 gv = *reinterpret_cast<const __nv_bfloat162*>(gate + o + nt * 8);
                    if (!(__bfloat162float(gv.x) > 0.f)) v0 = 0.f;
                    if (!(__bfloat162float(gv.y) > 0.f)) v1 = 0.f;
                }
                *reinterpret_cast<__nv_bfloat162*>(out + o + nt * 8) = __floats2bfloat162_rn(v0, v1);
            }
        }
}

// ---------------------------------------------------------------------------
// The same convolution on the fifth-generation tensor cores: tcgen05.mma
// (kind::f16, BF16 operands, FP32 accumulators in tensor memory), issued by
// one thread, operands described in shared memory.
//
// GEMM per CTA: M = 128 output voxels (an 8 x 16 x-y tile of one z plane),
// N = C_out, K = 27 taps x C_in; TZ consecutive z planes per CTA, each with
// its own 128 x N accumulator in tensor memory.  The input brick (tile plus
// a one-voxel halo, TZ + 2 planes) is staged per 16-channel chunk in a
// chunk-planar layout: [8-channel half][bz][by][bx] x 16 bytes.  In that
// layout the A operand of every tap is a plain K-major, no-swizzle operand
// inside the brick -- core matrices of 8 consecutive x voxels x 16 bytes
// (contiguous 128 B), 8-row groups one brick row (BX x 16 B) apart, the two
// 8-channel halves one plane apart -- so a tap is only a different start
// address: no im2col copy.  The weights of a chunk arrive pre-laid-out as
// [tap][8-channel half][n][8] (B operand, K-major: n rows 16 B apart, 8-row
// groups 128 B apart, halves N x 16 B apart).
namespace tc {

constexpr int TX = 8, TY = 16, BX = TX + 2, BY = TY + 2;
constexpr int kThreads = 256;

// Shared-memory matrix descriptor, no swizzle (start, leading- and
// stride-dimension byte offsets in 16-byte units; descriptor version 1).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
// One arrival on bar once every tcgen05.mma this thread issued has completed.
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// Zero 8 consecutive 32-bit columns of this thread's lane.
__device__ __forceinline__ void st8_zero(uint32_t taddr) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr), "r"(0u)
                 : "memory");
}

// 8 consecutive 32-bit columns of this thread's lane.
__device__ __forceinline__ void ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// Small output channel counts merge the three z taps into one MMA: an input
// brick plane bs feeds output planes bs, bs - 1 and bs - 2 through the taps
// dz = 0, 1, 2 with the same A operand, so their weights are stacked along N
// (N' = 3 N) and the planes' accumulators are laid out in reverse order
// (plane t at column (TZ + 1 - t) N): one MMA per input plane and (dx, dy)
// writes the three planes' columns.  Planes -2, -1, TZ, TZ + 1 take the edge
// products that no output needs.  Half the A-operand reads of the 27-tap
// loop, for the layers whose MMA is bound by that shared-memory traffic.
__host__ __device__ constexpr bool merge_dz(int n) { return n <= 32; }

template <int COUT> struct Cfg {
    static constexpr bool kMerge = merge_dz(COUT);
    static constexpr int TZ = COUT >= 96 ? 2 : 4;
    static constexpr int BZ = TZ + 2;
    static constexpr int kPlane = BX * BY * BZ * 16;      // one 8-channel half of the brick
    static constexpr int kBrick = 2 * kPlane;             // one 16-channel chunk
    static constexpr int kWTap = 2 * COUT * 16;           // one tap of one chunk
    static constexpr int kWTap9 = 3 * kWTap;              // merged: the three z taps of one (dx, dy)
    static constexpr int kWChunk = 27 * kWTap;
    static constexpr int kBrickOff = 128, kWOff = kBrickOff + kBrick;
    static constexpr size_t kSmem = 128 + (size_t)kBrick + kWChunk;
    static constexpr int kAccCols = kMerge ? (TZ + 4) * COUT : TZ * COUT;
    static constexpr int kCols = kAccCols <= 32 ? 32 : (kAccCols <= 64 ? 64 : (kAccCols <= 128 ? 128 : (kAccCols <= 256 ? 256 : 512)));
    static_assert(kAccCols <= 512, "accumulators must fit in tensor memory");
    static_assert(kPlane % 16 == 0 && kBrick % 128 == 0, "operand alignment");
    // tensor-memory column of output plane t's accumulator
    __host__ __device__ static constexpr int col(int t) { return kMerge ? (TZ + 1 - t) * COUT : t * COUT; }
};

struct Geom {
    int D, H, W;
    int tiles_x, tiles_y;
};

// wtc: [chunk][tap][half][n][8] BF16 (see above); err: set when a wait for
// the tensor cores gave up (the result is then not to be trusted).
template <int CIN, int COUT>
__global__ void __launch_bounds__(kThreads) k_conv_tc(const bf16* __restrict__ in, const bf16* __restrict__ wtc,
                                                      bf16* __restrict__ out, const bf16* __restrict__ gate, Geom G,
                                                      int epi, int* err) {
    typedef Cfg<COUT> C;
    constexpr int KC = CIN / 16, TZ = C::TZ;
    constexpr uint32_t kIdesc = idesc_bf16(128, COUT);
    extern __shared__ __align__(128) unsigned char tc_smem_raw[];
    unsigned char* const base = tc_smem_raw + ((128u - (smem_u32(tc_smem_raw) & 127u)) & 127u);
    uint64_t* const bar = (uint64_t*)base;
    uint32_t* const tslot = (uint32_t*)(base + 8);
    unsigned char* const brick = base + C::kBrickOff;
    unsigned char* const wsm = base + C::kWOff;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int t = blockIdx.x;
    const int x0 = (t % G.tiles_x) * TX;
    t /= G.tiles_x;
    const int y0 = (t % G.tiles_y) * TY;
    const int z0 = (t / G.tiles_y) * TZ;
    if (warp == 0) tmem_alloc(tslot, C::kCols);
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    if (C::kMerge) {  // every merged MMA accumulates: start the accumulators at zero
        if (warp < 4) {
            for (int c = 0; c < C::kAccCols; c += 8) st8_zero(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c);
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        }
        fence_before();
        __syncthreads();
        fence_after();
    }
    bool ok = true;  // block-uniform
    int committed = -1;
    for (int kc = 0; kc < KC; ++kc) {
        if (kc > 0) {  // the previous chunk's MMAs have read the brick and the weights
            bool w = true;
            if (tid == 0) w = mbar_wait(bar, (kc - 1) & 1);
            ok = !__syncthreads_or(!w);
            if (!ok) break;
        }
        // brick of this chunk: voxel (bx, by, bz) half hf at brick + hf * plane + voxel * 16
        constexpr int nvox = BX * BY * C::BZ;
        for (int i = tid; i < 2 * nvox; i += kThreads) {
            const int hf = i & 1, v = i >> 1;
            const int bx = v % BX, r = v / BX, by = r % BY, bz = r / BY;
            const int gx = x0 + bx - 1, gy = y0 + by - 1, gz = z0 + bz - 1;
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if ((unsigned)gx < (unsigned)G.W && (unsigned)gy < (unsigned)G.H && (unsigned)gz < (unsigned)G.D)
                val = __ldg(reinterpret_cast<const uint4*>(in + (((size_t)gz * G.H + gy) * G.W + gx) * CIN + kc * 16 +
                                                           hf * 8));
            *reinterpret_cast<uint4*>(brick + hf * C::kPlane + v * 16) = val;
        }
        // weights of this chunk (contiguous)
        {
            const uint4* src = reinterpret_cast<const uint4*>(wtc + (size_t)kc * (C::kWChunk / 2));
            uint4* dst = reinterpret_cast<uint4*>(wsm);
            for (int i = tid; i < C::kWChunk / 16; i += kThreads) dst[i] = __ldg(src + i);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic-proxy writes -> tensor-core reads
        __syncthreads();
        if (tid == 0) {
            fence_after();
            const uint32_t bs = smem_u32(brick), ws = smem_u32(wsm);
            if (C::kMerge) {
                constexpr uint32_t kIdesc3 = idesc_bf16(128, 3 * COUT);
#pragma unroll 1
                for (int tap9 = 0; tap9 < 9; ++tap9) {
                    const int dy = tap9 / 3, dx = tap9 % 3;
                    const uint64_t bdesc = sdesc(ws + tap9 * C::kWTap9, 3 * COUT * 16, 128);
#pragma unroll
                    for (int pz = 0; pz < C::BZ; ++pz) {
                        const uint32_t a = bs + (uint32_t)(((pz * BY + dy) * BX + dx) * 16);
                        mma(tmem + (uint32_t)C::col(pz), sdesc(a, C::kPlane, BX * 16), bdesc, kIdesc3, 1u);
                    }
                }
            } else {
#pragma unroll 1
                for (int tap = 0; tap < 27; ++tap) {
                    const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
                    const uint64_t bdesc = sdesc(ws + tap * C::kWTap, COUT * 16, 128);
#pragma unroll
                    for (int tz = 0; tz < TZ; ++tz) {
                        const uint32_t a = bs + (uint32_t)((((tz + dz) * BY + dy) * BX + dx) * 16);
                        mma(tmem + (uint32_t)(tz * COUT), sdesc(a, C::kPlane, BX * 16), bdesc, kIdesc,
                            (kc > 0 || tap > 0) ? 1u : 0u);
                    }
                }
            }
            commit(bar);
        }
        committed = kc;
    }
    // every MMA has completed before the accumulators are read
    if (ok) {
        bool w = true;
        if (tid == 0) w = mbar_wait(bar, (KC - 1) & 1);
        ok = !__syncthreads_or(!w);
    }
    if (!ok) {
        // a wait gave up: flag it, wait once more (bounded) for the tensor
        // cores' last committed group, and leave the accumulators unread
        if (tid == 0) {
            atomicExch(err, 1);
            if (committed >= 0) mbar_wait(bar, committed & 1);
        }
        __syncthreads();
    } else {
        fence_after();
        // warp w reads lanes 32 (w % 4) .. +31 (rows of the tile) of the planes of its half
        const int q = warp & 3, half = warp >> 2;
        const int m = q * 32 + lane;
        const int x = x0 + (m & 7), y = y0 + (m >> 3);
        constexpr int PZ = TZ / 2;
#pragma unroll 1
        for (int tz = half * PZ; tz < (half + 1) * PZ; ++tz) {
            const int z = z0 + tz;
            const bool in_grid = x < G.W && y < G.H && z < G.D;
            const size_t o = (((size_t)z * G.H + y) * G.W + x) * COUT;
#pragma unroll 1
            for (int cg = 0; cg < COUT / 8; ++cg) {
                float v[8];
                ld8(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(C::col(tz) + cg * 8), v);
                if (!in_grid) continue;
                if (epi == EPI_RELU) {
#pragma unroll
                    for (int i = 0; i < 8; ++i) v[i] = v[i] > 0.f ? v[i] : 0.f;
                } else if (epi == EPI_GATE) {
                    const uint4 gv = *reinterpret_cast<const uint4*>(gate + o + cg * 8);
                    const uint32_t gw[4] = {gv.x, gv.y, gv.z, gv.w};
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        __nv_bfloat162 pr;
                        memcpy(&pr, &gw[i], 4);
                        if (!(__bfloat162float(pr.x) > 0.f)) v[2 * i] = 0.f;
                        if (!(__bfloat162float(pr.y) > 0.f)) v[2 * i + 1] = 0.f;
                    }
                }
                *reinterpret_cast<uint4*>(out + o + cg * 8) =
                    make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                               pack_bf16(v[6], v[7]));
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        tmem_dealloc(tmem, C::kCols);
    }
}

// Weights of the tensor-core path: wtc[chunk][tap][half][n][8] with the
// K index k = 16 chunk + 8 half + j an input channel of the convolution and
// n an output channel; forward W[tap][k][n], backward-data (transposed,
// tap-mirrored) W[26 - tap][n][k] of the forward layer.
// With merge_dz(N) the three z taps of one (dx, dy) are stacked along N:
// wtc[chunk][dy 3 + dx][half][dz N + n][8].
__global__ void k_wprep_tc(const float* __restrict__ W, int cin, int cout, int transposed, bf16* __restrict__ wtc) {
    const int K = transposed ? cout : cin, N = transposed ? cin : cout;
    const bool merged = merge_dz(N);
    const int n_all = 27 * K * N;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_all; i += gridDim.x * blockDim.x) {
        const int j = i & 7;
        int r = i >> 3;
        int n, hf, tap, kc;
        if (merged) {
            const int nn = r % (3 * N);
            r /= 3 * N;
            hf = r & 1;
            r >>= 1;
            const int tap9 = r % 9;
            kc = r / 9;
            n = nn % N;
            tap = (nn / N) * 9 + tap9;
        } else {
            n = r % N;
            r /= N;
            hf = r & 1;
            r >>= 1;
            tap = r % 27;
            kc = r / 27;
        }
        const int k = kc * 16 + hf * 8 + j;
        const float v = transposed ? W[((size_t)(26 - tap) * cin + n) * cout + k] : W[((size_t)tap * cin + k) * cout + n];
        wtc[i] = __float2bfloat16_rn(v);
    }
}

}  // namespace tc

// ---------------------------------------------------------------------------
// Weight gradient: part[slab][tap][ci][co] = sum over the slab's voxels v of
// X[v + off(tap)][ci] * dZ[v][co].

constexpr int kWgChunk = 64;  // voxels staged per step

template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_wgrad(const bf16* __restrict__ X, const bf16* __restrict__ dZ,
                                               float* __restrict__ part, int D, int H, int W, i64 slab) {
    constexpr int MTL = CIN / 16, NTL = COUT / 8, U = MTL * NTL;
    static_assert(U < 8 || U % 8 == 0, "tile count must be < 8 or a multiple of 8");
    constexpr int G = U >= 8 ? 1 : (8 % U == 0 ? 8 / U : 1);  // warps sharing a tile (k split)
    constexpr int UPW = U >= 8 ? U / 8 : 1;                   // tiles per warp
    constexpr int XS = CIN * 2 + 16, ZS = COUT * 2 + 16;      // smem bytes per voxel row
    constexpr int XV = CIN / 8, ZV = COUT / 8;                // 16-byte vectors per voxel
    __shared__ __align__(16) unsigned char xs[kWgChunk * XS];
    __shared__ __align__(16) unsigned char zs[kWgChunk * ZS];
    __shared__ float red[8][128];
    const int tap = blockIdx.x;
    const int oz = tap / 9 - 1, oy = (tap / 3) % 3 - 1, ox = tap % 3 - 1;
    const i64 V = (i64)D * H * W;
    const i64 v0 = (i64)blockIdx.y * slab;
    const i64 v1 = min(V, v0 + slab);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int kslot = warp % G;
    const int tile0 = U >= 8 ? warp : warp / G;
    const bool active = U >= 8 || tile0 < U;
    const uint32_t xb = smem_addr(xs), zb = smem_addr(zs);
    float acc[UPW][4];
#pragma unroll
    for (int u = 0; u < UPW; ++u)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[u][j] = 0.f;

    for (i64 c0 = v0; c0 < v1; c0 += kWgChunk) {
        __syncthreads();
        for (int i = threadIdx.x; i < kWgChunk * (XV + ZV); i += 256) {
            const bool isx = i < kWgChunk * XV;
            const int j = isx ? i : i - kWgChunk * XV;
            const int vox = isx ? j / XV : j / ZV, prt = isx ? j % XV : j % ZV;
            const i64 v = c0 + vox;
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (v < v1) {
                if (isx) {
                    const int x = (int)(v % W);
                    const i64 r = v / W;
                    const int y = (int)(r % H), z = (int)(r / H);
                    const int xx = x + ox, yy = y + oy, zz = z + oz;
                    if ((unsigned)xx < (unsigned)W && (unsigned)yy < (unsigned)H && (unsigned)zz < (unsigned)D)
                        val = __ldg(reinterpret_cast<const uint4*>(X + (((size_t)zz * H + yy) * W + xx) * CIN + prt * 8));
                } else {
                    val = __ldg(reinterpret_cast<const uint4*>(dZ + (size_t)v * COUT + prt * 8));
                }
            }
            *reinterpret_cast<uint4*>((isx ? xs + vox * XS : zs + vox * ZS) + prt * 16) = val;
        }
        __syncthreads();
        if (active) {
            for (int ks = kslot; ks < kWgChunk / 16; ks += G) {
#pragma unroll
                for (int u = 0; u < UPW; ++u) {
                    const int tile = U >= 8 ? warp + 8 * u : tile0;
                    const int mi = tile / NTL, ni = tile % NTL;
                    uint32_t a[4];
                    ldsm_x4_t(a, xb + (ks * 16 + (lane >> 4) * 8 + (lane & 7)) * XS + (mi * 16 + ((lane >> 3) & 1) * 8) * 2);
                    uint32_t b0, b1;
                    ldsm_x2_t(b0, b1, zb + (ks * 16 + ((lane >> 3) & 1) * 8 + (lane & 7)) * ZS + ni * 16);
                    mma_bf16(acc[u], a, b0, b1);
                }
            }
        }
    }
    if (G > 1) {
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 4; ++j) red[warp][lane * 4 + j] = acc[0][j];
        __syncthreads();
        if (kslot != 0 || !active) return;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float s = 0.f;
            for (int k = 0; k < G; ++k) s += red[warp + k][lane * 4 + j];
            acc[0][j] = s;
        }
    }
    if (!active) return;
    float* out = part + ((size_t)blockIdx.y * 27 + tap) * CIN * COUT;
    const int g = lane >> 2, tq = lane & 3;
#pragma unroll
    for (int u = 0; u < UPW; ++u) {
        const int tile = U >= 8 ? warp + 8 * u : tile0;
        const int ci = (tile / NTL) * 16 + g, co = (tile % NTL) * 8 + 2 * tq;
        out[ci * COUT + co] = acc[u][0];
        out[ci * COUT + co + 1] = acc[u][1];
        out[(ci + 8) * COUT + co] = acc[u][2];
        out[(ci + 8) * COUT + co + 1] = acc[u][3];
    }
}

// grad[i] += sum_s part[s][i], s in order.
__global__ void k_wgrad_sum(const float* __restrict__ part, int S, int n, float* __restrict__ grad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int k = 0; k < S; ++k) s += part[(size_t)k * n + i];
        grad[i] += s;
    }
}

// ---------------------------------------------------------------------------
// Weight layouts: forward B fragments and the transposed, tap-mirrored ones
// of the backward-data pass (W'[tap][co][ci] = W[26 - tap][ci][co]).
__global__ void k_wprep(const float* __restrict__ W, int cin, int cout, uint2* __restrict__ wf,
                        uint2* __restrict__ wt) {
    const int KC = cin / 16, NT = cout / 8, KCt = cout / 16, NTt = cin / 8;
    const int nf = 27 * KC * NT * 32, ntr = wt ? 27 * KCt * NTt * 32 : 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf + ntr; i += gridDim.x * blockDim.x) {
        const bool fwd = i < nf;
        const int j = fwd ? i : i - nf;
        const int lane = j & 31, g = lane >> 2, tq = lane & 3;
        int r = j >> 5;
        const int nt = r % (fwd ? NT : NTt);
        r /= fwd ? NT : NTt;
        const int kc = r % (fwd ? KC : KCt), tap = r / (fwd ? KC : KCt);
        if (fwd) {
            const int co = nt * 8 + g, ci = kc * 16 + 2 * tq;
            const float* base = W + (size_t)tap * cin * cout + co;
            wf[j] = make_uint2(pack_bf16(base[ci * cout], base[(ci + 1) * cout]),
                               pack_bf16(base[(ci + 8) * cout], base[(ci + 9) * cout]));
        } else {
            const int ci = nt * 8 + g, co = kc * 16 + 2 * tq;
            const float* base = W + ((size_t)(26 - tap) * cin + ci) * cout + co;
            wt[j] = make_uint2(pack_bf16(base[0], base[1]), pack_bf16(base[8], base[9]));
        }
    }
}

// ---------------------------------------------------------------------------
// Input normalisation.

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 512;

__global__ void __launch_bounds__(kRedThreads) k_sumsq(const float* __restrict__ b, i64 n, double* __restrict__ part) {
    __shared__ double sm[32];
    double s = 0.0;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const double v = b[i];
        s += v * v;
    }
    s = block_sum<kRedThreads>(s, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// scal = {s, 1/s, s * out_scale, dt / (s * out_scale)}
__global__ void k_scalars(const double* __restrict__ part, int nparts, i64 n, float out_scale, float dt,
                          float* __restrict__ scal) {
    if (threadIdx.x != 0) return;
    double ss = 0.0;
    for (int i = 0; i < nparts; ++i) ss += part[i];
    const float s = (float)sqrt(ss / (double)n);
    const float scale = __fmul_rn(s, out_scale);
    scal[0] = s;
    scal[1] = s > 0.f ? __fdiv_rn(1.f, s) : 0.f;
    scal[2] = scale;
    scal[3] = scale > 0.f ? __fdiv_rn(dt, scale) : 0.f;
}

__global__ void k_input(const float* __restrict__ b, const uint8_t* __restrict__ flags, const float* __restrict__ scal,
                        i64 n, bf16* __restrict__ X0) {
    const float inv_s = scal[1];
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (i64)gridDim.x * blockDim.x) {
        const float c0 = __fmul_rn(b[v], inv_s);
        const float c1 = __fmul_rn((float)__popc(flags[v] & 63u), 1.0f / 6.0f);
        uint4 lo = make_uint4(pack_bf16(c0, c1), 0u, 0u, 0u);
        uint4* o = reinterpret_cast<uint4*>(X0 + v * 16);
        o[0] = lo;
        o[1] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// ---------------------------------------------------------------------------
// Pooling and upsampling (fine level dims D, H, W; coarse = half).

// out[u][c] = bf16(0.125 * sum of the 8 children, in (dz, dy, dx) order)
__global__ void k_pool(const bf16* __restrict__ in, int C, int D, int H, int W, bf16* __restrict__ out) {
    const int cd = D / 2, ch = H / 2, cw = W / 2;
    const i64 n = (i64)cd * ch * cw * C;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const i64 u = i / C;
        const int x = (int)(u % cw), y = (int)((u / cw) % ch), z = (int)(u / ((i64)cw * ch));
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int fz = 2 * z + (k >> 2), fy = 2 * y + ((k >> 1) & 1), fx = 2 * x + (k & 1);
            s = __fadd_rn(s, __bfloat162float(in[(((size_t)fz * H + fy) * W + fx) * C + c]));
        }
        out[i] = __float2bfloat16_rn(__fmul_rn(0.125f, s));
    }
}

// out[v] = [coarse[parent(v)] (ca channels) | skip[v] (cb channels)], 8-channel vectors
__global__ void k_upcat(const bf16* __restrict__ coarse, int ca, const bf16* __restrict__ skip, int cb, int D, int H,
                        int W, bf16* __restrict__ out) {
    const int ct = ca + cb, nv = ct / 8;
    const i64 n = (i64)D * H * W * nv;
    const int ch = H / 2, cw = W / 2;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const int k = (int)(i % nv);
        const i64 v = i / nv;
        const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / ((i64)W * H));
        uint4 val;
        if (k * 8 < ca) {
            const i64 u = ((i64)(z / 2) * ch + y / 2) * cw + x / 2;
            val = *reinterpret_cast<const uint4*>(coarse + u * ca + k * 8);
        } else {
            val = *reinterpret_cast<const uint4*>(skip + v * cb + (k * 8 - ca));
        }
        *reinterpret_cast<uint4*>(out + v * ct + k * 8) = val;
    }
}

// dz[u][c] = y[u][c] > 0 ? bf16(sum_children dcat[child][c]) : 0, c < ca
__global__ void k_upback_gate(const bf16* __restrict__ dcat, int ct, int ca, const bf16* __restrict__ y, int D, int H,
                              int W, bf16* __restrict__ dz) {
    const int cd = D / 2, ch = H / 2, cw = W / 2;
    const i64 n = (i64)cd * ch * cw * ca;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const int c = (int)(i % ca);
        const i64 u = i / ca;
        const int x = (int)(u % cw), yy = (int)((u / cw) % ch), z = (int)(u / ((i64)cw * ch));
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int fz = 2 * z + (k >> 2), fy = 2 * yy + ((k >> 1) & 1), fx = 2 * x + (k & 1);
            s = __fadd_rn(s, __bfloat162float(dcat[(((size_t)fz * H + fy) * W + fx) * ct + c]));
        }
        dz[i] = __bfloat162float(y[i]) > 0.f ? __float2bfloat16_rn(s) : __float2bfloat16_rn(0.f);
    }
}

// dz[v][c] = y[v][c] > 0 ? bf16(dcat[v][off + c] + 0.125 * dp[parent(v)][c]) : 0
__global__ void k_poolback_gate(const bf16* __restrict__ dcat, int ct, int off, const bf16* __restrict__ dp, int C,
                                const bf16* __restrict__ y, int D, int H, int W, bf16* __restrict__ dz) {
    const i64 n = (i64)D * H * W * C;
    const int ch = H / 2, cw = W / 2;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const i64 v = i / C;
        const int x = (int)(v % W), yy = (int)((v / W) % H), z = (int)(v / ((i64)W * H));
        const i64 u = ((i64)(z / 2) * ch + yy / 2) * cw + x / 2;
        const float s = __fadd_rn(__bfloat162float(dcat[v * ct + off + c]), __fmul_rn(0.125f, __bfloat162float(dp[u * C + c])));
        dz[i] = __bfloat162float(y[i]) > 0.f ? __float2bfloat16_rn(s) : __float2bfloat16_rn(0.f);
    }
}

// ---------------------------------------------------------------------------
// Output layer, guess and loss.
//   q = sum_c y9[c] * wh[c] (0 on solid cells); p_out = q * scale / dt.
//   Training, e = q - p_true * dt / scale on open cells (0 elsewhere):
//     loss kind MSE:    L = sum e^2 / cells,        g = e
//     loss kind energy: L = sum e (A1 e) / cells,   g = A1 e  (ae input)
//   (A1 = the masked Laplacian at dt = 1: the error's energy norm, the
//   quantity CG reduces; blind to the null-space constant.)
//   dq = g * c2 (c2 = 2 / cells), dZ9[c] = y9[c] > 0 ? dq * wh[c] : 0,
//   part[block] = {dwh[16], loss}.  With e_out set, only e is written.
constexpr int kHeadThreads = 256;

__global__ void __launch_bounds__(kHeadThreads)
    k_head(const bf16* __restrict__ Y9, const uint8_t* __restrict__ flags, const float* __restrict__ wh,
           const float* __restrict__ scal, i64 n, float dt, float* __restrict__ p_out, const float* __restrict__ p_true,
           float* __restrict__ e_out, const float* __restrict__ ae, float c2, bf16* __restrict__ dZ9,
           double* __restrict__ part) {
    __shared__ double sm[32];
    float w[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) w[c] = wh[c];
    const float scale = scal[2], inv_ps = scal[3];
    const bool train = p_true && !e_out;
    double dw[16], loss = 0.0;
#pragma unroll
    for (int c = 0; c < 16; ++c) dw[c] = 0.0;
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (i64)gridDim.x * blockDim.x) {
        float y[16];
        const uint4* yp = reinterpret_cast<const uint4*>(Y9 + v * 16);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint4 u = yp[h];
            const uint32_t wds[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                __nv_bfloat162 pr;
                memcpy(&pr, &wds[k], 4);
                y[h * 8 + 2 * k] = __bfloat162float(pr.x);
                y[h * 8 + 2 * k + 1] = __bfloat162float(pr.y);
            }
        }
        float q = 0.f;
#pragma unroll
        for (int c = 0; c < 16; ++c) q = __fadd_rn(q, __fmul_rn(y[c], w[c]));
        const bool m = (flags[v] & 63u) != 0;
        if (!m) q = 0.f;
        if (p_out) p_out[v] = __fdiv_rn(__fmul_rn(q, scale), dt);
        if (!p_true) continue;
        const float e = m ? __fsub_rn(q, __fmul_rn(p_true[v], inv_ps)) : 0.f;
        if (e_out) {
            e_out[v] = e;
            continue;
        }
        const float gv = ae ? ae[v] : e;
        const float dq = m ? __fmul_rn(gv, c2) : 0.f;
        if (m) loss += (double)e * (double)gv;
        uint32_t o[8];
#pragma unroll
        for (int c = 0; c < 16; c += 2) {
            dw[c] += (double)y[c] * (double)dq;
            dw[c + 1] += (double)y[c + 1] * (double)dq;
            o[c / 2] = pack_bf16(y[c] > 0.f ? __fmul_rn(dq, w[c]) : 0.f, y[c + 1] > 0.f ? __fmul_rn(dq, w[c + 1]) : 0.f);
        }
        uint4* dp = reinterpret_cast<uint4*>(dZ9 + v * 16);
        dp[0] = make_uint4(o[0], o[1], o[2], o[3]);
        dp[1] = make_uint4(o[4], o[5], o[6], o[7]);
    }
    if (!train) return;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
        const double s = block_sum<kHeadThreads>(dw[c], sm);
        if (threadIdx.x == 0) part[blockIdx.x * 17 + c] = s;
    }
    const double s = block_sum<kHeadThreads>(loss, sm);
    if (threadIdx.x == 0) part[blockIdx.x * 17 + 16] = s;
}

// Line search of the learned guess along d for A x = b with residual r:
// part[block] = {d . r, d . Ad}; then alpha = (d.r) / (d.Ad) (0 if d.Ad <= 0),
// x += alpha d, r -= alpha Ad.
__global__ void __launch_bounds__(kRedThreads) k_dots(const float* __restrict__ d, const float* __restrict__ r,
                                                      const float* __restrict__ ad, i64 n, double* __restrict__ part) {
    __shared__ double sm[32];
    double a = 0.0, b = 0.0;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const double di = d[i];
        a += di * (double)r[i];
        b += di * (double)ad[i];
    }
    a = block_sum<kRedThreads>(a, sm);
    b = block_sum<kRedThreads>(b, sm);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

__global__ void k_alpha(const double* __restrict__ part, int nb, float* __restrict__ alpha) {
    if (threadIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (int i = 0; i < nb; ++i) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    *alpha = (b > 0.0 && isfinite(a / b)) ? (float)(a / b) : 0.f;
}

__global__ void k_step(float* __restrict__ x, float* __restrict__ r, const float* __restrict__ d,
                       const float* __restrict__ ad, const float* __restrict__ alpha, i64 n) {
    const float a = *alpha;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        x[i] = __fadd_rn(x[i], __fmul_rn(a, d[i]));
        r[i] = __fsub_rn(r[i], __fmul_rn(a, ad[i]));
    }
}

// grad_wh[c] += sum_blocks part[c]; loss_out = sum part[16] / n
__global__ void k_head_sum(const double* __restrict__ part, int nb, i64 n, float* __restrict__ grad_wh,
                           double* __restrict__ loss_out) {
    const int c = threadIdx.x;
    if (c > 16) return;
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += part[b * 17 + c];
    if (c < 16)
        grad_wh[c] += (float)s;
    else
        *loss_out = s / (double)n;
}

// ---------------------------------------------------------------------------
__global__ void k_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       i64 n, float lr, float b1, float b2, float eps, float gscale, float c1, float c2) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const float gi = g[i] * gscale;
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        g[i] = 0.f;
    }
}

}  // namespace unet
}  // namespace pg

// ---------------------------------------------------------------------------
// Host side.

using namespace pg;
using namespace pg::unet;

struct pg_unet {
    int device = 0, num_sms = 0;
    int ld[3], lh[3], lw[3];
    i64 lv[3];
    cudaStream_t stream = nullptr;
    void* arena = nullptr;
    float* params = nullptr;
    float* grads = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    uint2* wf[kL] = {};
    uint2* wt[kL] = {};
    bf16* tcf[kL] = {};  // tensor-core (tcgen05) weight layouts: forward
    bf16* tct[kL] = {};  // and backward-data
    int* err = nullptr;  // set by a kernel whose bounded wait gave up
    bool wdirty = true;
    bf16 *X0 = nullptr, *Y[kL] = {}, *P0 = nullptr, *P1 = nullptr, *C1 = nullptr, *C0 = nullptr;
    bf16 *G0a = nullptr, *G0b = nullptr, *dC0 = nullptr, *G1a = nullptr, *G1b = nullptr, *dC1 = nullptr,
         *dP0 = nullptr, *G2a = nullptr, *G2b = nullptr, *dP1 = nullptr;
    float* q = nullptr;    // guess scratch (V0)
    float* r = nullptr;    // residual scratch (V0)
    float* ad = nullptr;   // A d scratch (V0)
    int loss_kind = 1;     // 0 MSE, 1 energy norm
    float* scal = nullptr;  // 4 floats
    double* red = nullptr;  // reduction partials
    double* loss = nullptr;
    float* wpart = nullptr;
    int wslabs = 0;
    double out_scale = 1.0;
    i64 adam_t = 0;
};

namespace {

int ceil_div(i64 a, i64 b) { return (int)((a + b - 1) / b); }
int pow2_floor(int x) {
    int p = 1;
    while (p * 2 <= x) p *= 2;
    return p;
}

int blocks_for(const pg_unet* net, i64 n, int threads = 256) {
    i64 b = (n + threads - 1) / threads;
    return (int)std::max<i64>(1, std::min<i64>(b, (i64)net->num_sms * 16));
}

ConvGeom conv_geom(int D, int H, int W, int mt) {
    ConvGeom G;
    G.D = D;
    G.H = H;
    G.W = W;
    const int nv = 128 * mt;
    G.TX = std::min(32, pow2_floor(W));
    G.TY = std::min(4, pow2_floor(H));
    G.TZ = nv / (G.TX * G.TY);
    G.BX = G.TX + 2;
    G.BY = G.TY + 2;
    G.tiles_x = ceil_div(W, G.TX);
    G.tiles_y = ceil_div(H, G.TY);
    return G;
}

template <int CIN, int COUT>
int conv_t(const pg_unet* net, int lvl, const bf16* in, const uint2* w, bf16* out, const bf16* gate, int epi) {
    constexpr int MT = COUT <= 32 ? 4 : (COUT <= 64 ? 2 : 1);
    const ConvGeom G = conv_geom(net->ld[lvl], net->lh[lvl], net->lw[lvl], MT);
    const size_t smem = (size_t)G.BX * G.BY * (G.TZ + 2) * kRowBytes;
    static bool attr_set = false;
    if (!attr_set) {
        PG_CUDA(cudaFuncSetAttribute(k_conv<CIN, COUT, MT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
        attr_set = true;
    }
    if (smem > 96 * 1024) return bad_arg("pg_unet: conv tile does not fit in shared memory");
    const int nb = G.tiles_x * G.tiles_y * ceil_div(G.D, G.TZ);
    PG_LAUNCH(KK_UNET_CONV, net->stream, k_conv<CIN, COUT, MT><<<nb, kConvThreads, smem, net->stream>>>(in, w, out, gate, G, epi));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

// The tensor-core convolution: one CTA per 8 x 16 x TZ output tile; the
// launch's dynamic shared memory also caps the CTAs per SM so that their
// tensor-memory columns fit in the SM's 512.
template <int CIN, int COUT>
int conv_tc_t(const pg_unet* net, int lvl, const bf16* in, const bf16* wtc, bf16* out, const bf16* gate, int epi) {
    typedef tc::Cfg<COUT> Cf;
    static size_t smem = 0;
    if (!smem) {
        size_t s = Cf::kSmem + 128;
        PG_CUDA(cudaFuncSetAttribute(tc::k_conv_tc<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     227 * 1024));
        const int maxb = 512 / Cf::kCols;
        int bps = 0;
        PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, tc::k_conv_tc<CIN, COUT>, tc::kThreads, s));
        if (bps > maxb) {
            s = std::max(s, (size_t)(228 * 1024 / (maxb + 1) - 1024 + 128));
            PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, tc::k_conv_tc<CIN, COUT>, tc::kThreads, s));
        }
        if (bps < 1 || bps > maxb) return bad_arg("pg_unet: tensor-core conv does not fit an SM");
        smem = s;
    }
    tc::Geom G;
    G.D = net->ld[lvl];
    G.H = net->lh[lvl];
    G.W = net->lw[lvl];
    G.tiles_x = ceil_div(G.W, tc::TX);
    G.tiles_y = ceil_div(G.H, tc::TY);
    const int nb = G.tiles_x * G.tiles_y * ceil_div(G.D, Cf::TZ);
    PG_LAUNCH(KK_UNET_CONV, net->stream,
              tc::k_conv_tc<CIN, COUT><<<nb, tc::kThreads, smem, net->stream>>>(in, wtc, out, gate, G, epi, net->err));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

// The tensor-core path unless PG_UNET_TC=0 (a diagnostic switch: the legacy
// warp-level mma.sync kernel, kept for comparison).
bool tc_enabled() {
    const char* env = getenv("PG_UNET_TC");
    return !(env && env[0] == '0');
}

int conv(const pg_unet* net, int lvl, int cin, int cout, const bf16* in, const uint2* w, const bf16* wtc, bf16* out,
         const bf16* gate, int epi) {
    if (tc_enabled()) {
#define PG_UNET_CONV_TC(A, B) \
    if (cin == A && cout == B) return conv_tc_t<A, B>(net, lvl, in, wtc, out, gate, epi);
        PG_UNET_CONV_TC(16, 16)
        PG_UNET_CONV_TC(16, 32)
        PG_UNET_CONV_TC(32, 32)
        PG_UNET_CONV_TC(32, 64)
        PG_UNET_CONV_TC(64, 64)
        PG_UNET_CONV_TC(96, 32)
        PG_UNET_CONV_TC(48, 16)
        PG_UNET_CONV_TC(16, 48)
        PG_UNET_CONV_TC(32, 96)
        PG_UNET_CONV_TC(64, 32)
        PG_UNET_CONV_TC(32, 16)
#undef PG_UNET_CONV_TC
        return bad_arg("pg_unet: no conv kernel for this channel pair");
    }
#define PG_UNET_CONV(A, B) \
    if (cin == A && cout == B) return conv_t<A, B>(net, lvl, in, w, out, gate, epi);
    PG_UNET_CONV(16, 16)
    PG_UNET_CONV(16, 32)
    PG_UNET_CONV(32, 32)
    PG_UNET_CONV(32, 64)
    PG_UNET_CONV(64, 64)
    PG_UNET_CONV(96, 32)
    PG_UNET_CONV(48, 16)
    PG_UNET_CONV(16, 48)
    PG_UNET_CONV(32, 96)
    PG_UNET_CONV(64, 32)
    PG_UNET_CONV(32, 16)
#undef PG_UNET_CONV
    return bad_arg("pg_unet: no conv kernel for this channel pair");
}

template <int CIN, int COUT>
int wgrad_t(pg_unet* net, int lvl, const bf16* X, const bf16* dZ, float* grad) {
    const int D = net->ld[lvl], H = net->lh[lvl], W = net->lw[lvl];
    const i64 V = net->lv[lvl];
    int S = std::max(1, std::min(net->wslabs, ceil_div(V, kWgChunk)));
    const i64 slab = (i64)ceil_div(ceil_div(V, S), kWgChunk) * kWgChunk;
    S = ceil_div(V, slab);
    const int n = 27 * CIN * COUT;
    PG_LAUNCH(KK_UNET_WGRAD, net->stream, k_wgrad<CIN, COUT><<<dim3(27, S), 256, 0, net->stream>>>(X, dZ, net->wpart, D, H, W, slab));
    PG_LAUNCH(KK_UNET_WGRAD, net->stream, k_wgrad_sum<<<ceil_div(n, 256), 256, 0, net->stream>>>(net->wpart, S, n, grad));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

int wgrad(pg_unet* net, int k, const bf16* X, const bf16* dZ) {
    float* grad = net->grads + param_offset(k);
    const int lvl = kLevel[k];
#define PG_UNET_WG(A, B) \
    if (kCin[k] == A && kCout[k] == B) return wgrad_t<A, B>(net, lvl, X, dZ, grad);
    PG_UNET_WG(16, 16)
    PG_UNET_WG(16, 32)
    PG_UNET_WG(32, 32)
    PG_UNET_WG(32, 64)
    PG_UNET_WG(64, 64)
    PG_UNET_WG(96, 32)
    PG_UNET_WG(48, 16)
#undef PG_UNET_WG
    return bad_arg("pg_unet: no weight-gradient kernel for this layer");
}

int prep_weights(pg_unet* net) {
    if (!net->wdirty) return PG_OK;
    for (int k = 0; k < kL; ++k) {
        const int n = 27 * kCin[k] * kCout[k] / 2;  // both layouts: 2 x (27 * cin/16 * cout/8 * 32)
        PG_LAUNCH(KK_UNET_MISC, net->stream,
                  k_wprep<<<ceil_div(n, 256), 256, 0, net->stream>>>(net->params + param_offset(k), kCin[k], kCout[k],
                                                                      net->wf[k], k ? net->wt[k] : nullptr));
        const int nt = 27 * kCin[k] * kCout[k];
        PG_LAUNCH(KK_UNET_MISC, net->stream,
                  tc::k_wprep_tc<<<ceil_div(nt, 256), 256, 0, net->stream>>>(net->params + param_offset(k), kCin[k],
                                                                              kCout[k], 0, net->tcf[k]));
        if (k)
            PG_LAUNCH(KK_UNET_MISC, net->stream,
                      tc::k_wprep_tc<<<ceil_div(nt, 256), 256, 0, net->stream>>>(net->params + param_offset(k), kCin[k],
                                                                                  kCout[k], 1, net->tct[k]));
    }
    PG_CHECK_LAUNCH();
    net->wdirty = false;
    return PG_OK;
}

// PG_TIMEOUT (and the flag cleared) when a tensor-core wait gave up since
// the last check; synchronous.
int check_err(pg_unet* net) {
    int e = 0;
    PG_CUDA(cudaMemcpy(&e, net->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (!e) return PG_OK;
    PG_CUDA(cudaMemset(net->err, 0, sizeof(int)));
    set_error("pg_unet: a wait for the tensor cores gave up; the network's last results are not to be trusted");
    return PG_TIMEOUT;
}

int check_grid(const pg_unet* net, const pg_grid* g) {
    if (!g) return bad_arg("pg_unet: NULL grid");
    if (g->dims.nd != 3 || g->dims.d != net->ld[0] || g->dims.h != net->lh[0] || g->dims.w != net->lw[0])
        return bad_arg("pg_unet: grid shape differs from the network's");
    return PG_OK;
}

// Normalise b, run the encoder/decoder; Y[9] holds the last features.
int forward(pg_unet* net, const pg_grid* g, const float* b, double dt) {
    int rc;
    if ((rc = prep_weights(net))) return rc;
    const i64 V0 = net->lv[0];
    cudaStream_t s = net->stream;
    PG_LAUNCH(KK_UNET_MISC, s, k_sumsq<<<kRedBlocks, kRedThreads, 0, s>>>(b, V0, net->red));
    PG_LAUNCH(KK_UNET_MISC, s, k_scalars<<<1, 32, 0, s>>>(net->red, kRedBlocks, V0, (float)net->out_scale, (float)dt, net->scal));
    PG_LAUNCH(KK_UNET_MISC, s, k_input<<<blocks_for(net, V0), 256, 0, s>>>(b, g->flags, net->scal, V0, net->X0));
    PG_CHECK_LAUNCH();
    auto C = [&](int k, const bf16* in) {
        return conv(net, kLevel[k], kCin[k], kCout[k], in, net->wf[k], net->tcf[k], net->Y[k], nullptr, EPI_RELU);
    };
    if ((rc = C(0, net->X0)) || (rc = C(1, net->Y[0]))) return rc;
    PG_LAUNCH(KK_UNET_MISC, s, k_pool<<<blocks_for(net, net->lv[1] * 16), 256, 0, s>>>(net->Y[1], 16, net->ld[0], net->lh[0], net->lw[0], net->P0));
    if ((rc = C(2, net->P0)) || (rc = C(3, net->Y[2]))) return rc;
    PG_LAUNCH(KK_UNET_MISC, s, k_pool<<<blocks_for(net, net->lv[2] * 32), 256, 0, s>>>(net->Y[3], 32, net->ld[1], net->lh[1], net->lw[1], net->P1));
    if ((rc = C(4, net->P1)) || (rc = C(5, net->Y[4]))) return rc;
    PG_LAUNCH(KK_UNET_MISC, s, k_upcat<<<blocks_for(net, net->lv[1] * 12), 256, 0, s>>>(net->Y[5], 64, net->Y[3], 32, net->ld[1], net->lh[1], net->lw[1], net->C1));
    if ((rc = C(6, net->C1)) || (rc = C(7, net->Y[6]))) return rc;
    PG_LAUNCH(KK_UNET_MISC, s, k_upcat<<<blocks_for(net, net->lv[0] * 6), 256, 0, s>>>(net->Y[7], 32, net->Y[1], 16, net->ld[0], net->lh[0], net->lw[0], net->C0));
    if ((rc = C(8, net->C0)) || (rc = C(9, net->Y[8]))) return rc;
    PG_CHECK_LAUNCH();
    return PG_OK;
}

int backward(pg_unet* net) {
    int rc;
    cudaStream_t s = net->stream;
    const int d0 = net->ld[0], h0 = net->lh[0], w0 = net->lw[0];
    const int d1 = net->ld[1], h1 = net->lh[1], w1 = net->lw[1];
    auto BD = [&](int k, const bf16* dz, bf16* out, const bf16* gate, int epi) {
        return conv(net, kLevel[k], kCout[k], kCin[k], dz, net->wt[k], net->tct[k], out, gate, epi);
    };
    // level 0 decoder: dZ9 = G0a (from k_head)
    if ((rc = wgrad(net, 9, net->Y[8], net->G0a)) || (rc = BD(9, net->G0a, net->G0b, net->Y[8], EPI_GATE))) return rc;
    if ((rc = wgrad(net, 8, net->C0, net->G0b)) || (rc = BD(8, net->G0b, net->dC0, nullptr, EPI_NONE))) return rc;
    PG_LAUNCH(KK_UNET_MISC, s, k_upback_gate<<<blocks_for(net, net->lv[1] * 32), 256, 0, s>>>(net->dC0, 48, 32, net->Y[7], d0, h0, w0, net->G1a));
    // level 1 decoder
    if ((rc = wgrad(net, 7, net->Y[6], net->G1a)) || (rc = BD(7, net->G1a, net->G1b, net->Y[6], EPI_GATE))) return rc;
    if ((rc = wgrad(net, 6, net->C1, net->G1b)) || (rc = BD(6, net->G1b, net->dC1, nullptr, EPI_NONE))) return rc;
    PG_LAUNCH(KK_UNET_MISC, s, k_upback_gate<<<blocks_for(net, net->lv[2] * 64), 256, 0, s>>>(net->dC1, 96, 64, net->Y[5], d1, h1, w1, net->G2a));
    // level 2
    if ((rc = wgrad(net, 5, net->Y[4], net->G2a)) || (rc = BD(5, net->G2a, net->G2b, net->Y[4], EPI_GATE))) return rc;
    if ((rc = wgrad(net, 4, net->P1, net->G2b)) || (rc = BD(4, net->G2b, net->dP1, nullptr, EPI_NONE))) return rc;
    PG_LAUNCH(KK_UNET_MISC, s, k_poolback_gate<<<blocks_for(net, net->lv[1] * 32), 256, 0, s>>>(net->dC1, 96, 64, net->dP1, 32, net->Y[3], d1, h1, w1, net->G1a));
    // level 1 encoder
    if ((rc = wgrad(net, 3, net->Y[2], net->G1a)) || (rc = BD(3, net->G1a, net->G1b, net->Y[2], EPI_GATE))) return rc;
    if ((rc = wgrad(net, 2, net->P0, net->G1b)) || (rc = BD(2, net->G1b, net->dP0, nullptr, EPI_NONE))) return rc;
    PG_LAUNCH(KK_UNET_MISC, s, k_poolback_gate<<<blocks_for(net, net->lv[0] * 16), 256, 0, s>>>(net->dC0, 48, 32, net->dP0, 16, net->Y[1], d0, h0, w0, net->G0a));
    // level 0 encoder
    if ((rc = wgrad(net, 1, net->Y[0], net->G0a)) || (rc = BD(1, net->G0a, net->G0b, net->Y[0], EPI_GATE))) return rc;
    if ((rc = wgrad(net, 0, net->X0, net->G0b))) return rc;
    PG_CHECK_LAUNCH();
    return PG_OK;
}

constexpr int kHeadBlocks = 256;

// out = A in on the network's stream (A = dt * the grid's masked Laplacian).
int apply_a(pg_unet* net, const pg_grid* g, float* out, const float* in, double dt) {
    pg_grid* gm = const_cast<pg_grid*>(g);
    cudaStream_t saved = gm->stream;
    gm->stream = net->stream;
    const int rc = launch_laplacian<float>(gm, out, in, dt);
    gm->stream = saved;
    return rc;
}

int head(pg_unet* net, const pg_grid* g, double dt, float* p_out, const float* p_true) {
    const i64 V0 = net->lv[0];
    const float c2 = 2.0f / (float)V0;
    cudaStream_t s = net->stream;
    const int nb = (int)std::min<i64>(kHeadBlocks, std::max<i64>(1, (V0 + kHeadThreads - 1) / kHeadThreads));
    const float* wh = net->params + param_offset(kL);
    const float* ae = nullptr;
    if (p_true && net->loss_kind == 1) {
        // e = q - t, then A1 e (dt = 1) into the scratch ad
        PG_LAUNCH(KK_UNET_MISC, s, k_head<<<nb, kHeadThreads, 0, s>>>(net->Y[9], g->flags, wh, net->scal, V0, (float)dt, nullptr, p_true, net->r, nullptr, c2, net->G0a, net->red));
        int rc;
        if ((rc = apply_a(net, g, net->ad, net->r, 1.0))) return rc;
        ae = net->ad;
    }
    PG_LAUNCH(KK_UNET_MISC, s, k_head<<<nb, kHeadThreads, 0, s>>>(net->Y[9], g->flags, wh, net->scal, V0, (float)dt, p_out, p_true, nullptr, ae, c2, net->G0a, net->red));
    if (p_true)
        PG_LAUNCH(KK_UNET_MISC, s, k_head_sum<<<1, 32, 0, s>>>(net->red, nb, V0, net->grads + param_offset(kL), net->loss));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

// ---------------------------------------------------------------------------
// The network as a preconditioner correction inside the CG.  For a residual
// r: q = net(r), a = (q.r) / (q.Aq) (0 when q.Aq <= 0; the step along q that
// minimises the error's energy norm), then one Jacobi step on what that
// leaves:
//     z = M(r) = a q + D^-1 (r - a A q).
// M is not linear in r (a and the network depend on r), so the CG is the
// flexible one: beta is the Polak-Ribiere ratio z'.(r' - r) / (z.r), which
// with r' - r = -alpha A p is -alpha (z'.Ap) / (z.r) -- read from the A p
// vector the iteration just used, with no copy of the previous residual.

__global__ void k_lp_z(float* __restrict__ z, const float* __restrict__ r, const float* __restrict__ q,
                       const float* __restrict__ aq, const uint8_t* __restrict__ flags, const float* __restrict__ alpha,
                       i64 n, float dt, const CgState* st) {
    if (st->done) return;
    const float a = *alpha;
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (i64)gridDim.x * blockDim.x) {
        const int open = __popc((unsigned)flags[v] & 63u);
        const float inv = open ? __frcp_rn((float)open * dt) : 0.f;
        z[v] = fmaf(a, q[v], (r[v] - a * aq[v]) * inv);
    }
}

// z.r and z.Ap (compensated FP32 per thread, FP64 across), then the last
// block folds them into the CG state: sigma = z.r; after the first
// iteration beta = -alpha (z.Ap) / sigma_old.
__global__ void __launch_bounds__(kRedThreads)
    k_lp_fold(const float* __restrict__ z, const float* __restrict__ r, const float* __restrict__ ap, i64 n,
              CgState* st, double* partials) {
    if (st->done) return;
    __shared__ double sm[32];
    Acc<float> zr, zap;
    const bool first = st->iter == 0;
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (i64)gridDim.x * blockDim.x) {
        const float zv = z[v];
        zr.add(zv * r[v]);
        if (!first) zap.add(zv * ap[v]);
    }
    const double s1 = block_sum<kRedThreads>(zr.value(), sm);
    const double s2 = block_sum<kRedThreads>(zap.value(), sm);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = s1;
        partials[kMaxBlocks + blockIdx.x] = s2;
    }
    if (!last_block(&st->counter[3])) return;
    const double rz = reduce_partials<false, kRedThreads>(partials, gridDim.x, sm);
    const double za = reduce_partials<false, kRedThreads>(partials + kMaxBlocks, gridDim.x, sm);
    if (threadIdx.x == 0) {
        st->counter[3] = 0;
        if (!isfinite(rz) || !isfinite(za)) {
            st->status = PG_NAN_DETECTED;
            st->done = 1;
        } else if (!(rz > 0.0)) {  // M(r) is not a descent direction for r
            st->status = PG_BREAKDOWN;
            st->done = 1;
        } else if (first) {
            st->sigma = rz;
        } else {
            st->beta = -st->alpha * za / st->sigma;
            st->sigma = rz;
            st->first = 0;
        }
    }
}

struct LearnedHook : ZHook {
    pg_unet* net = nullptr;
    double dt = 1.0;
    const float* ap = nullptr;
    void bind(const void* p) override { ap = (const float*)p; }
    uintptr_t key() const override { return (uintptr_t)net ^ (uintptr_t)0x9e3779b97f4a7c15ull; }
    int apply(pg_grid* g, const void* rv, void* zv) override {
        const float* r = (const float*)rv;
        float* z = (float*)zv;
        const i64 V0 = net->lv[0];
        // the network's kernels run on the CG's stream (a graph capture's)
        cudaStream_t saved = net->stream;
        net->stream = g->stream;
        cudaStream_t s = g->stream;
        float* alpha = net->scal + 5;
        int rc = forward(net, g, r, dt);
        if (!rc) rc = head(net, g, dt, net->q, nullptr);
        if (!rc) rc = apply_a(net, g, net->ad, net->q, dt);
        if (!rc) {
            PG_LAUNCH(KK_UNET_MISC, s, k_dots<<<kRedBlocks, kRedThreads, 0, s>>>(net->q, r, net->ad, V0, net->red));
            PG_LAUNCH(KK_UNET_MISC, s, k_alpha<<<1, 32, 0, s>>>(net->red, kRedBlocks, alpha));
            PG_LAUNCH(KK_UNET_MISC, s,
                      k_lp_z<<<blocks_for(net, V0), 256, 0, s>>>(z, r, net->q, net->ad, g->flags, alpha, V0,
                                                                 (float)dt, g->ws.state));
            const int nb = (int)std::min<i64>(kRedBlocks, std::max<i64>(1, (V0 + kRedThreads - 1) / kRedThreads));
            PG_LAUNCH(KK_UNET_MISC, s,
                      k_lp_fold<<<nb, kRedThreads, 0, s>>>(z, r, ap, V0, g->ws.state, g->ws.partials));
            const cudaError_t e = cudaPeekAtLastError();
            if (e != cudaSuccess) rc = cuda_fail(e, "learned preconditioner launch");
        }
        net->stream = saved;
        return rc;
    }
};

}  // namespace

extern "C" {

int64_t pg_unet_num_params(void) { return num_params(); }

int pg_unet_create(int64_t d, int64_t h, int64_t w, pg_unet** out) {
    if (!out) return bad_arg("pg_unet_create: NULL out");
    *out = nullptr;
    if (d < 16 || h < 16 || w < 16 || d % 4 || h % 4 || w % 4)
        return bad_arg("pg_unet_create: every side must be a multiple of 4 and >= 16");
    if (d * h * w * 48 >= ((int64_t)1 << 31)) return bad_arg("pg_unet_create: grid too large");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        set_error("pg_unet_create: no CUDA device");
        return PG_NO_DEVICE;
    }
    pg_unet* net = new (std::nothrow) pg_unet();
    if (!net) return PG_OUT_OF_MEMORY;
    PG_CUDA(cudaGetDevice(&net->device));
    PG_CUDA(cudaDeviceGetAttribute(&net->num_sms, cudaDevAttrMultiProcessorCount, net->device));
    for (int l = 0; l < 3; ++l) {
        net->ld[l] = (int)(d >> l);
        net->lh[l] = (int)(h >> l);
        net->lw[l] = (int)(w >> l);
        net->lv[l] = (i64)net->ld[l] * net->lh[l] * net->lw[l];
    }
    const i64 P = num_params();
    net->wslabs = std::max(1, 4 * net->num_sms / 27);
    // Arena layout (256-byte aligned pieces).
    std::vector<std::pair<void**, size_t>> parts;
    auto add = [&](void** p, size_t bytes) { parts.push_back({p, (bytes + 255) & ~(size_t)255}); };
    add((void**)&net->params, 4 * P);
    add((void**)&net->grads, 4 * P);
    add((void**)&net->adam_m, 4 * P);
    add((void**)&net->adam_v, 4 * P);
    for (int k = 0; k < kL; ++k) {
        add((void**)&net->wf[k], 8 * (size_t)27 * kCin[k] * kCout[k] / 4);
        if (k) add((void**)&net->wt[k], 8 * (size_t)27 * kCin[k] * kCout[k] / 4);
        add((void**)&net->tcf[k], 2 * (size_t)27 * kCin[k] * kCout[k]);
        if (k) add((void**)&net->tct[k], 2 * (size_t)27 * kCin[k] * kCout[k]);
    }
    add((void**)&net->err, sizeof(int));
    const i64 V0 = net->lv[0], V1 = net->lv[1], V2 = net->lv[2];
    add((void**)&net->X0, 2 * V0 * 16);
    for (int k = 0; k < kL; ++k) add((void**)&net->Y[k], 2 * (size_t)net->lv[kLevel[k]] * kCout[k]);
    add((void**)&net->P0, 2 * V1 * 16);
    add((void**)&net->P1, 2 * V2 * 32);
    add((void**)&net->C1, 2 * V1 * 96);
    add((void**)&net->C0, 2 * V0 * 48);
    add((void**)&net->G0a, 2 * V0 * 16);
    add((void**)&net->G0b, 2 * V0 * 16);
    add((void**)&net->dC0, 2 * V0 * 48);
    add((void**)&net->G1a, 2 * V1 * 32);
    add((void**)&net->G1b, 2 * V1 * 32);
    add((void**)&net->dC1, 2 * V1 * 96);
    add((void**)&net->dP0, 2 * V1 * 16);
    add((void**)&net->G2a, 2 * V2 * 64);
    add((void**)&net->G2b, 2 * V2 * 64);
    add((void**)&net->dP1, 2 * V2 * 32);
    add((void**)&net->q, 4 * V0);
    add((void**)&net->r, 4 * V0);
    add((void**)&net->ad, 4 * V0);
    add((void**)&net->scal, 32);
    add((void**)&net->red, 8 * std::max(kRedBlocks, kHeadBlocks * 17));
    add((void**)&net->loss, 8);
    add((void**)&net->wpart, 4 * (size_t)net->wslabs * 27 * 96 * 64);
    size_t total = 0;
    for (auto& p : parts) total += p.second;
    cudaError_t e = cudaMalloc(&net->arena, total);
    if (e != cudaSuccess) {
        delete net;
        set_error("pg_unet_create: cudaMalloc failed");
        return e == cudaErrorMemoryAllocation ? PG_OUT_OF_MEMORY : PG_CUDA_ERROR;
    }
    char* base = (char*)net->arena;
    for (auto& p : parts) {
        *p.first = base;
        base += p.second;
    }
    PG_CUDA(cudaMemset(net->arena, 0, total));
    *out = net;
    return PG_OK;
}

int pg_unet_destroy(pg_unet* net) {
    if (!net) return PG_OK;
    if (net->arena) cudaFree(net->arena);
    delete net;
    return PG_OK;
}

int pg_unet_set_stream(pg_unet* net, void* stream) {
    if (!net) return bad_arg("pg_unet_set_stream: NULL net");
    net->stream = (cudaStream_t)stream;
    return PG_OK;
}

int pg_unet_set_params(pg_unet* net, const float* host, double out_scale) {
    if (!net || !host) return bad_arg("pg_unet_set_params: NULL argument");
    if (!(out_scale > 0.0) || !std::isfinite(out_scale)) return bad_arg("pg_unet_set_params: out_scale must be > 0");
    const i64 P = num_params();
    PG_CUDA(cudaMemcpyAsync(net->params, host, 4 * P, cudaMemcpyHostToDevice, net->stream));
    PG_CUDA(cudaMemsetAsync(net->grads, 0, 4 * P, net->stream));
    PG_CUDA(cudaMemsetAsync(net->adam_m, 0, 4 * P, net->stream));
    PG_CUDA(cudaMemsetAsync(net->adam_v, 0, 4 * P, net->stream));
    PG_CUDA(cudaStreamSynchronize(net->stream));
    net->out_scale = out_scale;
    net->adam_t = 0;
    net->wdirty = true;
    return PG_OK;
}

int pg_unet_get_params(const pg_unet* net, float* host, double* out_scale) {
    if (!net) return bad_arg("pg_unet_get_params: NULL net");
    if (host) {
        PG_CUDA(cudaMemcpyAsync(host, net->params, 4 * num_params(), cudaMemcpyDeviceToHost, net->stream));
        PG_CUDA(cudaStreamSynchronize(net->stream));
    }
    if (out_scale) *out_scale = net->out_scale;
    return PG_OK;
}

int pg_unet_get_grads(const pg_unet* net, float* host) {
    if (!net || !host) return bad_arg("pg_unet_get_grads: NULL argument");
    PG_CUDA(cudaMemcpyAsync(host, net->grads, 4 * num_params(), cudaMemcpyDeviceToHost, net->stream));
    PG_CUDA(cudaStreamSynchronize(net->stream));
    return PG_OK;
}

int pg_unet_zero_grads(pg_unet* net) {
    if (!net) return bad_arg("pg_unet_zero_grads: NULL net");
    PG_CUDA(cudaMemsetAsync(net->grads, 0, 4 * num_params(), net->stream));
    return PG_OK;
}

int pg_unet_accumulate_f32(pg_unet* net, const pg_grid* g, const float* b, const float* p_true, double dt,
                           double* loss) {
    if (!net || !b || !p_true) return bad_arg("pg_unet_accumulate_f32: NULL argument");
    if (!(dt > 0.0)) return bad_arg("pg_unet_accumulate_f32: dt must be > 0");
    int rc;
    if ((rc = check_grid(net, g))) return rc;
    if ((rc = forward(net, g, b, dt)) || (rc = head(net, g, dt, nullptr, p_true)) || (rc = backward(net))) return rc;
    if (loss) {
        PG_CUDA(cudaMemcpyAsync(loss, net->loss, sizeof(double), cudaMemcpyDeviceToHost, net->stream));
        PG_CUDA(cudaStreamSynchronize(net->stream));
        return check_err(net);
    }
    return PG_OK;
}

int pg_unet_check(pg_unet* net) {
    if (!net) return bad_arg("pg_unet_check: NULL network");
    PG_CUDA(cudaStreamSynchronize(net->stream));
    return check_err(net);
}

int pg_unet_adam_step(pg_unet* net, const pg_adam_params* a) {
    if (!net || !a) return bad_arg("pg_unet_adam_step: NULL argument");
    net->adam_t += 1;
    const double c1 = 1.0 / (1.0 - std::pow(a->beta1, (double)net->adam_t));
    const double c2 = 1.0 / (1.0 - std::pow(a->beta2, (double)net->adam_t));
    const i64 P = num_params();
    PG_LAUNCH(KK_UNET_MISC, net->stream,
              k_adam<<<blocks_for(net, P), 256, 0, net->stream>>>(net->params, net->grads, net->adam_m, net->adam_v, P,
                                                                  (float)a->lr, (float)a->beta1, (float)a->beta2,
                                                                  (float)a->eps, (float)a->grad_scale, (float)c1,
                                                                  (float)c2));
    PG_CHECK_LAUNCH();
    net->wdirty = true;
    return PG_OK;
}

int pg_unet_set_loss(pg_unet* net, int kind) {
    if (!net) return bad_arg("pg_unet_set_loss: NULL net");
    if (kind != 0 && kind != 1) return bad_arg("pg_unet_set_loss: kind must be 0 (MSE) or 1 (energy norm)");
    net->loss_kind = kind;
    return PG_OK;
}

int pg_unet_forward_f32(pg_unet* net, const pg_grid* g, const float* b, double dt, float* p) {
    if (!net || !b || !p) return bad_arg("pg_unet_forward_f32: NULL argument");
    if (!(dt > 0.0)) return bad_arg("pg_unet_forward_f32: dt must be > 0");
    int rc;
    if ((rc = check_grid(net, g))) return rc;
    if ((rc = forward(net, g, b, dt)) || (rc = head(net, g, dt, p, nullptr))) return rc;
    return PG_OK;
}

int pg_unet_guess_f32(pg_unet* net, const pg_grid* g, const float* b, double dt, int corrections, float* x) {
    if (!net || !b || !x) return bad_arg("pg_unet_guess_f32: NULL argument");
    if (!(dt > 0.0)) return bad_arg("pg_unet_guess_f32: dt must be > 0");
    if (corrections < 0 || corrections > 16) return bad_arg("pg_unet_guess_f32: corrections must be in 0..16");
    if (x == b) return bad_arg("pg_unet_guess_f32: x must not alias b");
    int rc;
    if ((rc = check_grid(net, g))) return rc;
    const i64 V0 = net->lv[0];
    cudaStream_t s = net->stream;
    PG_CUDA(cudaMemsetAsync(x, 0, 4 * V0, s));
    PG_CUDA(cudaMemcpyAsync(net->r, b, 4 * V0, cudaMemcpyDeviceToDevice, s));
    float* alpha = net->scal + 4;
    for (int c = 0; c <= corrections; ++c) {
        // d = net(r); x += alpha d, r -= alpha A d with the A-optimal alpha.
        if ((rc = forward(net, g, net->r, dt)) || (rc = head(net, g, dt, net->q, nullptr))) return rc;
        if ((rc = apply_a(net, g, net->ad, net->q, dt))) return rc;
        PG_LAUNCH(KK_UNET_MISC, s, k_dots<<<kRedBlocks, kRedThreads, 0, s>>>(net->q, net->r, net->ad, V0, net->red));
        PG_LAUNCH(KK_UNET_MISC, s, k_alpha<<<1, 32, 0, s>>>(net->red, kRedBlocks, alpha));
        PG_LAUNCH(KK_UNET_MISC, s, k_step<<<blocks_for(net, V0), 256, 0, s>>>(x, net->r, net->q, net->ad, alpha, V0));
    }
    PG_CHECK_LAUNCH();
    return PG_OK;
}


// z = the learned correction (see LearnedHook) inside a flexible CG, with or
// without FP64-class refinement as params say.
int pg_solve_pressure_learned_f32(const pg_grid* g, const pg_solver_params* prm, pg_unet* net, float* x,
                                  const float* b, double dt, pg_pcg_stats* stats) {
    if (!g || !prm || !net || !x || !b) return bad_arg("pg_solve_pressure_learned_f32: NULL argument");
    if (!(dt > 0.0)) return bad_arg("pg_solve_pressure_learned_f32: dt must be > 0");
    int rc;
    if ((rc = check_grid(net, g))) return rc;
    if ((rc = prep_weights(net))) return rc;  // outside any capture of the CG loop
    LearnedHook hook;
    hook.net = net;
    hook.dt = dt;
    pg_pcg_stats s{};
    if ((rc = solve_pressure_hooked(const_cast<pg_grid*>(g), prm, x, b, dt, &hook, &s))) return rc;
    if ((rc = check_err(net))) return rc;
    if (stats) *stats = s;
    return s.status;
}

}  // extern "C"
