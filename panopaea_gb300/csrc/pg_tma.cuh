// pg_tma.cuh -- tensor-memory-accelerator (TMA) plane loads and mbarrier
// waits for the z-marching stencil kernels.
//
// A kernel stages each z plane of a field (a 2D box with a halo) into
// shared memory with one cp.async.bulk.tensor per array; an mbarrier per
// pipeline stage counts the transaction bytes.  Boxes may start at negative
// or out-of-range coordinates: the TMA unit fills those elements with zeros,
// which is how grid edges are handled.  The innermost coordinate of every
// load is a multiple of 16 bytes (callers round x down), and every wait is
// bounded: after kMbarSpinLimit polls it gives up and reports failure.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>

#include "pg_internal.cuh"

namespace pg {

constexpr unsigned kMbarSpinLimit = 1u << 22;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make barrier initialisation visible to the async (TMA) proxy; follow
// with __syncthreads before any thread waits or any copy is issued.
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Poll budget of the pipeline-stage waits below: kMbarSpinLimit, or 0 set
// through pg_debug_set_stage_wait_polls, with which every stage wait gives
// up at once -- the way a test drives the give-up path (drain the copies in
// flight, report PG_TIMEOUT) without any fault.  Each translation unit that
// waits keeps its own copy (set_stage_wait_polls_* below).
static __constant__ unsigned c_stage_wait_polls = kMbarSpinLimit;

// Wait for the phase with the given parity to complete; false once the poll
// budget or kMbarWaitNs nanoseconds have passed.
constexpr uint64_t kMbarWaitNs = 500000000ull;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    const unsigned limit = c_stage_wait_polls;
    if (limit == 0) return false;
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (unsigned k = 0; k < limit; ++k) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((k & 255) == 255 && global_ns() - t0 > kMbarWaitNs) return false;
    }
    return false;
}

// Host: the stage-wait poll budget of pg_spmv.cu's and pg_mg.cu's kernels.
int set_stage_wait_polls_spmv(unsigned polls);
int set_stage_wait_polls_mg(unsigned polls);

// 3D tiled load of the box at (x, y, z) into shared memory, completing on bar.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// An L2 policy that keeps the lines it is attached to over lines of normal
// priority (a hint: they are still evicted when L2 holds nothing else).
__device__ __forceinline__ uint64_t l2_evict_last() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// tma_load_3d with an L2 cache policy for the lines it reads.
__device__ __forceinline__ void tma_load_3d_hint(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y,
                                                 int z, uint64_t policy) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint"
        " [%0], [%1, {%2, %3, %4}], [%5], %6;" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

__device__ __forceinline__ void tma_prefetch_map(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

// Work split of the z-marching kernels: the ntiles * d plane-tiles of a
// grid, ordered tile by tile (each tile's column of planes in z order), are
// cut into gridDim.x equal contiguous ranges, so every block of a launch
// sized to the resident blocks has the same number of planes to compute.  A
// block walks its range as one item per tile column it touches: planes
// [z0, z1) of tile `tile`.
struct ZWalk {
    int pos, hi, d;
    __device__ __forceinline__ ZWalk(int ntiles, int d_) : d(d_) {
        const i64 total = (i64)ntiles * d_;
        pos = (int)(total * blockIdx.x / gridDim.x);
        hi = (int)(total * (blockIdx.x + 1) / gridDim.x);
    }
    __device__ __forceinline__ bool next(int& tile, int& z0, int& z1) {
        if (pos >= hi) return false;
        tile = pos / d;
        z0 = pos - tile * d;
        z1 = min(d, z0 + (hi - pos));
        pos += z1 - z0;
        return true;
    }
};

// Blocks of a z-marching launch: every resident block (cap), but no fewer
// than kZMinPlanes planes per block.
constexpr int kZMinPlanes = 8;
inline int zwalk_blocks(int ntiles, i64 d, int cap) {
    const i64 total = (i64)ntiles * d;
    i64 nb = total / kZMinPlanes;
    if (nb > cap) nb = cap;
    return nb < 1 ? 1 : (int)nb;
}

// Host: encode a 3D tiled map over a dense (d, h, w) array of elem-byte
// elements with box (bx, by, 1); false when the CUDA driver rejects it (base,
// stride or box alignment) -- callers then use their non-TMA path.
bool encode_map_3d(CUtensorMap* map, const void* base, int elem, i64 w, i64 h, i64 d, int bx, int by);

}  // namespace pg
