// pg_pocket.cu -- disconnected fluid components for the multigrid
// preconditioner.
//
// Solid cells can cut the fluid of a grid into several connected
// components.  On each one the masked Laplacian has the constant as a null
// vector, and the right-hand side's sum over the component is zero only up
// to FP32 rounding.  A multigrid V-cycle (Gauss-Seidel sweeps and the
// coarse solve integrate whatever constant the residual carries) turns that
// into search directions with a null-space constant: on a small pocket the
// constant grows until alpha blows up and the CG diverges; on the large
// component it pollutes the FP32 product A p (a large constant plus a small
// variation) until the recursive residual stalls at a floor.  So on grids
// with more than one component the preconditioner is applied as
// z = P V(P r), P removing the mean of every component -- the projection
// onto the consistent part, symmetric, so the preconditioned CG stays valid
// and its recursive residual measures the consistent part.  A grid whose
// fluid is connected keeps z = V(r) (its inconsistency is negligible).
//
// Components are labelled once per mask on the host (cells with any open
// face, connected through open faces).  Their cells are stored as one list
// sorted by component and cut into chunks that never straddle two
// components; the mean is formed from per-chunk partial sums folded per
// component in a fixed order (deterministic), then subtracted chunk-wise.
#include <algorithm>
#include <vector>

#include "pg_internal.cuh"

namespace pg {

constexpr int kPocketThreads = 256;
constexpr int kPocketChunk = 2048;  // cells per chunk

void find_pockets(const uint8_t* flags, int nd, i64 d, i64 h, i64 w, i64 base, std::vector<i64>& cells,
                  std::vector<int>& start) {
    const i64 n = d * h * w, hw = h * w;
    std::vector<int> label((size_t)n, -1);
    std::vector<i64> size;
    std::vector<i64> stack;
    for (i64 s = 0; s < n; ++s) {
        if (label[s] >= 0 || (flags[s] & 63) == 0) continue;
        const int k = (int)size.size();
        i64 cnt = 0;
        label[s] = k;
        stack.push_back(s);
        while (!stack.empty()) {
            const i64 c = stack.back();
            stack.pop_back();
            ++cnt;
            const uint8_t f = flags[c];
            const i64 nb[6] = {c - 1, c + 1, c - w, c + w, c - hw, c + hw};
            const uint8_t bits[6] = {XLO, XHI, YLO, YHI, ZLO, ZHI};
            for (int j = 0; j < (nd == 3 ? 6 : 4); ++j)
                if ((f & bits[j]) && label[nb[j]] < 0) {
                    label[nb[j]] = k;
                    stack.push_back(nb[j]);
                }
        }
        size.push_back(cnt);
    }
    const int nl = (int)size.size();
    if (nl <= 1) return;  // connected fluid: no projection
    // counting sort of the cells by component, cells in index order
    std::vector<i64> pos(nl, 0);
    if (start.empty()) start.push_back((int)cells.size());
    i64 at = (i64)cells.size();
    for (int k = 0; k < nl; ++k) {
        pos[k] = at;
        at += size[k];
        start.push_back((int)at);
    }
    cells.resize((size_t)at);
    for (i64 c = 0; c < n; ++c) {
        const int k = label[c];
        if (k >= 0) cells[pos[k]++] = base + c;
    }
}

void release_pockets(Pockets* pk) {
    void* ptrs[] = {pk->cells, pk->start, pk->chunk_start, pk->chunk_comp, pk->comp_chunk, pk->partials};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    *pk = Pockets{};
}

int upload_pockets(const std::vector<i64>& cells, const std::vector<int>& start, Pockets* pk) {
    release_pockets(pk);
    if (start.size() < 2) return PG_OK;
    if (cells.back() >= ((i64)1 << 31)) return bad_arg("component projection: too many cells for 32-bit indices");
    const int ncomp = (int)start.size() - 1;
    std::vector<int> c32(cells.begin(), cells.end());
    std::vector<int> chunk_start, chunk_comp, comp_chunk;
    for (int k = 0; k < ncomp; ++k) {
        comp_chunk.push_back((int)chunk_comp.size());
        for (int a = start[k]; a < start[k + 1]; a += kPocketChunk) {
            chunk_start.push_back(a);
            chunk_comp.push_back(k);
        }
    }
    comp_chunk.push_back((int)chunk_comp.size());
    chunk_start.push_back(start[ncomp]);
    pk->ncomp = ncomp;
    pk->nchunk = (int)chunk_comp.size();
    PG_CUDA(cudaMalloc(&pk->cells, sizeof(int) * c32.size()));
    PG_CUDA(cudaMalloc(&pk->start, sizeof(int) * start.size()));
    PG_CUDA(cudaMalloc(&pk->chunk_start, sizeof(int) * chunk_start.size()));
    PG_CUDA(cudaMalloc(&pk->chunk_comp, sizeof(int) * chunk_comp.size()));
    PG_CUDA(cudaMalloc(&pk->comp_chunk, sizeof(int) * comp_chunk.size()));
    PG_CUDA(cudaMalloc(&pk->partials, sizeof(double) * (chunk_comp.size() + ncomp)));
    PG_CUDA(cudaMemcpy(pk->cells, c32.data(), sizeof(int) * c32.size(), cudaMemcpyHostToDevice));
    PG_CUDA(cudaMemcpy(pk->start, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
    PG_CUDA(cudaMemcpy(pk->chunk_start, chunk_start.data(), sizeof(int) * chunk_start.size(), cudaMemcpyHostToDevice));
    PG_CUDA(cudaMemcpy(pk->chunk_comp, chunk_comp.data(), sizeof(int) * chunk_comp.size(), cudaMemcpyHostToDevice));
    PG_CUDA(cudaMemcpy(pk->comp_chunk, comp_chunk.data(), sizeof(int) * comp_chunk.size(), cudaMemcpyHostToDevice));
    return PG_OK;
}

// partials[chunk] = sum of a over the chunk's cells
__global__ void __launch_bounds__(kPocketThreads)
    k_pocket_sum(const float* __restrict__ a, const int* __restrict__ cells, const int* __restrict__ chunk_start,
                 int nchunk, double* __restrict__ partials) {
    __shared__ double sm[32];
    for (int k = blockIdx.x; k < nchunk; k += gridDim.x) {
        double s = 0.0;
        for (int i = chunk_start[k] + threadIdx.x; i < chunk_start[k + 1]; i += blockDim.x) s += (double)a[cells[i]];
        s = block_sum<kPocketThreads>(s, sm);
        if (threadIdx.x == 0) partials[k] = s;
        __syncthreads();
    }
}

// mean[comp] = sum of its chunks' partials (in order) / its cell count
__global__ void k_pocket_mean(const int* __restrict__ start, const int* __restrict__ comp_chunk, int ncomp,
                              const double* __restrict__ partials, double* __restrict__ mean) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncomp; k += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = comp_chunk[k]; c < comp_chunk[k + 1]; ++c) s += partials[c];
        mean[k] = s / (double)(start[k + 1] - start[k]);
    }
}

// a -= mean of its component, chunk by chunk
__global__ void __launch_bounds__(kPocketThreads)
    k_pocket_sub(float* __restrict__ a, const int* __restrict__ cells, const int* __restrict__ chunk_start,
                 const int* __restrict__ chunk_comp, int nchunk, const double* __restrict__ mean) {
    for (int k = blockIdx.x; k < nchunk; k += gridDim.x) {
        const float m = (float)mean[chunk_comp[k]];
        for (int i = chunk_start[k] + threadIdx.x; i < chunk_start[k + 1]; i += blockDim.x) a[cells[i]] -= m;
    }
}

void pocket_project(cudaStream_t s, float* a, const Pockets& pk) {
    if (!pk.ncomp) return;
    const int nb = std::min(pk.nchunk, 4096);
    double* mean = pk.partials + pk.nchunk;
    PG_LAUNCH(KK_STEP_MISC, s, k_pocket_sum<<<nb, kPocketThreads, 0, s>>>(a, pk.cells, pk.chunk_start, pk.nchunk, pk.partials));
    PG_LAUNCH(KK_STEP_MISC, s, k_pocket_mean<<<(pk.ncomp + 127) / 128, 128, 0, s>>>(pk.start, pk.comp_chunk, pk.ncomp, pk.partials, mean));
    PG_LAUNCH(KK_STEP_MISC, s, k_pocket_sub<<<nb, kPocketThreads, 0, s>>>(a, pk.cells, pk.chunk_start, pk.chunk_comp, pk.nchunk, mean));
}

}  // namespace pg
