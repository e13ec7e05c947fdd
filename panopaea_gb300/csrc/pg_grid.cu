// pg_grid.cu -- grid handles, solid masks, field storage, errors.
#include <cstdio>
#include <cstring>
#include <vector>

#include "pg_internal.cuh"

namespace pg {

static thread_local std::string t_last_error;

void set_error(const std::string& msg) { t_last_error = msg; }

int cuda_fail(cudaError_t e, const char* what) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    set_error(buf);
    if (e == cudaErrorMemoryAllocation) return PG_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PG_NO_DEVICE;
    return PG_CUDA_ERROR;
}

__global__ void k_words_out(const unsigned* __restrict__ src, unsigned* dst, int nwords) {
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) dst[i] = src[i];
}

int ensure_workspace(pg_grid* g) {
    Workspace& ws = g->ws;
    if (ws.state) return PG_OK;
    PG_CUDA(cudaMalloc(&ws.partials, sizeof(double) * 4 * kMaxBlocks));
    PG_CUDA(cudaMalloc(&ws.state, sizeof(CgState)));
    PG_CUDA(cudaMemset(ws.state, 0, sizeof(CgState)));
    // slots 0, 1: the host-polled loop; slot 2: the final state; then one
    // double (a reduction result read back by the host)
    PG_CUDA(cudaMallocHost(&ws.state_host, 3 * sizeof(CgState) + sizeof(double)));
    PG_CUDA(cudaEventCreateWithFlags(&ws.ev[0], cudaEventDisableTiming));
    PG_CUDA(cudaEventCreateWithFlags(&ws.ev[1], cudaEventDisableTiming));
    return PG_OK;
}

int ensure_vec(pg_grid* g, size_t bytes) {
    Workspace& ws = g->ws;
    if (ws.vec_bytes >= bytes) return PG_OK;
    if (ws.vec) {
        PG_CUDA(cudaStreamSynchronize(g->stream));
        PG_CUDA(cudaFree(ws.vec));
        ws.vec = nullptr;
        ws.vec_bytes = 0;
    }
    PG_CUDA(cudaMalloc(&ws.vec, bytes));
    ws.vec_bytes = bytes;
    return PG_OK;
}

// Laplacian face-open bits from an optional per-face solid array (host).
static void build_flags(const Dims& D, const uint8_t* fs, std::vector<uint8_t>& flags) {
    flags.assign((size_t)D.nc(), 0);
    for (i64 z = 0; z < D.d; ++z)
        for (i64 y = 0; y < D.h; ++y)
            for (i64 x = 0; x < D.w; ++x) {
                uint8_t f = 0;
                auto open = [&](i64 face) { return !(fs && fs[face]); };
                if (x > 0 && open(D.fx(z, y, x))) f |= XLO;
                if (x < D.w - 1 && open(D.fx(z, y, x + 1))) f |= XHI;
                if (y > 0 && open(D.fy(z, y, x))) f |= YLO;
                if (y < D.h - 1 && open(D.fy(z, y + 1, x))) f |= YHI;
                if (D.nd == 3) {
                    if (z > 0 && open(D.fz(z, y, x))) f |= ZLO;
                    if (z < D.d - 1 && open(D.fz(z + 1, y, x))) f |= ZHI;
                }
                flags[(size_t)D.cell(z, y, x)] = f;
            }
}

static int upload_mask(pg_grid* g, const uint8_t* host_face_solid) {
    const Dims& D = g->dims;
    std::vector<uint8_t> flags;
    build_flags(D, host_face_solid, flags);
    ++g->mask_version;
    PG_CUDA(cudaMemcpy(g->flags, flags.data(), flags.size(), cudaMemcpyHostToDevice));
    if (host_face_solid) {
        if (!g->face_solid) PG_CUDA(cudaMalloc(&g->face_solid, (size_t)D.nf()));
        PG_CUDA(cudaMemcpy(g->face_solid, host_face_solid, (size_t)D.nf(), cudaMemcpyHostToDevice));
    } else if (g->face_solid) {
        PG_CUDA(cudaFree(g->face_solid));
        g->face_solid = nullptr;
    }
    return PG_OK;
}

static int create(int nd, i64 d, i64 h, i64 w, pg_grid** out) {
    if (!out) return bad_arg("pg_grid_create: out is NULL");
    *out = nullptr;
    if (d < 1 || h < 1 || w < 1) return bad_arg("pg_grid_create: every dimension must be >= 1");
    const i64 lim = (i64)1 << 40;
    if (d > lim / h / w) return bad_arg("pg_grid_create: grid too large");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        set_error("pg_grid_create: no CUDA device");
        return PG_NO_DEVICE;
    }
    pg_grid* g = new pg_grid();
    g->dims = Dims{nd, d, h, w};
    PG_CUDA(cudaGetDevice(&g->device));
    PG_CUDA(cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device));
    cudaError_t ea = cudaMalloc(&g->flags, (size_t)g->dims.nc());
    if (ea != cudaSuccess) {
        delete g;
        return cuda_fail(ea, "cudaMalloc(flags)");
    }
    int rc = upload_mask(g, nullptr);
    if (rc == PG_OK) rc = ensure_workspace(g);
    if (rc != PG_OK) {
        pg_grid_destroy(g);
        return rc;
    }
    *out = g;
    return PG_OK;
}

}  // namespace pg

using namespace pg;

extern "C" {

const char* pg_status_string(int s) {
    switch (s) {
        case PG_OK: return "PG_OK";
        case PG_NOT_CONVERGED: return "PG_NOT_CONVERGED";
        case PG_NAN_DETECTED: return "PG_NAN_DETECTED";
        case PG_TIMEOUT: return "PG_TIMEOUT";
        case PG_BAD_ARG: return "PG_BAD_ARG";
        case PG_CUDA_ERROR: return "PG_CUDA_ERROR";
        case PG_NO_DEVICE: return "PG_NO_DEVICE";
        case PG_OUT_OF_MEMORY: return "PG_OUT_OF_MEMORY";
        case PG_BREAKDOWN: return "PG_BREAKDOWN";
        default: return "PG_UNKNOWN";
    }
}

const char* pg_last_error(void) { return t_last_error.c_str(); }

int pg_version(void) { return 1; }

int pg_grid_create_2d(int64_t h, int64_t w, pg_grid** out) { return create(2, 1, h, w, out); }

int pg_grid_create_3d(int64_t d, int64_t h, int64_t w, pg_grid** out) { return create(3, d, h, w, out); }

int pg_grid_destroy(pg_grid* g) {
    if (!g) return PG_OK;
    if (g->stream) cudaStreamSynchronize(g->stream);
    else cudaDeviceSynchronize();
    cudaFree(g->flags);
    cudaFree(g->face_solid);
    cudaFree(g->ws.partials);
    cudaFree(g->ws.state);
    cudaFreeHost(g->ws.state_host);
    cudaFree(g->ws.vec);
    if (g->ws.ev[0]) cudaEventDestroy(g->ws.ev[0]);
    if (g->ws.ev[1]) cudaEventDestroy(g->ws.ev[1]);
    release_extras(g);
    release_cg_graphs(g);
    delete g;
    return PG_OK;
}

int pg_grid_dim(const pg_grid* g, int64_t dim_out[3]) {
    if (!g || !dim_out) return -PG_BAD_ARG;
    dim_out[0] = g->dims.d;
    dim_out[1] = g->dims.h;
    dim_out[2] = g->dims.w;
    return g->dims.nd;
}

int64_t pg_grid_num_elem_1(const pg_grid* g) { return g ? g->dims.nf() : -1; }
int64_t pg_grid_num_elem_2(const pg_grid* g) { return g ? g->dims.nc() : -1; }

int pg_grid_set_stream(pg_grid* g, void* s) {
    if (!g) return bad_arg("pg_grid_set_stream: grid is NULL");
    g->stream = (cudaStream_t)s;
    return PG_OK;
}

int pg_grid_synchronize(pg_grid* g) {
    if (!g) return bad_arg("pg_grid_synchronize: grid is NULL");
    PG_CUDA(cudaStreamSynchronize(g->stream));
    return PG_OK;
}

int pg_grid_set_solid_faces(pg_grid* g, const uint8_t* fs) {
    if (!g) return bad_arg("pg_grid_set_solid_faces: grid is NULL");
    PG_CUDA(cudaStreamSynchronize(g->stream));
    return upload_mask(g, fs);
}

int pg_grid_set_solid_cells(pg_grid* g, const uint8_t* cs) {
    if (!g) return bad_arg("pg_grid_set_solid_cells: grid is NULL");
    if (!cs) return pg_grid_set_solid_faces(g, nullptr);
    const Dims& D = g->dims;
    std::vector<uint8_t> fs((size_t)D.nf(), 0);
    auto solid = [&](i64 z, i64 y, i64 x) { return cs[(size_t)D.cell(z, y, x)] != 0; };
    for (i64 z = 0; z < D.d; ++z)
        for (i64 y = 0; y < D.h; ++y)
            for (i64 x = 0; x <= D.w; ++x)
                fs[(size_t)D.fx(z, y, x)] = (x > 0 && solid(z, y, x - 1)) || (x < D.w && solid(z, y, x));
    for (i64 z = 0; z < D.d; ++z)
        for (i64 y = 0; y <= D.h; ++y)
            for (i64 x = 0; x < D.w; ++x)
                fs[(size_t)D.fy(z, y, x)] = (y > 0 && solid(z, y - 1, x)) || (y < D.h && solid(z, y, x));
    if (D.nd == 3)
        for (i64 z = 0; z <= D.d; ++z)
            for (i64 y = 0; y < D.h; ++y)
                for (i64 x = 0; x < D.w; ++x)
                    fs[(size_t)D.fz(z, y, x)] = (z > 0 && solid(z - 1, y, x)) || (z < D.d && solid(z, y, x));
    return pg_grid_set_solid_faces(g, fs.data());
}

int pg_field_alloc(const pg_grid* g, int kind, int dtype, void** out) {
    if (!g || !out) return bad_arg("pg_field_alloc: NULL argument");
    *out = nullptr;
    i64 n;
    if (kind == PG_FACES) n = g->dims.nf();
    else if (kind == PG_CELLS) n = g->dims.nc();
    else return bad_arg("pg_field_alloc: kind must be PG_FACES or PG_CELLS");
    size_t es;
    if (dtype == PG_F32) es = 4;
    else if (dtype == PG_F64) es = 8;
    else return bad_arg("pg_field_alloc: dtype must be PG_F32 or PG_F64");
    void* p = nullptr;
    PG_CUDA(cudaMalloc(&p, es * (size_t)n));
    cudaError_t e = cudaMemsetAsync(p, 0, es * (size_t)n, g->stream);
    if (e != cudaSuccess) {
        cudaFree(p);
        return cuda_fail(e, "cudaMemsetAsync");
    }
    *out = p;
    return PG_OK;
}

int pg_field_free(void* p) {
    if (p) PG_CUDA(cudaFree(p));
    return PG_OK;
}

int pg_copy_h2d(const pg_grid* g, void* dst, const void* src, size_t bytes) {
    if (!g || (!dst && bytes) || (!src && bytes)) return bad_arg("pg_copy_h2d: NULL argument");
    PG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g->stream));
    return PG_OK;
}

int pg_copy_d2h(const pg_grid* g, void* dst, const void* src, size_t bytes) {
    if (!g || (!dst && bytes) || (!src && bytes)) return bad_arg("pg_copy_d2h: NULL argument");
    PG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, g->stream));
    return PG_OK;
}

}  // extern "C"
