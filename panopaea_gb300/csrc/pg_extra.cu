// pg_extra.cu -- the reference's sparse-matrix products and its image
// transfer, on the device.
//
// * SparseMatrix::mul_vec (panopaea/src/sparse.rs:119-128): CSR with usize
//   (here int64) row and column indices; b[i] is the left fold
//   acc + data[k] * x[col[k]] over row i in storage order, from zero -- one
//   thread per row, the same order, unfused, so f32/f64 results are
//   bit-identical to the Rust fold.
// * DiagonalMatrix::mul_vec (sparse.rs:20-25): b = x * a.
// * imgproc::transfer (panopaea_utils/src/imgproc.rs:2-5) applied to a cell
//   field and laid out as png::export writes it (png.rs:6-18: image row y
//   shows field row h-1-y, three equal channels), so a density snapshot of
//   examples/dec_fluid.rs:143-164 is produced on the device and only the
//   8-bit image crosses to the host.  The transfer runs in f64 as in the
//   reference (`&f64` input).
#include "pg_internal.cuh"

namespace pg {

template <class T>
__global__ void k_csr_mul_vec(i64 rows, const i64* __restrict__ rowp, const i64* __restrict__ cols,
                              const T* __restrict__ data, const T* __restrict__ x, T* __restrict__ b) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (i64)gridDim.x * blockDim.x) {
        T acc = T(0);
        const i64 e = rowp[i + 1];
        for (i64 k = rowp[i]; k < e; ++k) acc = add_rn(acc, mul_rn(data[k], x[cols[k]]));
        b[i] = acc;
    }
}

template <class T>
__global__ void k_diag_mul_vec(i64 n, const T* __restrict__ a, const T* __restrict__ x, T* __restrict__ b) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        b[i] = mul_rn(x[i], a[i]);
}

// imgproc.rs:2-5: v = x.min(upper).max(lower); ((v - lower) / (upper -
// lower) * 255.0) as u8 (a saturating cast that truncates toward zero).
template <class T>
__global__ void k_transfer_rgb8(i64 h, i64 w, const T* __restrict__ f, double lo, double hi, uint8_t* __restrict__ rgb) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < h * w; i += (i64)gridDim.x * blockDim.x) {
        const i64 yi = i / w, x = i - yi * w;
        const double val = (double)f[(h - 1 - yi) * w + x];
        const double v = fmax(fmin(val, hi), lo);
        const double s = __dmul_rn(__ddiv_rn(__dsub_rn(v, lo), __dsub_rn(hi, lo)), 255.0);
        const uint8_t u = (s != s) ? 0 : (s <= 0.0 ? 0 : (s >= 255.0 ? 255 : (uint8_t)s));
        rgb[3 * i + 0] = u;
        rgb[3 * i + 1] = u;
        rgb[3 * i + 2] = u;
    }
}

static int blocks_for(i64 n) {
    i64 b = (n + 255) / 256;
    if (b > 4096) b = 4096;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace pg

using namespace pg;

#define PG_EXTRA_ABI(T, SFX)                                                                                    \
    extern "C" int pg_csr_mul_vec_##SFX(int64_t rows, const int64_t* row_indices, const int64_t* col_indices,  \
                                        const T* data, const T* x, T* b, void* stream) {                        \
        if (rows < 0 || (rows && (!row_indices || !b))) return bad_arg("pg_csr_mul_vec: bad arguments");       \
        if (rows == 0) return PG_OK;                                                                            \
        cudaStream_t s = (cudaStream_t)stream;                                                                  \
        PG_LAUNCH(KK_DEC_OP, s,                                                                                 \
                  k_csr_mul_vec<T><<<blocks_for(rows), 256, 0, s>>>(rows, row_indices, col_indices, data, x, b)); \
        PG_CHECK_LAUNCH();                                                                                      \
        return PG_OK;                                                                                           \
    }                                                                                                           \
    extern "C" int pg_diag_mul_vec_##SFX(int64_t n, const T* a, const T* x, T* b, void* stream) {              \
        if (n < 0 || (n && (!a || !x || !b))) return bad_arg("pg_diag_mul_vec: bad arguments");                \
        if (n == 0) return PG_OK;                                                                               \
        cudaStream_t s = (cudaStream_t)stream;                                                                  \
        PG_LAUNCH(KK_DEC_OP, s, k_diag_mul_vec<T><<<blocks_for(n), 256, 0, s>>>(n, a, x, b));                  \
        PG_CHECK_LAUNCH();                                                                                      \
        return PG_OK;                                                                                           \
    }                                                                                                           \
    extern "C" int pg_transfer_rgb8_##SFX(int64_t h, int64_t w, const T* field, double lower, double upper,     \
                                          uint8_t* rgb, void* stream) {                                         \
        if (h < 1 || w < 1 || !field || !rgb) return bad_arg("pg_transfer_rgb8: bad arguments");               \
        cudaStream_t s = (cudaStream_t)stream;                                                                  \
        PG_LAUNCH(KK_DEC_OP, s, k_transfer_rgb8<T><<<blocks_for(h * w), 256, 0, s>>>(h, w, field, lower, upper, rgb)); \
        PG_CHECK_LAUNCH();                                                                                      \
        return PG_OK;                                                                                           \
    }

PG_EXTRA_ABI(float, f32)
PG_EXTRA_ABI(double, f64)
