// pg_wavelet.cu -- wavelet and divergence-free wavelet transforms
// (panopaea/src/math/wavelet/mod.rs:1-681; the filters of haar.rs and
// spline.rs).  The reference marks the module as early, mostly abandoned
// tests; its behaviour is restated as written, boundary rules included.
//
// FP64 arrays on the device.  A 1D transform step over every line of a
// block is one launch, one thread per output sample:
//   down (mod.rs:52-79): out[i] = fold over f of src[mirror(2i + f - n/2 + 1)]
//     * filter[n-1-f], low pass for i < half, high pass for i >= half;
//   up (mod.rs:81-112): the reference scatters out[(2i + f - n/2 + 1) wrapped]
//     += src[i] * low[f] + src[i + half] * high[f]; here each output gathers
//     its contributions and adds them in the reference's (i, f) order, so
//     the sums round the same way.
// The level loops, the copies to the temporary and the axis orders are
// those of fwt_1d / ifwt_1d / fwt_2d_isotropic / ifwt_2d_isotropic /
// fwt_2d_separate_isotropic / ifwt_2d_separate_isotropic /
// fwt_2d_anisotropic (mod.rs:114-294); div_coeff_2d / inv_div_coeff_2d
// (mod.rs:296-451) are one launch per level.  The border variants
// (mod.rs:454-681) run the passes of pg_wavelet_border.cuh: one launch per
// 1D pass over every line of a band, into a packed output.
#include <algorithm>

#include "pg_internal.cuh"
#include "pg_wavelet_border.cuh"

namespace pg {

namespace {

constexpr int kWThreads = 256;
using wv::filter_of;
using wv::kMaxTaps;
using wv::WFilter;

// mod.rs:38-48 MirrorSampler::fetch
__device__ __forceinline__ double mirror(const double* line, i64 stride, i64 len, i64 idx) {
    if (idx < 0) return line[(-idx) * stride];
    if (idx >= len) return line[(len - 1 - (idx % len)) * stride];
    return line[idx * stride];
}

// down_convolution over `lines` lines of length `len` (element k of line l
// at l * lstride + k * estride), src -> dst (same addressing).
__global__ void __launch_bounds__(kWThreads) k_wdown(const double* __restrict__ src, double* __restrict__ dst, i64 lines,
                                                     i64 len, i64 lstride, i64 estride, WFilter F) {
    const i64 half = len / 2, total = lines * 2 * half;
    const int n = F.n, fh = n / 2;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (i64)gridDim.x * blockDim.x) {
        const i64 l = t / (2 * half), o = t - l * 2 * half;
        const bool high = o >= half;
        const i64 i = high ? o - half : o;
        const double* line = src + l * lstride;
        const double* filt = high ? F.down_high : F.down_low;
        double acc = 0.0;
        for (int f = 0; f < n; ++f)
            acc = __dadd_rn(__dmul_rn(mirror(line, estride, len, 2 * i + f - fh + 1), filt[n - 1 - f]), acc);
        dst[l * lstride + o * estride] = acc;
    }
}

// up_convolution, gathered: output j receives, in increasing (i, f) order,
// src[i] * up_low[f] + src[i + half] * up_high[f] for every (i, f) whose
// wrapped index 2i + f - n/2 + 1 is j.
__global__ void __launch_bounds__(kWThreads) k_wup(const double* __restrict__ src, double* __restrict__ dst, i64 lines,
                                                   i64 len, i64 lstride, i64 estride, WFilter F) {
    const i64 half = len / 2, total = lines * len;
    const int n = F.n, fh = n / 2;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (i64)gridDim.x * blockDim.x) {
        const i64 l = t / len, j = t - l * len;
        const double* line = src + l * lstride;
        // contributions (i, f): at most three wrapped images of j per tap
        i64 ci[3 * kMaxTaps];
        int cf[3 * kMaxTaps];
        int m = 0;
        for (int f = 0; f < n; ++f)
            for (int w = -1; w <= 1; ++w) {
                const i64 idx = j + w * len;  // unwrapped 2i + f - fh + 1
                const i64 two_i = idx - f + fh - 1;
                if (two_i < 0 || (two_i & 1) || two_i / 2 >= half) continue;
                // the reference's wrap of idx must land on j
                const i64 wrapped = idx < 0 ? (idx + len) % len : idx % len;
                if (wrapped != j) continue;
                ci[m] = two_i / 2;
                cf[m] = f;
                ++m;
            }
        // insertion sort by (i, f)
        for (int a = 1; a < m; ++a) {
            const i64 ki = ci[a];
            const int kf = cf[a];
            int b = a - 1;
            while (b >= 0 && (ci[b] > ki || (ci[b] == ki && cf[b] > kf))) {
                ci[b + 1] = ci[b];
                cf[b + 1] = cf[b];
                --b;
            }
            ci[b + 1] = ki;
            cf[b + 1] = kf;
        }
        double out = 0.0;
        for (int a = 0; a < m; ++a) {
            const i64 i = ci[a];
            const int f = cf[a];
            const double v = __dadd_rn(__dmul_rn(mirror(line, estride, len, i), F.up_low[f]),
                                       __dmul_rn(mirror(line, estride, len, i + half), F.up_high[f]));
            out = __dadd_rn(out, v);
        }
        dst[l * lstride + j * estride] = out;
    }
}

// temp[block] = out[block]: the (rows x cols) top-left block of a row-major
// array with row stride w.
__global__ void k_wcopy(const double* __restrict__ src, double* __restrict__ dst, i64 rows, i64 cols, i64 w) {
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < rows * cols; t += (i64)gridDim.x * blockDim.x) {
        const i64 r = t / cols, c = t - r * cols;
        dst[r * w + c] = src[r * w + c];
    }
}

// mod.rs:296-376, one level: quadrants of the (2 hh) x (2 hw) block.
__global__ void k_div_coeff(const double* __restrict__ vx, const double* __restrict__ vy, double* __restrict__ dv,
                            double* __restrict__ nn, i64 hh, i64 hw, i64 w, int last) {
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < hh * hw; t += (i64)gridDim.x * blockDim.x) {
        const i64 y = t / hw, x = t - y * hw;
        const i64 ym = y > 0 ? y - 1 : 0, xm = x > 0 ? x - 1 : 0;
        const i64 q00 = y * w + x, q01 = y * w + hw + x, q10 = (y + hh) * w + x, q11 = (y + hh) * w + hw + x;
        dv[q01] = vy[q01];
        dv[q10] = vx[q10];
        dv[q11] = __ddiv_rn(__dsub_rn(vx[q11], vy[q11]), 2.0);
        nn[q01] = __dadd_rn(vx[q01], __ddiv_rn(__dsub_rn(vy[q01], vy[ym * w + hw + x]), 4.0));
        nn[q10] = __dadd_rn(vy[q10], __ddiv_rn(__dsub_rn(vx[q10], vx[(y + hh) * w + xm]), 4.0));
        nn[q11] = __ddiv_rn(__dadd_rn(vx[q11], vy[q11]), 2.0);
        if (last) {
            dv[q00] = vx[q00];
            nn[q00] = vy[q00];
        }
    }
}

// mod.rs:378-451, one level.
__global__ void k_inv_div_coeff(const double* __restrict__ dv, const double* __restrict__ nn, double* __restrict__ vx,
                                double* __restrict__ vy, i64 hh, i64 hw, i64 w, int first) {
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < hh * hw; t += (i64)gridDim.x * blockDim.x) {
        const i64 y = t / hw, x = t - y * hw;
        const i64 ym = y > 0 ? y - 1 : 0, xm = x > 0 ? x - 1 : 0;
        const i64 q00 = y * w + x, q01 = y * w + hw + x, q10 = (y + hh) * w + x, q11 = (y + hh) * w + hw + x;
        vx[q01] = __dsub_rn(nn[q01], __ddiv_rn(__dsub_rn(dv[ym * w + hw + x], dv[q01]), 4.0));
        vx[q10] = dv[q10];
        vx[q11] = __dadd_rn(dv[q11], nn[q11]);
        vy[q01] = dv[q01];
        vy[q10] = __dsub_rn(nn[q10], __ddiv_rn(__dsub_rn(dv[(y + hh) * w + xm], dv[q10]), 4.0));
        vy[q11] = __dsub_rn(nn[q11], dv[q11]);
        if (first) {
            vx[q00] = dv[q00];
            vy[q00] = nn[q00];
        }
    }
}

// Border variants: one thread per output sample of a pass.
__global__ void __launch_bounds__(kWThreads) k_wdown_border(const double* __restrict__ src, wv::WLines in, double* lo,
                                                            double* hi, wv::WLines out, WFilter F) {
    const i64 total = in.lines * 2 * out.len;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (i64)gridDim.x * blockDim.x)
        wv::wdown_border_at(src, in, lo, hi, out, F, t);
}

__global__ void __launch_bounds__(kWThreads) k_wup_border(const double* __restrict__ cs, wv::WLines c,
                                                          const double* __restrict__ ds, wv::WLines d,
                                                          double* __restrict__ dst, wv::WLines out, WFilter F) {
    const i64 total = out.lines * out.len;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (i64)gridDim.x * blockDim.x)
        wv::wup_border_at(cs, c, ds, d, dst, out, F, t);
}

__global__ void __launch_bounds__(kWThreads) k_wdiv_border(const double* __restrict__ vx, const double* __restrict__ vy,
                                                           double* __restrict__ dv, double* __restrict__ nn, i64 R,
                                                           i64 C) {
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < R * C; t += (i64)gridDim.x * blockDim.x)
        wv::wdiv_border_at(vx, vy, dv, nn, R, C, t);
}

__global__ void k_wcopy_flat(const double* __restrict__ src, double* __restrict__ dst, i64 n) {
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (i64)gridDim.x * blockDim.x) dst[t] = src[t];
}

int wblocks(i64 n) { return (int)std::max<i64>(1, std::min<i64>((n + kWThreads - 1) / kWThreads, 4096)); }

int down(cudaStream_t s, const double* src, double* dst, i64 lines, i64 len, i64 ls, i64 es, const WFilter& F) {
    PG_LAUNCH(KK_DEC_OP, s, k_wdown<<<wblocks(lines * len), kWThreads, 0, s>>>(src, dst, lines, len, ls, es, F));
    PG_CHECK_LAUNCH();
    return PG_OK;
}
int up(cudaStream_t s, const double* src, double* dst, i64 lines, i64 len, i64 ls, i64 es, const WFilter& F) {
    PG_LAUNCH(KK_DEC_OP, s, k_wup<<<wblocks(lines * len), kWThreads, 0, s>>>(src, dst, lines, len, ls, es, F));
    PG_CHECK_LAUNCH();
    return PG_OK;
}
int copy(cudaStream_t s, const double* src, double* dst, i64 rows, i64 cols, i64 w) {
    PG_LAUNCH(KK_DEC_OP, s, k_wcopy<<<wblocks(rows * cols), kWThreads, 0, s>>>(src, dst, rows, cols, w));
    PG_CHECK_LAUNCH();
    return PG_OK;
}

// The sizes the reference handles without indexing out of range: every
// transformed length a multiple of 2^levels, and the shortest one (the
// last level's) at least the filter length.
int check_levels(i64 n, int levels, const WFilter& F) {
    if (levels < 0 || levels > 40) return bad_arg("wavelet: levels must be in 0..40");
    if (levels > 0 && (n >> levels) << levels != n) return bad_arg("wavelet: size must be divisible by 2^levels");
    if (levels > 0 && (n >> (levels - 1)) < F.n) return bad_arg("wavelet: the last level is shorter than the filter");
    return PG_OK;
}

// The device executor of the border passes.
struct DeviceExec {
    cudaStream_t s;
    int down(const double* src, wv::WLines in, double* lo, double* hi, wv::WLines out, const WFilter& F) {
        PG_LAUNCH(KK_DEC_OP, s,
                  k_wdown_border<<<wblocks(in.lines * 2 * out.len), kWThreads, 0, s>>>(src, in, lo, hi, out, F));
        PG_CHECK_LAUNCH();
        return PG_OK;
    }
    int up(const double* c, wv::WLines cl, const double* d, wv::WLines dl, double* dst, wv::WLines out,
           const WFilter& F) {
        if (out.lines * out.len == 0) return PG_OK;
        PG_LAUNCH(KK_DEC_OP, s, k_wup_border<<<wblocks(out.lines * out.len), kWThreads, 0, s>>>(c, cl, d, dl, dst, out, F));
        PG_CHECK_LAUNCH();
        return PG_OK;
    }
    int div(const double* vx, const double* vy, double* dv, double* nn, i64 R, i64 C) {
        PG_LAUNCH(KK_DEC_OP, s, k_wdiv_border<<<wblocks(R * C), kWThreads, 0, s>>>(vx, vy, dv, nn, R, C));
        PG_CHECK_LAUNCH();
        return PG_OK;
    }
    int copy(const double* src, double* dst, i64 n) {
        PG_LAUNCH(KK_DEC_OP, s, k_wcopy_flat<<<wblocks(n), kWThreads, 0, s>>>(src, dst, n));
        PG_CHECK_LAUNCH();
        return PG_OK;
    }
};

// Distinct, non-overlapping device ranges [p, p + n) (n in doubles).
bool disjoint(const double* a, i64 na, const double* b, i64 nb) { return a + na <= b || b + nb <= a; }

}  // namespace
}  // namespace pg

using namespace pg;

extern "C" {

int pg_wavelet_fwt_1d(int wavelet, double* data, int64_t n, int levels, double* temp, void* stream) {
    WFilter F;
    if (!data || !temp || n < 2) return bad_arg("pg_wavelet_fwt_1d: bad arguments");
    if (!filter_of(wavelet, &F)) return bad_arg("pg_wavelet_fwt_1d: unknown wavelet");
    int rc;
    if ((rc = check_levels(n, levels, F))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    i64 size = n;
    for (int k = 0; k < levels; ++k) {  // mod.rs:114-129
        if ((rc = copy(s, data, temp, 1, size, size)) || (rc = down(s, temp, data, 1, size, 0, 1, F))) return rc;
        size /= 2;
    }
    return PG_OK;
}

int pg_wavelet_ifwt_1d(int wavelet, double* data, int64_t n, int levels, double* temp, void* stream) {
    WFilter F;
    if (!data || !temp || n < 2) return bad_arg("pg_wavelet_ifwt_1d: bad arguments");
    if (!filter_of(wavelet, &F)) return bad_arg("pg_wavelet_ifwt_1d: unknown wavelet");
    int rc;
    if ((rc = check_levels(n, levels, F))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    i64 size = n >> levels;
    for (int k = 0; k < levels; ++k) {  // mod.rs:131-143
        size *= 2;
        if ((rc = copy(s, data, temp, 1, size, size)) || (rc = up(s, temp, data, 1, size, 0, 1, F))) return rc;
    }
    return PG_OK;
}

int pg_wavelet_fwt_2d(int mode, int wavelet_x, int wavelet_y, double* data, int64_t h, int64_t w, int levels,
                      double* temp, void* stream) {
    WFilter Fx, Fy;
    if (!data || !temp || h < 2 || w < 2) return bad_arg("pg_wavelet_fwt_2d: bad arguments");
    if (!filter_of(wavelet_x, &Fx) || !filter_of(wavelet_y, &Fy)) return bad_arg("pg_wavelet_fwt_2d: unknown wavelet");
    int rc;
    if ((rc = check_levels(h, levels, Fy)) || (rc = check_levels(w, levels, Fx))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (mode == PG_WAVELET_ISOTROPIC) {  // mod.rs:145-170, 206-231
        i64 r = h, c = w;
        for (int k = 0; k < levels; ++k) {
            if ((rc = copy(s, data, temp, r, c, w)) || (rc = down(s, temp, data, r, c, w, 1, Fx))) return rc;
            if ((rc = copy(s, data, temp, r, c, w)) || (rc = down(s, temp, data, c, r, 1, w, Fy))) return rc;
            r /= 2;
            c /= 2;
        }
        return PG_OK;
    }
    if (mode == PG_WAVELET_ANISOTROPIC) {  // mod.rs:262-294
        i64 r = h, c = w;
        for (int k = 0; k < levels; ++k) {  // x: every row, the coarse prefix halving
            if ((rc = copy(s, data, temp, r, c, w)) || (rc = down(s, temp, data, r, c, w, 1, Fx))) return rc;
            c /= 2;
        }
        r = h;
        c = w;
        for (int k = 0; k < levels; ++k) {  // y: every column, the coarse prefix halving
            if ((rc = copy(s, data, temp, r, c, w)) || (rc = down(s, temp, data, c, r, 1, w, Fy))) return rc;
            r /= 2;
        }
        return PG_OK;
    }
    return bad_arg("pg_wavelet_fwt_2d: unknown mode");
}

int pg_wavelet_ifwt_2d(int mode, int wavelet_x, int wavelet_y, double* data, int64_t h, int64_t w, int levels,
                       double* temp, void* stream) {
    WFilter Fx, Fy;
    if (!data || !temp || h < 2 || w < 2) return bad_arg("pg_wavelet_ifwt_2d: bad arguments");
    if (!filter_of(wavelet_x, &Fx) || !filter_of(wavelet_y, &Fy)) return bad_arg("pg_wavelet_ifwt_2d: unknown wavelet");
    int rc;
    if ((rc = check_levels(h, levels, Fy)) || (rc = check_levels(w, levels, Fx))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    i64 r = h >> levels, c = w >> levels;
    for (int k = 0; k < levels; ++k) {
        r *= 2;
        c *= 2;
        if (mode == PG_WAVELET_ISOTROPIC) {  // mod.rs:172-204: y, then x
            if ((rc = copy(s, data, temp, r, c, w)) || (rc = up(s, temp, data, c, r, 1, w, Fy))) return rc;
            if ((rc = copy(s, data, temp, r, c, w)) || (rc = up(s, temp, data, r, c, w, 1, Fx))) return rc;
        } else if (mode == PG_WAVELET_SEPARATE) {  // mod.rs:233-260: x, then y
            if ((rc = copy(s, data, temp, r, c, w)) || (rc = up(s, temp, data, r, c, w, 1, Fx))) return rc;
            if ((rc = copy(s, data, temp, r, c, w)) || (rc = up(s, temp, data, c, r, 1, w, Fy))) return rc;
        } else {
            return bad_arg("pg_wavelet_ifwt_2d: mode must be ISOTROPIC or SEPARATE");
        }
    }
    return PG_OK;
}

int pg_wavelet_div_coeff_2d(int levels, const double* vx, const double* vy, double* div, double* n, int64_t h,
                            int64_t w, void* stream) {
    if (!vx || !vy || !div || !n || h < 2 || w < 2 || levels < 1 || levels > 40 || (h >> levels) << levels != h ||
        (w >> levels) << levels != w)
        return bad_arg("pg_wavelet_div_coeff_2d: bad arguments (sizes must be multiples of 2^levels)");
    cudaStream_t s = (cudaStream_t)stream;
    i64 r = h, c = w;
    for (int k = 0; k < levels; ++k) {
        r /= 2;
        c /= 2;
        PG_LAUNCH(KK_DEC_OP, s, k_div_coeff<<<wblocks(r * c), kWThreads, 0, s>>>(vx, vy, div, n, r, c, w, k == levels - 1));
    }
    PG_CHECK_LAUNCH();
    return PG_OK;
}

int pg_wavelet_inv_div_coeff_2d(int levels, const double* div, const double* n, double* vx, double* vy, int64_t h,
                                int64_t w, void* stream) {
    if (!vx || !vy || !div || !n || h < 2 || w < 2 || levels < 1 || levels > 40 || (h >> levels) << levels != h ||
        (w >> levels) << levels != w)
        return bad_arg("pg_wavelet_inv_div_coeff_2d: bad arguments (sizes must be multiples of 2^levels)");
    cudaStream_t s = (cudaStream_t)stream;
    i64 r = h >> levels, c = w >> levels;
    for (int k = 0; k < levels; ++k) {
        PG_LAUNCH(KK_DEC_OP, s, k_inv_div_coeff<<<wblocks(r * c), kWThreads, 0, s>>>(div, n, vx, vy, r, c, w, k == 0));
        r *= 2;
        c *= 2;
    }
    PG_CHECK_LAUNCH();
    return PG_OK;
}

int pg_wavelet_border_sizes_1d(int wavelet, int64_t n, int levels, int64_t* packed, int64_t* temp,
                               int64_t* inverse_n) {
    WFilter F;
    wv::Plan1d P;
    if (!filter_of(wavelet, &F)) return bad_arg("pg_wavelet_border_sizes_1d: unknown wavelet");
    if (!wv::plan_1d(F, n, levels, &P)) return bad_arg("pg_wavelet_border_sizes_1d: n must be >= 2, levels in 0..40");
    if (packed) *packed = P.packed;
    if (temp) *temp = P.temp;
    if (inverse_n) *inverse_n = P.inverse_n;
    return PG_OK;
}

int pg_wavelet_border_sizes_2d(int wavelet_x, int wavelet_y, int64_t h, int64_t w, int levels, int64_t* packed,
                               int64_t* temp, int64_t* inverse_h, int64_t* inverse_w) {
    WFilter Fx, Fy;
    wv::Plan2d P;
    if (!filter_of(wavelet_x, &Fx) || !filter_of(wavelet_y, &Fy))
        return bad_arg("pg_wavelet_border_sizes_2d: unknown wavelet");
    if (!wv::plan_2d(Fx, Fy, h, w, levels, &P))
        return bad_arg("pg_wavelet_border_sizes_2d: h and w must be >= 2, levels in 0..40");
    if (packed) *packed = P.packed;
    if (temp) *temp = P.temp;
    if (inverse_h) *inverse_h = P.inverse_h;
    if (inverse_w) *inverse_w = P.inverse_w;
    return PG_OK;
}

int pg_wavelet_fwt_1d_border(int wavelet, const double* input, int64_t n, int levels, double* packed, double* temp,
                             void* stream) {
    WFilter F;
    wv::Plan1d P;
    if (!filter_of(wavelet, &F)) return bad_arg("pg_wavelet_fwt_1d_border: unknown wavelet");
    if (!wv::plan_1d(F, n, levels, &P)) return bad_arg("pg_wavelet_fwt_1d_border: n must be >= 2, levels in 0..40");
    if (!input || !packed || (P.temp && !temp) || !disjoint(input, n, packed, P.packed) ||
        (P.temp && (!disjoint(input, n, temp, P.temp) || !disjoint(packed, P.packed, temp, P.temp))))
        return bad_arg("pg_wavelet_fwt_1d_border: input, packed and temp must be distinct arrays");
    DeviceExec ex{(cudaStream_t)stream};
    return wv::run_fwt_1d(ex, F, P, input, packed, temp);
}

int pg_wavelet_ifwt_1d_border(int wavelet, const double* packed, int64_t n, int levels, double* output, double* temp,
                              void* stream) {
    WFilter F;
    wv::Plan1d P;
    if (!filter_of(wavelet, &F)) return bad_arg("pg_wavelet_ifwt_1d_border: unknown wavelet");
    if (!wv::plan_1d(F, n, levels, &P)) return bad_arg("pg_wavelet_ifwt_1d_border: n must be >= 2, levels in 0..40");
    if (!P.inv_ok) return bad_arg("pg_wavelet_ifwt_1d_border: the inverse's length goes below zero at a level");
    if (!packed || (P.inverse_n && !output) || (P.temp && !temp) || !disjoint(packed, P.packed, output, P.inverse_n) ||
        (P.temp && (!disjoint(packed, P.packed, temp, P.temp) || !disjoint(output, P.inverse_n, temp, P.temp))))
        return bad_arg("pg_wavelet_ifwt_1d_border: packed, output and temp must be distinct arrays");
    DeviceExec ex{(cudaStream_t)stream};
    return wv::run_ifwt_1d(ex, F, P, packed, output, temp);
}

int pg_wavelet_fwt_2d_border(int wavelet_x, int wavelet_y, const double* input, int64_t h, int64_t w, int levels,
                             double* packed, double* temp, void* stream) {
    WFilter Fx, Fy;
    wv::Plan2d P;
    if (!filter_of(wavelet_x, &Fx) || !filter_of(wavelet_y, &Fy))
        return bad_arg("pg_wavelet_fwt_2d_border: unknown wavelet");
    if (!wv::plan_2d(Fx, Fy, h, w, levels, &P))
        return bad_arg("pg_wavelet_fwt_2d_border: h and w must be >= 2, levels in 0..40");
    const i64 nin = h * w;
    if (!input || !packed || (P.temp && !temp) || !disjoint(input, nin, packed, P.packed) ||
        (P.temp && (!disjoint(input, nin, temp, P.temp) || !disjoint(packed, P.packed, temp, P.temp))))
        return bad_arg("pg_wavelet_fwt_2d_border: input, packed and temp must be distinct arrays");
    DeviceExec ex{(cudaStream_t)stream};
    return wv::run_fwt_2d(ex, Fx, Fy, P, input, packed, temp);
}

int pg_wavelet_ifwt_2d_border(int wavelet_x, int wavelet_y, const double* packed, int64_t h, int64_t w, int levels,
                              double* output, double* temp, void* stream) {
    WFilter Fx, Fy;
    wv::Plan2d P;
    if (!filter_of(wavelet_x, &Fx) || !filter_of(wavelet_y, &Fy))
        return bad_arg("pg_wavelet_ifwt_2d_border: unknown wavelet");
    if (!wv::plan_2d(Fx, Fy, h, w, levels, &P))
        return bad_arg("pg_wavelet_ifwt_2d_border: h and w must be >= 2, levels in 0..40");
    if (!P.inv_ok) return bad_arg("pg_wavelet_ifwt_2d_border: the inverse's size goes below zero at a level");
    const i64 nout = P.inverse_h * P.inverse_w;
    if (!packed || (nout && !output) || (P.temp && !temp) || !disjoint(packed, P.packed, output, nout) ||
        (P.temp && (!disjoint(packed, P.packed, temp, P.temp) || !disjoint(output, nout, temp, P.temp))))
        return bad_arg("pg_wavelet_ifwt_2d_border: packed, output and temp must be distinct arrays");
    DeviceExec ex{(cudaStream_t)stream};
    return wv::run_ifwt_2d(ex, Fx, Fy, P, packed, output, temp);
}

int pg_wavelet_div_coeff_2d_border(int wavelet_x, int wavelet_y, const double* vx, const double* vy, int64_t h,
                                   int64_t w, int levels, double* div, double* n, void* stream) {
    WFilter Fx, Fy;
    wv::Plan2d P;
    if (!filter_of(wavelet_x, &Fx) || !filter_of(wavelet_y, &Fy))
        return bad_arg("pg_wavelet_div_coeff_2d_border: unknown wavelet");
    if (!wv::plan_2d(Fx, Fy, h, w, levels, &P))
        return bad_arg("pg_wavelet_div_coeff_2d_border: h and w must be >= 2, levels in 0..40");
    const i64 m = P.packed;
    if (!vx || !vy || !div || !n || !disjoint(div, m, n, m) || !disjoint(div, m, vx, m) || !disjoint(div, m, vy, m) ||
        !disjoint(n, m, vx, m) || !disjoint(n, m, vy, m))
        return bad_arg("pg_wavelet_div_coeff_2d_border: outputs must not overlap each other or the inputs");
    DeviceExec ex{(cudaStream_t)stream};
    return wv::run_div_coeff_2d(ex, P, vx, vy, div, n);
}

}  // extern "C"
