// wavelet_oracle.cpp -- CPU restatement of panopaea/src/math/wavelet
// (mod.rs:1-451, filters haar.rs:6-9 and spline.rs), TEST INFRASTRUCTURE
// ONLY: the GPU transforms of panopaea_gb300/csrc/pg_wavelet.cu are checked
// against it.  Loops follow the reference as written: down_convolution
// folds with MirrorSampler (mod.rs:52-79), up_convolution scatters with the
// wrapped index (mod.rs:81-112), and the level loops, temporaries and axis
// orders of fwt_1d ... div_coeff_2d, inv_div_coeff_2d (mod.rs:114-451).
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <vector>

#define WVO_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

typedef long idx;

struct Filt {
    int n;
    double ul[10], uh[10], dl[10], dh[10];
};

const double S = 0.70710678118654752440084436210484903, A = 0.08838834764831844055010554526310612,
             B = 0.35355339059327376220042218105242451, C = 0.17677669529663688110021109052621225,
             D = 1.06066017177982128660126654315727355, E = 0.5303300858899107, F = 0.03314563036811942,
             G = 0.06629126073623884, H = 0.4198446513295126, I = 0.9943689110435825;

Filt filt(int w) {
    Filt f{};
    auto put = [](double* dst, std::initializer_list<double> v) {
        int k = 0;
        for (double x : v) dst[k++] = x;
    };
    switch (w) {
        case 0:  // haar.rs
            f.n = 2;
            put(f.ul, {S, S});
            put(f.uh, {S, -S});
            put(f.dl, {S, S});
            put(f.dh, {-S, S});
            break;
        case 1:  // spline.rs Bior13
            f.n = 6;
            put(f.ul, {0, 0, S, S, 0, 0});
            put(f.uh, {-A, -A, S, -S, A, A});
            put(f.dl, {-A, A, S, S, A, -A});
            put(f.dh, {0, 0, -S, S, 0, 0});
            break;
        case 2:  // Bior22
            f.n = 6;
            put(f.ul, {0, B, S, B, 0, 0});
            put(f.uh, {0, C, B, -D, B, C});
            put(f.dl, {0, -C, B, D, B, -C});
            put(f.dh, {0, B, -S, B, 0, 0});
            break;
        case 3:  // Bior24
            f.n = 10;
            put(f.ul, {0, 0, 0, B, S, B, 0, 0, 0, 0});
            put(f.uh, {0, -F, -G, C, H, -I, H, C, -G, -F});
            put(f.dl, {0, F, -G, -C, H, I, H, -C, -G, F});
            put(f.dh, {0, 0, 0, B, -S, B, 0, 0, 0, 0});
            break;
        default:  // Bior31
            f.n = 4;
            put(f.ul, {C, E, E, C});
            put(f.uh, {-B, -D, D, B});
            put(f.dl, {-B, D, D, -B});
            put(f.dh, {-C, E, -E, C});
    }
    return f;
}

// A strided 1D view.
struct Line {
    double* p;
    idx stride, len;
    double& operator[](idx k) const { return p[k * stride]; }
};

double mirror(const Line& in, idx i) {  // mod.rs:38-48
    if (i < 0) return in[-i];
    if (i >= in.len) return in[in.len - 1 - (i % in.len)];
    return in[i];
}

void down_convolution(const Filt& W, const Line& in, const Line& out) {  // mod.rs:52-79
    const idx half = out.len / 2, n = W.n, fh = n / 2;
    for (idx i = 0; i < half; ++i) {
        double acc = 0.0;
        for (idx f = 0; f < n; ++f) acc = mirror(in, 2 * i + f - fh + 1) * W.dl[n - 1 - f] + acc;
        out[i] = acc;
    }
    for (idx i = 0; i < half; ++i) {
        double acc = 0.0;
        for (idx f = 0; f < n; ++f) acc = mirror(in, 2 * i + f - fh + 1) * W.dh[n - 1 - f] + acc;
        out[i + half] = acc;
    }
}

void up_convolution(const Filt& W, const Line& in, const Line& out) {  // mod.rs:81-112
    const idx half = out.len / 2, n = W.n, fh = n / 2, len = out.len;
    for (idx k = 0; k < len; ++k) out[k] = 0.0;
    for (idx i = 0; i < half; ++i)
        for (idx f = 0; f < n; ++f) {
            const idx id = 2 * i + f - fh + 1;
            const idx o = id < 0 ? (id + len) % len : id % len;
            out[o] += mirror(in, i) * W.ul[f] + mirror(in, i + half) * W.uh[f];
        }
}

// temp[block] = out[block] (src.assign(&dest) of the level loops)
void assign(double* dst, const double* src, idx rows, idx cols, idx w) {
    for (idx r = 0; r < rows; ++r)
        for (idx c = 0; c < cols; ++c) dst[r * w + c] = src[r * w + c];
}

void rows_down(const Filt& W, double* src, double* dst, idx rows, idx cols, idx w) {
    for (idx r = 0; r < rows; ++r) down_convolution(W, Line{src + r * w, 1, cols}, Line{dst + r * w, 1, cols});
}
void cols_down(const Filt& W, double* src, double* dst, idx rows, idx cols, idx w) {
    for (idx c = 0; c < cols; ++c) down_convolution(W, Line{src + c, w, rows}, Line{dst + c, w, rows});
}
void rows_up(const Filt& W, double* src, double* dst, idx rows, idx cols, idx w) {
    for (idx r = 0; r < rows; ++r) up_convolution(W, Line{src + r * w, 1, cols}, Line{dst + r * w, 1, cols});
}
void cols_up(const Filt& W, double* src, double* dst, idx rows, idx cols, idx w) {
    for (idx c = 0; c < cols; ++c) up_convolution(W, Line{src + c, w, rows}, Line{dst + c, w, rows});
}

}  // namespace

WVO_EXPORT void wvo_fwt_1d(int wavelet, double* out, long n, int levels) {  // mod.rs:114-129
    const Filt W = filt(wavelet);
    std::vector<double> temp(n);
    idx size = n;
    for (int k = 0; k < levels; ++k) {
        assign(temp.data(), out, 1, size, size);
        down_convolution(W, Line{temp.data(), 1, size}, Line{out, 1, size});
        size /= 2;
    }
}

WVO_EXPORT void wvo_ifwt_1d(int wavelet, double* out, long n, int levels) {  // mod.rs:131-143
    const Filt W = filt(wavelet);
    std::vector<double> temp(n);
    idx size = n >> levels;
    for (int k = 0; k < levels; ++k) {
        size *= 2;
        assign(temp.data(), out, 1, size, size);
        up_convolution(W, Line{temp.data(), 1, size}, Line{out, 1, size});
    }
}

// mode 0: isotropic (mod.rs:145-170; = fwt_2d_separate_isotropic with Wx = Wy
// as to the order, mod.rs:206-231); mode 1: anisotropic (mod.rs:262-294)
WVO_EXPORT void wvo_fwt_2d(int mode, int wx, int wy, double* out, long h, long w, int levels) {
    const Filt Fx = filt(wx), Fy = filt(wy);
    std::vector<double> temp(h * w);
    double* t = temp.data();
    if (mode == 0) {
        idx r = h, c = w;
        for (int k = 0; k < levels; ++k) {
            assign(t, out, r, c, w);
            rows_down(Fx, t, out, r, c, w);
            assign(t, out, r, c, w);
            cols_down(Fy, t, out, r, c, w);
            r /= 2;
            c /= 2;
        }
    } else {
        idx r = h, c = w;
        for (int k = 0; k < levels; ++k) {
            assign(t, out, r, c, w);
            rows_down(Fx, t, out, r, c, w);
            c /= 2;
        }
        r = h;
        c = w;
        for (int k = 0; k < levels; ++k) {
            assign(t, out, r, c, w);
            cols_down(Fy, t, out, r, c, w);
            r /= 2;
        }
    }
}

// mode 0: ifwt_2d_isotropic (y then x, mod.rs:172-204);
// mode 2: ifwt_2d_separate_isotropic (x then y, mod.rs:233-260)
WVO_EXPORT void wvo_ifwt_2d(int mode, int wx, int wy, double* out, long h, long w, int levels) {
    const Filt Fx = filt(wx), Fy = filt(wy);
    std::vector<double> temp(h * w);
    double* t = temp.data();
    idx r = h >> levels, c = w >> levels;
    for (int k = 0; k < levels; ++k) {
        r *= 2;
        c *= 2;
        if (mode == 0) {
            assign(t, out, r, c, w);
            cols_up(Fy, t, out, r, c, w);
            assign(t, out, r, c, w);
            rows_up(Fx, t, out, r, c, w);
        } else {
            assign(t, out, r, c, w);
            rows_up(Fx, t, out, r, c, w);
            assign(t, out, r, c, w);
            cols_up(Fy, t, out, r, c, w);
        }
    }
}

WVO_EXPORT void wvo_div_coeff_2d(int levels, const double* vx, const double* vy, double* dv, double* nn, long h,
                                 long w) {  // mod.rs:296-376
    idx r = h, c = w;
    for (int lv = 0; lv < levels; ++lv) {
        r /= 2;
        c /= 2;
        for (idx y = 0; y < r; ++y)
            for (idx x = 0; x < c; ++x) {
                const idx ym = y > 0 ? y - 1 : 0, xm = x > 0 ? x - 1 : 0;
                const idx q01 = y * w + c + x, q10 = (y + r) * w + x, q11 = (y + r) * w + c + x;
                dv[q01] = vy[q01];
                dv[q10] = vx[q10];
                dv[q11] = (vx[q11] - vy[q11]) / 2.0;
                nn[q01] = vx[q01] + (vy[q01] - vy[ym * w + c + x]) / 4.0;
                nn[q10] = vy[q10] + (vx[q10] - vx[(y + r) * w + xm]) / 4.0;
                nn[q11] = (vx[q11] + vy[q11]) / 2.0;
            }
        if (lv == levels - 1)
            for (idx y = 0; y < r; ++y)
                for (idx x = 0; x < c; ++x) {
                    dv[y * w + x] = vx[y * w + x];
                    nn[y * w + x] = vy[y * w + x];
                }
    }
}

WVO_EXPORT void wvo_inv_div_coeff_2d(int levels, const double* dv, const double* nn, double* vx, double* vy, long h,
                                     long w) {  // mod.rs:378-451
    idx r = h >> levels, c = w >> levels;
    for (int lv = 0; lv < levels; ++lv) {
        for (idx y = 0; y < r; ++y)
            for (idx x = 0; x < c; ++x) {
                const idx ym = y > 0 ? y - 1 : 0, xm = x > 0 ? x - 1 : 0;
                const idx q01 = y * w + c + x, q10 = (y + r) * w + x, q11 = (y + r) * w + c + x;
                vx[q01] = nn[q01] - (dv[ym * w + c + x] - dv[q01]) / 4.0;
                vx[q10] = dv[q10];
                vx[q11] = dv[q11] + nn[q11];
                vy[q01] = dv[q01];
                vy[q10] = nn[q10] - (dv[(y + r) * w + xm] - dv[q10]) / 4.0;
                vy[q11] = nn[q11] - dv[q11];
            }
        if (lv == 0)
            for (idx y = 0; y < r; ++y)
                for (idx x = 0; x < c; ++x) {
                    vx[y * w + x] = dv[y * w + x];
                    vy[y * w + x] = nn[y * w + x];
                }
        r *= 2;
        c *= 2;
    }
}
