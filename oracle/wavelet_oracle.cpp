// wavelet_oracle.cpp -- CPU restatement of panopaea/src/math/wavelet
// (mod.rs:1-681, filters haar.rs:6-9 and spline.rs), TEST INFRASTRUCTURE
// ONLY: the GPU transforms of panopaea_gb300/csrc/pg_wavelet.cu are checked
// against it.  Loops follow the reference as written: down_convolution
// folds with MirrorSampler (mod.rs:52-79), up_convolution scatters with the
// wrapped index (mod.rs:81-112), and the level loops, temporaries and axis
// orders of fwt_1d ... div_coeff_2d, inv_div_coeff_2d (mod.rs:114-451), and
// the border variants fwt_1d_border ... div_coeff_2d_border (mod.rs:454-681).
#include <algorithm>
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

// ---------------------------------------------------------------------------
// Border variants (mod.rs:454-681): zero sampling, bands of s / 2 + 2 B
// samples (B = the border width, the filter length), the forward down
// convolution shifted by B bands and the inverse scatter shifted back by 2 B.
// Transforms are packed into one array: the coarse band, then per level
// (finest first) its detail band(s) -- 1D: detail; 2D: lyhx, hylx, hyhx
// (the [detail_lyhx, detail_hylx, detail_hyhx] order of mod.rs:594).

namespace {

double zero_fetch(const Line& in, idx i) { return i >= 0 && i < in.len ? in[i] : 0.0; }  // mod.rs:26-35

void down_convolution_border(const Filt& W, const Line& in, const Line& coarse, const Line& detail) {  // mod.rs:488-514
    const idx n = W.n, fh = n / 2, bw = n, half = detail.len;
    for (idx i = 0; i < half; ++i) {
        double acc = 0.0;
        for (idx f = 0; f < n; ++f) acc = zero_fetch(in, 2 * (i - bw) + f - fh + 1) * W.dl[n - 1 - f] + acc;
        coarse[i] = acc;
    }
    for (idx i = 0; i < half; ++i) {
        double acc = 0.0;
        for (idx f = 0; f < n; ++f) acc = zero_fetch(in, 2 * (i - bw) + f - fh + 1) * W.dh[n - 1 - f] + acc;
        detail[i] = acc;
    }
}

void up_convolution_border(const Filt& W, const Line& coarse, const Line& detail, const Line& out) {  // mod.rs:516-549
    const idx n = W.n, len = coarse.len + detail.len, half = len / 2, fh = n / 2, bw = n;
    for (idx k = 0; k < out.len; ++k) out[k] = 0.0;
    for (idx i = 0; i < half; ++i)
        for (idx f = 0; f < n; ++f) {
            const idx id = 2 * i + f - fh + 1;
            const idx o = (id < 0 ? (id + len) % len : id % len) - 2 * bw;
            if (o < 0 || o >= out.len) continue;
            out[o] += zero_fetch(coarse, i) * W.ul[f] + zero_fetch(detail, i) * W.uh[f];
        }
}

struct Arr2 {
    idx r = 0, c = 0;
    std::vector<double> v;
    Arr2() = default;
    Arr2(idx r_, idx c_) : r(r_), c(c_), v(r_ * c_, 0.0) {}
    Line row(idx i) { return Line{v.data() + i * c, 1, c}; }
    Line col(idx j) { return Line{v.data() + j, c, r}; }
};

// fwt_1d_border (mod.rs:454-472)
void fwt1b(const Filt& W, std::vector<double> coarse, int levels, std::vector<double>* out_coarse,
           std::vector<std::vector<double>>* details) {
    for (int k = 0; k < levels; ++k) {
        const idx band = (idx)coarse.size() / 2 + 2 * W.n;
        std::vector<double> detail(band), down(band);
        down_convolution_border(W, Line{coarse.data(), 1, (idx)coarse.size()}, Line{down.data(), 1, band},
                                Line{detail.data(), 1, band});
        details->push_back(detail);
        coarse = down;
    }
    *out_coarse = coarse;
}

// fwt_2d_separate_isotropic_border (mod.rs:551-597)
void fwt2b(const Filt& Wx, const Filt& Wy, Arr2 coarse, int levels, Arr2* out_coarse, std::vector<Arr2>* details) {
    for (int k = 0; k < levels; ++k) {
        const idx br = coarse.r / 2 + 2 * Wy.n, bc = coarse.c / 2 + 2 * Wx.n;
        Arr2 down_lx(coarse.r, bc), detail_hx(coarse.r, bc), lyhx(br, bc), hylx(br, bc), hyhx(br, bc), down(br, bc);
        for (idx i = 0; i < coarse.r; ++i) down_convolution_border(Wx, coarse.row(i), down_lx.row(i), detail_hx.row(i));
        for (idx i = 0; i < bc; ++i) {
            down_convolution_border(Wy, down_lx.col(i), down.col(i), hylx.col(i));
            down_convolution_border(Wy, detail_hx.col(i), lyhx.col(i), hyhx.col(i));
        }
        coarse = down;
        details->push_back(lyhx);
        details->push_back(hylx);
        details->push_back(hyhx);
    }
    *out_coarse = coarse;
}

// ifwt_2d_separate_isotropic_border (mod.rs:599-641): y, then x
Arr2 ifwt2b(const Filt& Wx, const Filt& Wy, Arr2 coarse, std::vector<Arr2>& details, int levels) {
    for (int k = levels - 1; k >= 0; --k) {
        Arr2& lyhx = details[3 * k];
        Arr2& hylx = details[3 * k + 1];
        Arr2& hyhx = details[3 * k + 2];
        const idx ur = 2 * coarse.r - 4 * Wy.n, uc = 2 * coarse.c - 4 * Wx.n;
        Arr2 up(ur, uc), up_lx(ur, coarse.c), detail_hx(ur, coarse.c);
        for (idx i = 0; i < coarse.c; ++i) {
            up_convolution_border(Wy, coarse.col(i), hylx.col(i), up_lx.col(i));
            up_convolution_border(Wy, lyhx.col(i), hyhx.col(i), detail_hx.col(i));
        }
        for (idx i = 0; i < ur; ++i) up_convolution_border(Wx, up_lx.row(i), detail_hx.row(i), up.row(i));
        coarse = up;
    }
    return coarse;
}

// Band sizes of the forward transforms: s_{k+1} = s_k / 2 + 2 B.
std::vector<idx> bands(idx s, int levels, idx bw) {
    std::vector<idx> b;
    for (int k = 0; k < levels; ++k) {
        s = s / 2 + 2 * bw;
        b.push_back(s);
    }
    return b;
}

}  // namespace

WVO_EXPORT void wvo_fwt_1d_border(int wavelet, const double* in, long n, int levels, double* packed) {
    const Filt W = filt(wavelet);
    std::vector<double> coarse;
    std::vector<std::vector<double>> details;
    fwt1b(W, std::vector<double>(in, in + n), levels, &coarse, &details);
    for (double v : coarse) *packed++ = v;
    for (auto& d : details)
        for (double v : d) *packed++ = v;
}

// ifwt_1d_border (mod.rs:474-486) of a packed fwt_1d_border of length n
WVO_EXPORT long wvo_ifwt_1d_border(int wavelet, const double* packed, long n, int levels, double* out) {
    const Filt W = filt(wavelet);
    const std::vector<idx> b = bands(n, levels, W.n);
    std::vector<double> coarse(packed, packed + (levels ? b.back() : n));
    const double* p = packed + coarse.size();
    std::vector<const double*> dp;
    for (int k = 0; k < levels; ++k) {
        dp.push_back(p);
        p += b[k];
    }
    for (int k = levels - 1; k >= 0; --k) {
        const idx len = (idx)coarse.size() + b[k];
        std::vector<double> up(len - 4 * W.n);
        up_convolution_border(W, Line{coarse.data(), 1, (idx)coarse.size()}, Line{(double*)dp[k], 1, b[k]},
                              Line{up.data(), 1, (idx)up.size()});
        coarse = up;
    }
    for (double v : coarse) *out++ = v;
    return (long)coarse.size();
}

WVO_EXPORT void wvo_fwt_2d_border(int wx, int wy, const double* in, long h, long w, int levels, double* packed) {
    const Filt Fx = filt(wx), Fy = filt(wy);
    Arr2 x(h, w), coarse;
    std::copy(in, in + h * w, x.v.begin());
    std::vector<Arr2> details;
    fwt2b(Fx, Fy, x, levels, &coarse, &details);
    for (double v : coarse.v) *packed++ = v;
    for (auto& d : details)
        for (double v : d.v) *packed++ = v;
}

namespace {
// The packed 2D transform of an (h, w) input as arrays.
void unpack2(const Filt& Fx, const Filt& Fy, const double* packed, long h, long w, int levels, Arr2* coarse,
             std::vector<Arr2>* details) {
    const std::vector<idx> br = bands(h, levels, Fy.n), bc = bands(w, levels, Fx.n);
    *coarse = levels ? Arr2(br.back(), bc.back()) : Arr2(h, w);
    std::copy(packed, packed + coarse->v.size(), coarse->v.begin());
    packed += coarse->v.size();
    for (int k = 0; k < levels; ++k)
        for (int q = 0; q < 3; ++q) {
            Arr2 a(br[k], bc[k]);
            std::copy(packed, packed + a.v.size(), a.v.begin());
            packed += a.v.size();
            details->push_back(a);
        }
}
void pack2(const Arr2& coarse, const std::vector<Arr2>& details, double* packed) {
    for (double v : coarse.v) *packed++ = v;
    for (auto& d : details)
        for (double v : d.v) *packed++ = v;
}
}  // namespace

// ifwt_2d_separate_isotropic_border (mod.rs:599-641) of a packed 2D border
// transform of an (h, w) input; returns the result's number of elements
WVO_EXPORT long wvo_ifwt_2d_border(int wx, int wy, const double* packed, long h, long w, int levels, double* out) {
    const Filt Fx = filt(wx), Fy = filt(wy);
    Arr2 coarse;
    std::vector<Arr2> details;
    unpack2(Fx, Fy, packed, h, w, levels, &coarse, &details);
    const Arr2 r = ifwt2b(Fx, Fy, coarse, details, levels);
    std::copy(r.v.begin(), r.v.end(), out);
    return (long)r.v.size();
}

// div_coeff_2d_border (mod.rs:645-681) of two packed 2D border transforms
WVO_EXPORT void wvo_div_coeff_2d_border(int wx, int wy, const double* vxp, const double* vyp, long h, long w,
                                        int levels, double* divp, double* np_) {
    const Filt Fx = filt(wx), Fy = filt(wy);
    Arr2 vxc, vyc;
    std::vector<Arr2> vxd, vyd;
    unpack2(Fx, Fy, vxp, h, w, levels, &vxc, &vxd);
    unpack2(Fx, Fy, vyp, h, w, levels, &vyc, &vyd);
    std::vector<Arr2> dd, nd;
    for (int k = 0; k < levels; ++k) {
        Arr2 &vx01 = vxd[3 * k], &vx10 = vxd[3 * k + 1], &vx11 = vxd[3 * k + 2];
        Arr2 &vy01 = vyd[3 * k], &vy10 = vyd[3 * k + 1], &vy11 = vyd[3 * k + 2];
        const idx R = vx01.r, Cc = vx01.c;
        Arr2 d01(R, Cc), d10(R, Cc), d11(R, Cc), n01(R, Cc), n10(R, Cc), n11(R, Cc);
        for (idx y = 0; y < R; ++y)
            for (idx x = 0; x < Cc; ++x) {
                const idx q = y * Cc + x, ym = (y > 0 ? y - 1 : 0) * Cc + x, xm = y * Cc + (x > 0 ? x - 1 : 0);
                d01.v[q] = vy01.v[q];
                d10.v[q] = vx10.v[q];
                d11.v[q] = (vx11.v[q] - vy11.v[q]) / 2.0;
                n01.v[q] = vx01.v[q] + (vy01.v[q] - vy01.v[ym]) / 4.0;
                n10.v[q] = vy10.v[q] + (vx10.v[q] - vx10.v[xm]) / 4.0;
                n11.v[q] = (vx11.v[q] + vy11.v[q]) / 2.0;
            }
        dd.push_back(d01);
        dd.push_back(d10);
        dd.push_back(d11);
        nd.push_back(n01);
        nd.push_back(n10);
        nd.push_back(n11);
    }
    pack2(vxc, dd, divp);
    pack2(vyc, nd, np_);
}
