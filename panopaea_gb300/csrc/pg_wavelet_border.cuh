// pg_wavelet_border.cuh -- the border variants of the wavelet transforms
// (panopaea/src/math/wavelet/mod.rs:454-681): the per-sample arithmetic and
// the level plans.  The same code drives the device launches of
// pg_wavelet.cu and the host check of the index arithmetic in
// tests/cpp/wavelet_border_check.cpp (an executor that loops on the CPU).
//
// The border transforms sample outside a line as zero (ZeroSampler,
// mod.rs:26-35) and keep B extra coefficients on each side of every band,
// B the border width (the filter length): a band of an s-sample line has
// s / 2 + 2 B samples.  The inverse scatters with the index wrapped over
// the coarse + detail length and shifted back by 2 B.  A transform is packed
// into one array: the coarse band, then per level (finest first) its detail
// band (1D) or its three detail bands lyhx, hylx, hyhx (2D, the order of
// mod.rs:594), each row-major.
#pragma once

#include <algorithm>
#include <cstdint>
#include <initializer_list>
#include <vector>

#include "panopaea_gpu.h"

namespace pg {
namespace wv {

typedef int64_t i64;

constexpr int kMaxTaps = 10;

struct WFilter {
    int n;
    double down_low[kMaxTaps], down_high[kMaxTaps], up_low[kMaxTaps], up_high[kMaxTaps];
};

// The filter tables of haar.rs:6-9 and spline.rs (bior 1.3, 2.2, 2.4, 3.1).
constexpr double kS = 0.70710678118654752440084436210484903;
constexpr double kA = 0.08838834764831844055010554526310612;
constexpr double kB = 0.35355339059327376220042218105242451;
constexpr double kC = 0.17677669529663688110021109052621225;
constexpr double kD = 1.06066017177982128660126654315727355;
constexpr double kE = 0.5303300858899107;
constexpr double kF = 0.03314563036811942;
constexpr double kG = 0.06629126073623884;
constexpr double kH = 0.4198446513295126;
constexpr double kI = 0.9943689110435825;

inline bool filter_of(int wavelet, WFilter* out) {
    WFilter f{};
    auto set = [&](int n, std::initializer_list<double> ul, std::initializer_list<double> uh,
                   std::initializer_list<double> dl, std::initializer_list<double> dh) {
        f.n = n;
        int k = 0;
        for (double v : ul) f.up_low[k++] = v;
        k = 0;
        for (double v : uh) f.up_high[k++] = v;
        k = 0;
        for (double v : dl) f.down_low[k++] = v;
        k = 0;
        for (double v : dh) f.down_high[k++] = v;
    };
    switch (wavelet) {
        case PG_WAVELET_HAAR:
            set(2, {kS, kS}, {kS, -kS}, {kS, kS}, {-kS, kS});
            break;
        case PG_WAVELET_BIOR13:
            set(6, {0, 0, kS, kS, 0, 0}, {-kA, -kA, kS, -kS, kA, kA}, {-kA, kA, kS, kS, kA, -kA}, {0, 0, -kS, kS, 0, 0});
            break;
        case PG_WAVELET_BIOR22:
            set(6, {0, kB, kS, kB, 0, 0}, {0, kC, kB, -kD, kB, kC}, {0, -kC, kB, kD, kB, -kC}, {0, kB, -kS, kB, 0, 0});
            break;
        case PG_WAVELET_BIOR24:
            set(10, {0, 0, 0, kB, kS, kB, 0, 0, 0, 0}, {0, -kF, -kG, kC, kH, -kI, kH, kC, -kG, -kF},
                {0, kF, -kG, -kC, kH, kI, kH, -kC, -kG, kF}, {0, 0, 0, kB, -kS, kB, 0, 0, 0, 0});
            break;
        case PG_WAVELET_BIOR31:
            set(4, {kC, kE, kE, kC}, {-kB, -kD, kD, kB}, {-kB, kD, kD, -kB}, {-kC, kE, -kE, kC});
            break;
        default:
            return false;
    }
    *out = f;
    return true;
}

// Correctly rounded FP64 operations, never contracted into a fused
// multiply-add: the reference evaluates a * b + c as two roundings.
__host__ __device__ __forceinline__ double wmul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ __forceinline__ double wadd(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ __forceinline__ double wsub(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
__host__ __device__ __forceinline__ double wdiv(double a, double b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}

// `lines` lines of `len` samples; sample k of line l at l * ls + k * es.
struct WLines {
    i64 lines, len, ls, es;
};

// ZeroSampler::fetch (mod.rs:26-35)
__host__ __device__ __forceinline__ double zfetch(const double* line, i64 es, i64 len, i64 k) {
    return k >= 0 && k < len ? line[k * es] : 0.0;
}

// down_convolution_border (mod.rs:488-514), output t of in.lines * 2 *
// out.len: sample i of line l of the low band (lo) or the high band (hi),
// the fold over taps f of zero(src, 2 (i - B) + f - n/2 + 1) * filter[n-1-f].
__host__ __device__ __forceinline__ void wdown_border_at(const double* src, const WLines& in, double* lo, double* hi,
                                                         const WLines& out, const WFilter& F, i64 t) {
    const i64 band = out.len;
    const i64 l = t / (2 * band), o = t - l * 2 * band;
    const bool high = o >= band;
    const i64 i = high ? o - band : o;
    const int n = F.n, fh = n / 2;
    const double* line = src + l * in.ls;
    const double* filt = high ? F.down_high : F.down_low;
    double acc = 0.0;
    for (int f = 0; f < n; ++f)
        acc = wadd(wmul(zfetch(line, in.es, in.len, 2 * (i - n) + f - fh + 1), filt[n - 1 - f]), acc);
    (high ? hi : lo)[l * out.ls + i * out.es] = acc;
}

// up_convolution_border (mod.rs:516-549) gathered, output t of out.lines *
// out.len: sample j of line l receives, in increasing (i, f) order,
// zero(c, i) * up_low[f] + zero(d, i) * up_high[f] for every i < (c.len +
// d.len) / 2 and tap f whose index 2 i + f - n/2 + 1, wrapped over c.len +
// d.len and less 2 B, is j.  The host guarantees c.len + d.len >= n, so the
// unwrapped index is within one period of the wrapped one, and at most one
// i per tap contributes.
__host__ __device__ __forceinline__ void wup_border_at(const double* cs, const WLines& c, const double* ds,
                                                       const WLines& d, double* dst, const WLines& out,
                                                       const WFilter& F, i64 t) {
    const i64 l = t / out.len, j = t - l * out.len;
    const i64 L = c.len + d.len, half = L / 2;
    const int n = F.n, fh = n / 2;
    const i64 wrapped = j + 2 * n;
    i64 ci[kMaxTaps];
    int cf[kMaxTaps];
    int m = 0;
    if (wrapped < L)
        for (int f = 0; f < n; ++f)
            for (int w = -1; w <= 1; ++w) {
                const i64 idx = wrapped + w * L;  // unwrapped 2 i + f - n/2 + 1
                const i64 two_i = idx - f + fh - 1;
                if (two_i < 0 || (two_i & 1) || two_i / 2 >= half) continue;
                const i64 ref = idx < 0 ? (idx + L) % L : idx % L;  // the reference's wrap
                if (ref != wrapped || m == kMaxTaps) continue;
                ci[m] = two_i / 2;
                cf[m] = f;
                ++m;
            }
    for (int a = 1; a < m; ++a) {  // insertion sort by (i, f)
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
    const double* cl = cs + l * c.ls;
    const double* dl = ds + l * d.ls;
    double acc = 0.0;
    for (int a = 0; a < m; ++a) {
        const i64 i = ci[a];
        const int f = cf[a];
        acc = wadd(acc, wadd(wmul(zfetch(cl, c.es, c.len, i), F.up_low[f]), wmul(zfetch(dl, d.es, d.len, i), F.up_high[f])));
    }
    dst[l * out.ls + j * out.es] = acc;
}

// div_coeff_2d_border (mod.rs:645-681), sample t of one level's R x C
// bands; each pointer is the level's [01 | 10 | 11] = [lyhx | hylx | hyhx]
// triple.
__host__ __device__ __forceinline__ void wdiv_border_at(const double* vx, const double* vy, double* dv, double* nn,
                                                        i64 R, i64 C, i64 t) {
    const i64 y = t / C, x = t - y * C, P = R * C;
    const i64 qym = (y > 0 ? y - 1 : 0) * C + x, qxm = y * C + (x > 0 ? x - 1 : 0);
    dv[t] = vy[t];
    dv[P + t] = vx[P + t];
    dv[2 * P + t] = wdiv(wsub(vx[2 * P + t], vy[2 * P + t]), 2.0);
    nn[t] = wadd(vx[t], wdiv(wsub(vy[t], vy[qym]), 4.0));
    nn[P + t] = wadd(vy[P + t], wdiv(wsub(vx[P + t], vx[P + qxm]), 4.0));
    nn[2 * P + t] = wdiv(wadd(vx[2 * P + t], vy[2 * P + t]), 2.0);
}

// ---------------------------------------------------------------------------
// Level plans: band sizes, packed offsets, scratch sizes.

struct Plan1d {
    int levels = 0, bw = 0;
    i64 n = 0;
    std::vector<i64> band;     // band[k]: samples of level k's bands (finest first)
    std::vector<i64> det_off;  // packed offset of level k's detail band
    std::vector<i64> inv;      // inv[k]: length after the inverse undoes level k
    i64 packed = 0, slot = 0, temp = 0, inverse_n = 0;
    bool inv_ok = true;  // false: a level of the inverse has a negative length
};

// false: arguments the forward transform does not take (n < 2, levels
// outside 0..40).  inv_ok false: the inverse's size arithmetic goes below
// zero at some level (in the reference an unsigned underflow, which stops
// the program), so only the forward transform runs.
inline bool plan_1d(const WFilter& F, i64 n, int levels, Plan1d* P) {
    if (n < 2 || levels < 0 || levels > 40) return false;
    Plan1d p;
    p.levels = levels;
    p.bw = F.n;
    p.n = n;
    i64 s = n;
    for (int k = 0; k < levels; ++k) {  // fwt_1d_border, mod.rs:454-472
        s = s / 2 + 2 * p.bw;
        p.band.push_back(s);
    }
    if (levels == 0) {
        p.packed = p.inverse_n = n;
        *P = p;
        return true;
    }
    i64 off = p.band.back();
    for (int k = 0; k < levels; ++k) {
        p.det_off.push_back(off);
        off += p.band[k];
    }
    p.packed = off;
    p.inv.assign(levels, 0);
    i64 cl = p.band.back(), slot = *std::max_element(p.band.begin(), p.band.end());
    for (int k = levels - 1; k >= 0 && p.inv_ok; --k) {  // ifwt_1d_border, mod.rs:474-486
        const i64 len = cl + p.band[k];
        // the gather of wup_border_at also wants len >= n (always true here:
        // both lengths are at least 2 B - 1)
        if (len < F.n || len - 4 * p.bw < 0) {
            p.inv_ok = false;
            break;
        }
        p.inv[k] = cl = len - 4 * p.bw;
        slot = std::max(slot, cl);
    }
    p.inverse_n = p.inv_ok ? p.inv[0] : -1;
    p.slot = slot;
    p.temp = 2 * slot;
    *P = p;
    return true;
}

struct Plan2d {
    int levels = 0, bx = 0, by = 0;
    i64 h = 0, w = 0;
    std::vector<i64> br, bc;    // band rows, columns of level k
    std::vector<i64> det_off;   // packed offset of level k's lyhx (hylx, hyhx follow)
    std::vector<i64> ur, uc;    // the inverse's output rows, columns at level k
    i64 packed = 0, slot_lx = 0, slot_c = 0, temp = 0, inverse_h = 0, inverse_w = 0;
    bool inv_ok = true;  // false: a level of the inverse has a negative size
    i64 coarse_r() const { return levels ? br.back() : h; }
    i64 coarse_c() const { return levels ? bc.back() : w; }
};

// As plan_1d: false for arguments the forward transform does not take,
// inv_ok false where the inverse's sizes go below zero.
inline bool plan_2d(const WFilter& Fx, const WFilter& Fy, i64 h, i64 w, int levels, Plan2d* P) {
    if (h < 2 || w < 2 || levels < 0 || levels > 40) return false;
    Plan2d p;
    p.levels = levels;
    p.bx = Fx.n;
    p.by = Fy.n;
    p.h = h;
    p.w = w;
    i64 r = h, c = w, lx = 0, cs = 0;
    for (int k = 0; k < levels; ++k) {  // fwt_2d_separate_isotropic_border, mod.rs:551-597
        const i64 brk = r / 2 + 2 * p.by, bck = c / 2 + 2 * p.bx;
        lx = std::max(lx, r * bck);  // down_lx, detail_hx
        cs = std::max(cs, brk * bck);
        p.br.push_back(brk);
        p.bc.push_back(bck);
        r = brk;
        c = bck;
    }
    i64 off = p.coarse_r() * p.coarse_c();
    for (int k = 0; k < levels; ++k) {
        p.det_off.push_back(off);
        off += 3 * p.br[k] * p.bc[k];
    }
    p.packed = off;
    p.ur.assign(levels, 0);
    p.uc.assign(levels, 0);
    i64 cr = p.coarse_r(), cc = p.coarse_c();
    for (int k = levels - 1; k >= 0 && p.inv_ok; --k) {  // ifwt_2d_separate_isotropic_border, mod.rs:599-641
        const i64 urk = 2 * cr - 4 * p.by, uck = 2 * cc - 4 * p.bx;
        // the y pass reads columns 0..cc of the detail bands and wraps over
        // cr + br (coarse with hylx) and 2 br (lyhx with hyhx); the x pass
        // wraps over 2 cc.  Where the sizes stay non-negative, cc <= bc,
        // cr <= br and both wrap lengths are at least the filter length.
        if (urk < 0 || uck < 0 || cc > p.bc[k] || cr > p.br[k] || cr + p.br[k] < Fy.n || 2 * cc < Fx.n) {
            p.inv_ok = false;
            break;
        }
        lx = std::max(lx, urk * cc);  // up_lx, detail_hx
        cs = std::max(cs, urk * uck);
        p.ur[k] = cr = urk;
        p.uc[k] = cc = uck;
    }
    p.inverse_h = !p.inv_ok ? -1 : levels ? p.ur[0] : h;
    p.inverse_w = !p.inv_ok ? -1 : levels ? p.uc[0] : w;
    p.slot_lx = lx;
    p.slot_c = cs;
    p.temp = 2 * lx + 2 * cs;
    *P = p;
    return true;
}

// ---------------------------------------------------------------------------
// The transforms as sequences of passes.  Exec provides
//   int down(const double* src, WLines in, double* lo, double* hi, WLines out, const WFilter&)
//   int up(const double* c, WLines cl, const double* d, WLines dl, double* dst, WLines out, const WFilter&)
//   int div(const double* vx, const double* vy, double* dv, double* nn, i64 R, i64 C)
//   int copy(const double* src, double* dst, i64 count)
// each returning 0 on success.

template <class Exec>
int run_fwt_1d(Exec& ex, const WFilter& F, const Plan1d& P, const double* in, double* packed, double* temp) {
    if (P.levels == 0) return ex.copy(in, packed, P.n);
    const double* src = in;
    i64 s = P.n;
    for (int k = 0; k < P.levels; ++k) {
        double* coarse = k == P.levels - 1 ? packed : temp + (k & 1) * P.slot;
        const i64 b = P.band[k];
        if (int rc = ex.down(src, WLines{1, s, 0, 1}, coarse, packed + P.det_off[k], WLines{1, b, 0, 1}, F)) return rc;
        src = coarse;
        s = b;
    }
    return 0;
}

template <class Exec>
int run_ifwt_1d(Exec& ex, const WFilter& F, const Plan1d& P, const double* packed, double* out, double* temp) {
    if (P.levels == 0) return ex.copy(packed, out, P.n);
    const double* cur = packed;
    i64 cl = P.band.back();
    for (int k = P.levels - 1; k >= 0; --k) {
        double* dst = k == 0 ? out : temp + (k & 1) * P.slot;
        const i64 b = P.band[k];
        if (int rc = ex.up(cur, WLines{1, cl, 0, 1}, packed + P.det_off[k], WLines{1, b, 0, 1}, dst,
                           WLines{1, P.inv[k], 0, 1}, F))
            return rc;
        cur = dst;
        cl = P.inv[k];
    }
    return 0;
}

template <class Exec>
int run_fwt_2d(Exec& ex, const WFilter& Fx, const WFilter& Fy, const Plan2d& P, const double* in, double* packed,
               double* temp) {
    if (P.levels == 0) return ex.copy(in, packed, P.h * P.w);
    double* lx = temp;
    double* hx = temp + P.slot_lx;
    const double* src = in;
    i64 r = P.h, c = P.w;
    for (int k = 0; k < P.levels; ++k) {
        const i64 R = P.br[k], C = P.bc[k];
        double* coarse = k == P.levels - 1 ? packed : temp + 2 * P.slot_lx + (k & 1) * P.slot_c;
        double* lyhx = packed + P.det_off[k];
        double* hylx = lyhx + R * C;
        double* hyhx = hylx + R * C;
        int rc;
        // x: every row of the coarse block -> down_lx, detail_hx (r x C)
        if ((rc = ex.down(src, WLines{r, c, c, 1}, lx, hx, WLines{r, C, C, 1}, Fx))) return rc;
        // y: every column -> (down, hylx) and (lyhx, hyhx) (R x C)
        if ((rc = ex.down(lx, WLines{C, r, 1, C}, coarse, hylx, WLines{C, R, 1, C}, Fy))) return rc;
        if ((rc = ex.down(hx, WLines{C, r, 1, C}, lyhx, hyhx, WLines{C, R, 1, C}, Fy))) return rc;
        src = coarse;
        r = R;
        c = C;
    }
    return 0;
}

template <class Exec>
int run_ifwt_2d(Exec& ex, const WFilter& Fx, const WFilter& Fy, const Plan2d& P, const double* packed, double* out,
                double* temp) {
    if (P.levels == 0) return ex.copy(packed, out, P.h * P.w);
    double* ulx = temp;
    double* uhx = temp + P.slot_lx;
    const double* cur = packed;
    i64 cr = P.coarse_r(), cc = P.coarse_c();
    for (int k = P.levels - 1; k >= 0; --k) {
        const i64 R = P.br[k], C = P.bc[k], ur = P.ur[k], uc = P.uc[k];
        const double* lyhx = packed + P.det_off[k];
        const double* hylx = lyhx + R * C;
        const double* hyhx = hylx + R * C;
        double* dst = k == 0 ? out : temp + 2 * P.slot_lx + (k & 1) * P.slot_c;
        int rc;
        // y: columns 0..cc -> up_lx (coarse with hylx), detail_hx (lyhx with hyhx), ur x cc
        if ((rc = ex.up(cur, WLines{cc, cr, 1, cc}, hylx, WLines{cc, R, 1, C}, ulx, WLines{cc, ur, 1, cc}, Fy)))
            return rc;
        if ((rc = ex.up(lyhx, WLines{cc, R, 1, C}, hyhx, WLines{cc, R, 1, C}, uhx, WLines{cc, ur, 1, cc}, Fy)))
            return rc;
        // x: every row -> up (ur x uc)
        if ((rc = ex.up(ulx, WLines{ur, cc, cc, 1}, uhx, WLines{ur, cc, cc, 1}, dst, WLines{ur, uc, uc, 1}, Fx)))
            return rc;
        cur = dst;
        cr = ur;
        cc = uc;
    }
    return 0;
}

template <class Exec>
int run_div_coeff_2d(Exec& ex, const Plan2d& P, const double* vx, const double* vy, double* dv, double* nn) {
    const i64 nc = P.coarse_r() * P.coarse_c();
    int rc;
    if ((rc = ex.copy(vx, dv, nc)) || (rc = ex.copy(vy, nn, nc))) return rc;
    for (int k = 0; k < P.levels; ++k) {
        const i64 o = P.det_off[k];
        if ((rc = ex.div(vx + o, vy + o, dv + o, nn + o, P.br[k], P.bc[k]))) return rc;
    }
    return 0;
}

}  // namespace wv
}  // namespace pg
