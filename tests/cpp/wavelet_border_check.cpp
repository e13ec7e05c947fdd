// Host check of the border wavelet transforms' index arithmetic
// (panopaea_gb300/csrc/pg_wavelet_border.cuh, the code the device launches
// run): an executor that runs every pass as a loop over its output samples
// on the CPU, on arrays sized exactly as the level plans say (built with
// AddressSanitizer where the compiler has it, so a read or write outside an
// array stops the check).  Each result is compared bit for bit with the
// oracle's restatement of mod.rs:454-681 (oracle/wavelet_oracle.cpp).  No
// kernel runs.  Prints "<cases> cases, <bad> wrong".
#define __host__
#define __device__
#define __forceinline__ inline
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "pg_wavelet_border.cuh"

extern "C" {
void wvo_fwt_1d_border(int wavelet, const double* in, long n, int levels, double* packed);
long wvo_ifwt_1d_border(int wavelet, const double* packed, long n, int levels, double* out);
void wvo_fwt_2d_border(int wx, int wy, const double* in, long h, long w, int levels, double* packed);
long wvo_ifwt_2d_border(int wx, int wy, const double* packed, long h, long w, int levels, double* out);
void wvo_div_coeff_2d_border(int wx, int wy, const double* vxp, const double* vyp, long h, long w, int levels,
                             double* divp, double* np_);
}

using namespace pg::wv;

namespace {

struct HostExec {
    int down(const double* src, WLines in, double* lo, double* hi, WLines out, const WFilter& F) {
        for (i64 t = 0; t < in.lines * 2 * out.len; ++t) wdown_border_at(src, in, lo, hi, out, F, t);
        return 0;
    }
    int up(const double* c, WLines cl, const double* d, WLines dl, double* dst, WLines out, const WFilter& F) {
        for (i64 t = 0; t < out.lines * out.len; ++t) wup_border_at(c, cl, d, dl, dst, out, F, t);
        return 0;
    }
    int div(const double* vx, const double* vy, double* dv, double* nn, i64 R, i64 C) {
        for (i64 t = 0; t < R * C; ++t) wdiv_border_at(vx, vy, dv, nn, R, C, t);
        return 0;
    }
    int copy(const double* src, double* dst, i64 n) {
        std::memcpy(dst, src, sizeof(double) * n);
        return 0;
    }
};

std::mt19937_64 rng(11);
std::vector<double> randn(i64 n) {
    std::normal_distribution<double> d;
    std::vector<double> v(n);
    for (auto& x : v) x = d(rng);
    return v;
}
// a null pointer for an empty scratch array, as callers may pass
double* data_or_null(std::vector<double>& v) { return v.empty() ? nullptr : v.data(); }

long cases = 0, bad = 0;
void expect(bool ok, const char* what, int a, int b, long h, long w, int levels) {
    ++cases;
    if (!ok) {
        ++bad;
        if (bad <= 20) std::printf("MISMATCH %s wavelets %d,%d size %ld x %ld levels %d\n", what, a, b, h, w, levels);
    }
}
bool same(const std::vector<double>& a, const std::vector<double>& b) {
    return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), sizeof(double) * a.size()) == 0);
}

void check_1d(int wavelet, long n, int levels) {
    WFilter F;
    Plan1d P;
    if (!filter_of(wavelet, &F) || !plan_1d(F, n, levels, &P)) {
        expect(false, "plan_1d", wavelet, 0, n, 1, levels);
        return;
    }
    HostExec ex;
    std::vector<double> in = randn(n), packed(P.packed), temp(P.temp), out(P.inv_ok ? P.inverse_n : 0);
    run_fwt_1d(ex, F, P, in.data(), packed.data(), data_or_null(temp));
    std::vector<double> ref(P.packed);
    wvo_fwt_1d_border(wavelet, in.data(), n, levels, ref.data());
    expect(same(packed, ref), "fwt_1d_border", wavelet, 0, n, 1, levels);
    if (!P.inv_ok) return;  // the reference's inverse sizes underflow
    run_ifwt_1d(ex, F, P, packed.data(), data_or_null(out), data_or_null(temp));
    std::vector<double> iref(P.packed + n);
    const long m = wvo_ifwt_1d_border(wavelet, packed.data(), n, levels, iref.data());
    iref.resize(m);
    expect(same(out, iref), "ifwt_1d_border", wavelet, 0, n, 1, levels);
}

void check_2d(int wx, int wy, long h, long w, int levels) {
    WFilter Fx, Fy;
    Plan2d P;
    if (!filter_of(wx, &Fx) || !filter_of(wy, &Fy) || !plan_2d(Fx, Fy, h, w, levels, &P)) {
        expect(false, "plan_2d", wx, wy, h, w, levels);
        return;
    }
    HostExec ex;
    std::vector<double> in = randn(h * w), packed(P.packed), temp(P.temp),
        out(P.inv_ok ? P.inverse_h * P.inverse_w : 0);
    run_fwt_2d(ex, Fx, Fy, P, in.data(), packed.data(), data_or_null(temp));
    std::vector<double> ref(P.packed);
    wvo_fwt_2d_border(wx, wy, in.data(), h, w, levels, ref.data());
    expect(same(packed, ref), "fwt_2d_border", wx, wy, h, w, levels);
    if (P.inv_ok) {
        run_ifwt_2d(ex, Fx, Fy, P, packed.data(), data_or_null(out), data_or_null(temp));
        std::vector<double> iref(P.inverse_h * P.inverse_w + 1);
        const long m = wvo_ifwt_2d_border(wx, wy, packed.data(), h, w, levels, iref.data());
        iref.resize(m);
        expect(same(out, iref), "ifwt_2d_border", wx, wy, h, w, levels);
    }
    // div_coeff_2d_border of two transforms
    std::vector<double> vy = randn(P.packed), dv(P.packed), nn(P.packed), dref(P.packed), nref(P.packed);
    run_div_coeff_2d(ex, P, packed.data(), vy.data(), dv.data(), nn.data());
    wvo_div_coeff_2d_border(wx, wy, packed.data(), vy.data(), h, w, levels, dref.data(), nref.data());
    expect(same(dv, dref) && same(nn, nref), "div_coeff_2d_border", wx, wy, h, w, levels);
}

}  // namespace

int main() {
    for (int wv = 0; wv < 5; ++wv)
        for (long n = 2; n <= 72; ++n)
            for (int levels = 0; levels <= 6; ++levels) check_1d(wv, n, levels);
    for (int wv = 0; wv < 5; ++wv)
        for (long n : {255L, 256L, 1000L, 4097L})
            for (int levels = 0; levels <= 8; ++levels) check_1d(wv, n, levels);
    const int pairs[][2] = {{0, 0}, {1, 1}, {2, 2}, {3, 3}, {4, 4}, {0, 3}, {3, 0}, {1, 4}, {4, 2}, {2, 1}};
    const long sizes[] = {2, 3, 5, 8, 13, 16, 31, 40};
    for (auto& p : pairs)
        for (long h : sizes)
            for (long w : sizes)
                for (int levels = 0; levels <= 4; ++levels) check_2d(p[0], p[1], h, w, levels);
    for (auto& p : pairs) check_2d(p[0], p[1], 96, 130, 3);
    std::printf("%ld cases, %ld wrong\n", cases, bad);
    return bad ? 1 : 0;
}
