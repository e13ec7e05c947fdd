// unet_oracle.cpp -- CPU restatement of the learned pressure-guess network.
//
// TEST INFRASTRUCTURE ONLY: the GPU kernels of panopaea_gb300/csrc/pg_unet.cu
// are checked against this file (forward output, loss and every weight
// gradient); the product never links it.  The network has no counterpart in
// the reference (panopaea has no learned component); its definition is the
// one the GPU kernels implement:
//
//   level l has dims (d, h, w) >> l, l = 0, 1, 2; tensors are channels-last.
//   X0[v] = (b[v] / s, n_open[v] / 6, 0 x 14), s = sqrt(mean(b^2))
//   L0 16->16, L1 16->16 (skip0)            3x3x3 conv, zero padding, ReLU
//   P0 = avgpool2(L1)                        level 1
//   L2 16->32, L3 32->32 (skip1)
//   P1 = avgpool2(L3)                        level 2
//   L4 32->64, L5 64->64
//   C1 = [up2(L5) | L3]  (96 ch)             level 1, nearest upsampling
//   L6 96->32, L7 32->32
//   C0 = [up2(L7) | L1]  (48 ch)             level 0
//   L8 48->16, L9 16->16
//   q[v] = sum_c L9[v][c] * wh[c]  (0 on solid cells)
//   guess p = q * s * out_scale / dt
//
// Storage rounding (mode "bf16", the GPU's): every stored tensor (inputs,
// activations, activation gradients) and the conv weights are rounded to
// bfloat16 (round to nearest even); sums run in float.  Mode "exact" (double,
// no rounding) is for finite-difference checks of the backward pass.
//
// Loss, e = m (q - t), t = p_true * dt / (s * out_scale), m = 1 on cells with
// an open face: kind 0 (MSE) L = sum e^2 / V0; kind 1 (energy norm)
// L = sum e (A1 e) / V0 with A1 the masked Laplacian at dt = 1 (the fluid
// oracle's operator).  Weight gradients accumulate in double.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#define UNO_EXPORT extern "C" __attribute__((visibility("default")))

// The masked Laplacian of the fluid oracle (pg_oracle.cpp).
extern "C" void pgo_laplacian_f32(float* out, const float* p, double dt, const uint8_t* fs, int nd, long d, long h,
                                  long w);
extern "C" void pgo_laplacian_f64(double* out, const double* p, double dt, const uint8_t* fs, int nd, long d, long h,
                                  long w);

namespace {

typedef long idx;

constexpr int kL = 10;
constexpr int kCin[kL] = {16, 16, 16, 32, 32, 64, 96, 32, 48, 16};
constexpr int kCout[kL] = {16, 16, 32, 32, 64, 64, 32, 32, 16, 16};
constexpr int kLevel[kL] = {0, 0, 1, 1, 2, 2, 1, 1, 0, 0};

idx param_offset(int k) {
    idx o = 0;
    for (int j = 0; j < k; ++j) o += 27L * kCin[j] * kCout[j];
    return o;
}
idx num_params() { return param_offset(kL) + 16; }

float bf16_round(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) {  // inf stays, NaN stays NaN
        if (u & 0x007fffffu) u |= 0x00400000u;
        u &= 0xffff0000u;
    } else {
        u += 0x7fffu + ((u >> 16) & 1u);
        u &= 0xffff0000u;
    }
    std::memcpy(&x, &u, 4);
    return x;
}

template <class R> struct Rnd {
    static R r(R x) { return x; }
};
template <> struct Rnd<float> {
    static float r(float x) { return bf16_round(x); }
};

struct Lv {
    idx d, h, w;
    idx n() const { return d * h * w; }
};

// out[v][co] = relu(sum_tap sum_ci in[v + off(tap)][ci] * w[tap][ci][co])
template <class R>
void conv_fwd(const R* in, int cin, const R* w, int cout, const Lv& L, R* out) {
#pragma omp parallel for schedule(static)
    for (idx z = 0; z < L.d; ++z) {
        std::vector<R> acc(cout);
        for (idx y = 0; y < L.h; ++y)
            for (idx x = 0; x < L.w; ++x) {
                std::fill(acc.begin(), acc.end(), R(0));
                for (int tap = 0; tap < 27; ++tap) {
                    const idx zz = z + tap / 9 - 1, yy = y + (tap / 3) % 3 - 1, xx = x + tap % 3 - 1;
                    if (zz < 0 || zz >= L.d || yy < 0 || yy >= L.h || xx < 0 || xx >= L.w) continue;
                    const R* a = in + ((zz * L.h + yy) * L.w + xx) * cin;
                    const R* wt = w + (idx)tap * cin * cout;
                    for (int ci = 0; ci < cin; ++ci) {
                        const R av = a[ci];
                        if (av == R(0)) continue;
                        for (int co = 0; co < cout; ++co) acc[co] += av * wt[ci * cout + co];
                    }
                }
                R* o = out + ((z * L.h + y) * L.w + x) * cout;
                for (int co = 0; co < cout; ++co) o[co] = Rnd<R>::r(acc[co] > R(0) ? acc[co] : R(0));
            }
    }
}

// dx[u][ci] = sum_tap sum_co dz[u - off(tap)][co] * w[tap][ci][co]  (unrounded)
template <class R>
void conv_bwd_data(const R* dz, int cout, const R* w, int cin, const Lv& L, R* dx) {
#pragma omp parallel for schedule(static)
    for (idx z = 0; z < L.d; ++z) {
        for (idx y = 0; y < L.h; ++y)
            for (idx x = 0; x < L.w; ++x) {
                R* o = dx + ((z * L.h + y) * L.w + x) * cin;
                for (int ci = 0; ci < cin; ++ci) o[ci] = R(0);
                for (int tap = 0; tap < 27; ++tap) {
                    const idx zz = z - (tap / 9 - 1), yy = y - ((tap / 3) % 3 - 1), xx = x - (tap % 3 - 1);
                    if (zz < 0 || zz >= L.d || yy < 0 || yy >= L.h || xx < 0 || xx >= L.w) continue;
                    const R* g = dz + ((zz * L.h + yy) * L.w + xx) * cout;
                    const R* wt = w + (idx)tap * cin * cout;
                    for (int ci = 0; ci < cin; ++ci) {
                        R s = 0;
                        for (int co = 0; co < cout; ++co) s += g[co] * wt[ci * cout + co];
                        o[ci] += s;
                    }
                }
            }
    }
}

// gw[tap][ci][co] += sum_v x[v + off(tap)][ci] * dz[v][co]
template <class R>
void conv_wgrad(const R* x, int cin, const R* dz, int cout, const Lv& L, double* gw) {
#pragma omp parallel for schedule(dynamic)
    for (int tap = 0; tap < 27; ++tap) {
        std::vector<double> acc((size_t)cin * cout, 0.0);
        const int oz = tap / 9 - 1, oy = (tap / 3) % 3 - 1, ox = tap % 3 - 1;
        for (idx z = 0; z < L.d; ++z)
            for (idx y = 0; y < L.h; ++y)
                for (idx xx = 0; xx < L.w; ++xx) {
                    const idx zz = z + oz, yy = y + oy, x2 = xx + ox;
                    if (zz < 0 || zz >= L.d || yy < 0 || yy >= L.h || x2 < 0 || x2 >= L.w) continue;
                    const R* a = x + ((zz * L.h + yy) * L.w + x2) * cin;
                    const R* g = dz + ((z * L.h + y) * L.w + xx) * cout;
                    for (int ci = 0; ci < cin; ++ci) {
                        const double av = (double)a[ci];
                        if (av == 0.0) continue;
                        for (int co = 0; co < cout; ++co) acc[(size_t)ci * cout + co] += av * (double)g[co];
                    }
                }
        double* o = gw + (size_t)tap * cin * cout;
        for (size_t i = 0; i < acc.size(); ++i) o[i] += acc[i];
    }
}

template <class R> void pool(const R* in, int c, const Lv& F, R* out) {
    const Lv C{F.d / 2, F.h / 2, F.w / 2};
    for (idx z = 0; z < C.d; ++z)
        for (idx y = 0; y < C.h; ++y)
            for (idx x = 0; x < C.w; ++x)
                for (int ch = 0; ch < c; ++ch) {
                    R s = 0;
                    for (int k = 0; k < 8; ++k) {
                        const idx zz = 2 * z + (k >> 2), yy = 2 * y + ((k >> 1) & 1), xx = 2 * x + (k & 1);
                        s += in[((zz * F.h + yy) * F.w + xx) * c + ch];
                    }
                    out[((z * C.h + y) * C.w + x) * c + ch] = Rnd<R>::r(R(0.125) * s);
                }
}

// out[v] = [coarse[parent(v)] (ca) | skip[v] (cb)]
template <class R> void upcat(const R* coarse, int ca, const R* skip, int cb, const Lv& F, R* out) {
    const Lv C{F.d / 2, F.h / 2, F.w / 2};
    for (idx z = 0; z < F.d; ++z)
        for (idx y = 0; y < F.h; ++y)
            for (idx x = 0; x < F.w; ++x) {
                const idx v = (z * F.h + y) * F.w + x, u = ((z / 2) * C.h + y / 2) * C.w + x / 2;
                for (int c = 0; c < ca; ++c) out[v * (ca + cb) + c] = coarse[u * ca + c];
                for (int c = 0; c < cb; ++c) out[v * (ca + cb) + ca + c] = skip[v * cb + c];
            }
}

// dz[u][c] = y[u][c] > 0 ? sum_children dcat[child][c] : 0   (c < ca)
template <class R> void upback_gate(const R* dcat, int ct, int ca, const R* y, const Lv& F, R* dz) {
    const Lv C{F.d / 2, F.h / 2, F.w / 2};
    for (idx z = 0; z < C.d; ++z)
        for (idx yy = 0; yy < C.h; ++yy)
            for (idx x = 0; x < C.w; ++x) {
                const idx u = (z * C.h + yy) * C.w + x;
                for (int c = 0; c < ca; ++c) {
                    R s = 0;
                    for (int k = 0; k < 8; ++k) {
                        const idx fz = 2 * z + (k >> 2), fy = 2 * yy + ((k >> 1) & 1), fx = 2 * x + (k & 1);
                        s += dcat[((fz * F.h + fy) * F.w + fx) * ct + c];
                    }
                    dz[u * ca + c] = y[u * ca + c] > R(0) ? Rnd<R>::r(s) : R(0);
                }
            }
}

// dz[v][c] = y[v][c] > 0 ? dcat[v][off + c] + dp[parent(v)][c] / 8 : 0
template <class R>
void poolback_gate(const R* dcat, int ct, int off, const R* dp, int c, const R* y, const Lv& F, R* dz) {
    const Lv C{F.d / 2, F.h / 2, F.w / 2};
    for (idx z = 0; z < F.d; ++z)
        for (idx yy = 0; yy < F.h; ++yy)
            for (idx x = 0; x < F.w; ++x) {
                const idx v = (z * F.h + yy) * F.w + x, u = ((z / 2) * C.h + yy / 2) * C.w + x / 2;
                for (int ch = 0; ch < c; ++ch) {
                    const R s = dcat[v * ct + off + ch] + R(0.125) * dp[u * c + ch];
                    dz[v * c + ch] = y[v * c + ch] > R(0) ? Rnd<R>::r(s) : R(0);
                }
            }
}

template <class R> void gate_round(R* dx, const R* y, idx n) {
    for (idx i = 0; i < n; ++i) dx[i] = y[i] > R(0) ? Rnd<R>::r(dx[i]) : R(0);
}
inline void laplacian1(float* out, const float* p, const uint8_t* fs, idx d, idx h, idx w) {
    pgo_laplacian_f32(out, p, 1.0, fs, 3, d, h, w);
}
inline void laplacian1(double* out, const double* p, const uint8_t* fs, idx d, idx h, idx w) {
    pgo_laplacian_f64(out, p, 1.0, fs, 3, d, h, w);
}

template <class R> void round_all(R* a, idx n) {
    for (idx i = 0; i < n; ++i) a[i] = Rnd<R>::r(a[i]);
}

// Forward (+ loss and gradients when p_true / grad are given).
template <class R>
void run(const R* params, double out_scale, double dt, idx d, idx h, idx w, const R* b, const uint8_t* nopen,
         const uint8_t* face_solid, int loss_kind, const R* p_true, R* p_out, R* grad, double* loss_out) {
    const Lv L0{d, h, w}, L1{d / 2, h / 2, w / 2}, L2{d / 4, h / 4, w / 4};
    const Lv lv[3] = {L0, L1, L2};
    const idx V0 = L0.n();
    std::vector<R> wq(num_params());
    for (idx i = 0; i < num_params(); ++i) wq[i] = i < param_offset(kL) ? Rnd<R>::r(params[i]) : params[i];
    auto W = [&](int k) { return wq.data() + param_offset(k); };
    const R* wh = wq.data() + param_offset(kL);

    double ss = 0.0;
    for (idx v = 0; v < V0; ++v) ss += (double)b[v] * (double)b[v];
    const R s = (R)std::sqrt(ss / (double)V0);
    const R inv_s = s > R(0) ? R(1) / s : R(0);
    std::vector<R> X0(V0 * 16, R(0));
    for (idx v = 0; v < V0; ++v) {
        X0[v * 16] = Rnd<R>::r(b[v] * inv_s);
        X0[v * 16 + 1] = Rnd<R>::r((R)nopen[v] * (R)(1.0f / 6.0f));
    }
    std::vector<R> Y[kL];
    for (int k = 0; k < kL; ++k) Y[k].assign(lv[kLevel[k]].n() * kCout[k], R(0));
    std::vector<R> P0(L1.n() * 16), P1(L2.n() * 32), C1(L1.n() * 96), C0(V0 * 48);
    conv_fwd(X0.data(), 16, W(0), 16, L0, Y[0].data());
    conv_fwd(Y[0].data(), 16, W(1), 16, L0, Y[1].data());
    pool(Y[1].data(), 16, L0, P0.data());
    conv_fwd(P0.data(), 16, W(2), 32, L1, Y[2].data());
    conv_fwd(Y[2].data(), 32, W(3), 32, L1, Y[3].data());
    pool(Y[3].data(), 32, L1, P1.data());
    conv_fwd(P1.data(), 32, W(4), 64, L2, Y[4].data());
    conv_fwd(Y[4].data(), 64, W(5), 64, L2, Y[5].data());
    upcat(Y[5].data(), 64, Y[3].data(), 32, L1, C1.data());
    conv_fwd(C1.data(), 96, W(6), 32, L1, Y[6].data());
    conv_fwd(Y[6].data(), 32, W(7), 32, L1, Y[7].data());
    upcat(Y[7].data(), 32, Y[1].data(), 16, L0, C0.data());
    conv_fwd(C0.data(), 48, W(8), 16, L0, Y[8].data());
    conv_fwd(Y[8].data(), 16, W(9), 16, L0, Y[9].data());

    const R scale = s * (R)out_scale;
    std::vector<R> q(V0);
    for (idx v = 0; v < V0; ++v) {
        R a = 0;
        for (int c = 0; c < 16; ++c) a = a + Y[9][v * 16 + c] * wh[c];
        q[v] = nopen[v] ? a : R(0);
        if (p_out) p_out[v] = q[v] * scale / (R)dt;
    }
    if (!p_true) return;

    const R inv_ps = scale > R(0) ? (R)dt / scale : R(0);
    const R c2 = R(2) / (R)V0;
    std::vector<R> dq(V0), e(V0), ae;
    for (idx v = 0; v < V0; ++v) e[v] = nopen[v] ? q[v] - p_true[v] * inv_ps : R(0);
    if (loss_kind == 1) {
        ae.resize(V0);
        laplacian1(ae.data(), e.data(), face_solid, d, h, w);
    }
    double loss = 0.0;
    for (idx v = 0; v < V0; ++v) {
        const R gv = loss_kind == 1 ? ae[v] : e[v];
        if (nopen[v]) {
            loss += (double)e[v] * (double)gv;
            dq[v] = gv * c2;
        } else {
            dq[v] = R(0);
        }
    }
    if (loss_out) *loss_out = loss / (double)V0;
    if (!grad) return;

    std::vector<double> g(num_params(), 0.0);
    std::vector<R> dZ9(V0 * 16);
    for (idx v = 0; v < V0; ++v)
        for (int c = 0; c < 16; ++c) {
            g[param_offset(kL) + c] += (double)Y[9][v * 16 + c] * (double)dq[v];
            dZ9[v * 16 + c] = Y[9][v * 16 + c] > R(0) ? Rnd<R>::r(dq[v] * wh[c]) : R(0);
        }
    auto gW = [&](int k) { return g.data() + param_offset(k); };
    // L9
    conv_wgrad(Y[8].data(), 16, dZ9.data(), 16, L0, gW(9));
    std::vector<R> dZ8(V0 * 16);
    conv_bwd_data(dZ9.data(), 16, W(9), 16, L0, dZ8.data());
    gate_round(dZ8.data(), Y[8].data(), V0 * 16);
    // L8
    conv_wgrad(C0.data(), 48, dZ8.data(), 16, L0, gW(8));
    std::vector<R> dC0(V0 * 48);
    conv_bwd_data(dZ8.data(), 16, W(8), 48, L0, dC0.data());
    round_all(dC0.data(), V0 * 48);
    std::vector<R> dZ7(L1.n() * 32);
    upback_gate(dC0.data(), 48, 32, Y[7].data(), L0, dZ7.data());
    // L7
    conv_wgrad(Y[6].data(), 32, dZ7.data(), 32, L1, gW(7));
    std::vector<R> dZ6(L1.n() * 32);
    conv_bwd_data(dZ7.data(), 32, W(7), 32, L1, dZ6.data());
    gate_round(dZ6.data(), Y[6].data(), L1.n() * 32);
    // L6
    conv_wgrad(C1.data(), 96, dZ6.data(), 32, L1, gW(6));
    std::vector<R> dC1(L1.n() * 96);
    conv_bwd_data(dZ6.data(), 32, W(6), 96, L1, dC1.data());
    round_all(dC1.data(), L1.n() * 96);
    std::vector<R> dZ5(L2.n() * 64);
    upback_gate(dC1.data(), 96, 64, Y[5].data(), L1, dZ5.data());
    // L5
    conv_wgrad(Y[4].data(), 64, dZ5.data(), 64, L2, gW(5));
    std::vector<R> dZ4(L2.n() * 64);
    conv_bwd_data(dZ5.data(), 64, W(5), 64, L2, dZ4.data());
    gate_round(dZ4.data(), Y[4].data(), L2.n() * 64);
    // L4
    conv_wgrad(P1.data(), 32, dZ4.data(), 64, L2, gW(4));
    std::vector<R> dP1(L2.n() * 32);
    conv_bwd_data(dZ4.data(), 64, W(4), 32, L2, dP1.data());
    round_all(dP1.data(), L2.n() * 32);
    std::vector<R> dZ3(L1.n() * 32);
    poolback_gate(dC1.data(), 96, 64, dP1.data(), 32, Y[3].data(), L1, dZ3.data());
    // L3
    conv_wgrad(Y[2].data(), 32, dZ3.data(), 32, L1, gW(3));
    std::vector<R> dZ2(L1.n() * 32);
    conv_bwd_data(dZ3.data(), 32, W(3), 32, L1, dZ2.data());
    gate_round(dZ2.data(), Y[2].data(), L1.n() * 32);
    // L2
    conv_wgrad(P0.data(), 16, dZ2.data(), 32, L1, gW(2));
    std::vector<R> dP0(L1.n() * 16);
    conv_bwd_data(dZ2.data(), 32, W(2), 16, L1, dP0.data());
    round_all(dP0.data(), L1.n() * 16);
    std::vector<R> dZ1(V0 * 16);
    poolback_gate(dC0.data(), 48, 32, dP0.data(), 16, Y[1].data(), L0, dZ1.data());
    // L1
    conv_wgrad(Y[0].data(), 16, dZ1.data(), 16, L0, gW(1));
    std::vector<R> dZ0(V0 * 16);
    conv_bwd_data(dZ1.data(), 16, W(1), 16, L0, dZ0.data());
    gate_round(dZ0.data(), Y[0].data(), V0 * 16);
    // L0
    conv_wgrad(X0.data(), 16, dZ0.data(), 16, L0, gW(0));
    for (idx i = 0; i < num_params(); ++i) grad[i] = (R)g[i];
}

}  // namespace

UNO_EXPORT long pgo_unet_num_params() { return num_params(); }

UNO_EXPORT void pgo_unet_run_f32(const float* params, double out_scale, double dt, long d, long h, long w,
                                 const float* b, const uint8_t* nopen, const uint8_t* face_solid, int loss_kind,
                                 const float* p_true, float* p_out, float* grad, double* loss) {
    run<float>(params, out_scale, dt, d, h, w, b, nopen, face_solid, loss_kind, p_true, p_out, grad, loss);
}

UNO_EXPORT void pgo_unet_run_f64(const double* params, double out_scale, double dt, long d, long h, long w,
                                 const double* b, const uint8_t* nopen, const uint8_t* face_solid, int loss_kind,
                                 const double* p_true, double* p_out, double* grad, double* loss) {
    run<double>(params, out_scale, dt, d, h, w, b, nopen, face_solid, loss_kind, p_true, p_out, grad, loss);
}

UNO_EXPORT float pgo_bf16_round(float x) { return bf16_round(x); }
