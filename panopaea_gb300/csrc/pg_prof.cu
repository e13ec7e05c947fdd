// pg_prof.cu -- launch counting and per-kernel CUDA-event timing.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <deque>
#include <mutex>
#include <vector>

#include "pg_internal.cuh"

namespace pg {

static const char* kKindNames[KK_COUNT] = {
    "cg_init", "cg_spmv", "cg_update", "cg_tail", "advect", "advect_mac", "rhs", "project", "dec_op",
    "residual64", "refine_update", "mg_smooth", "mg_restrict", "mg_smooth_coarse", "mg_restrict_coarse",
    "mg_coarse", "mg_setup", "step_misc", "unet_conv", "unet_wgrad", "unet_misc", "mg_pair",
};

namespace {
std::atomic<int64_t> g_launches{0};
thread_local bool t_capturing = false;
thread_local int64_t t_captured = 0;

struct Pending {
    cudaEvent_t a, b;
    int kind;
};

struct Prof {
    std::mutex m;
    bool on = false;
    std::vector<cudaEvent_t> pool;
    std::deque<Pending> pending;
    cudaEvent_t open[KK_COUNT] = {};
    double ms[KK_COUNT] = {};
    int64_t n[KK_COUNT] = {};
    std::vector<float> each[KK_COUNT];  // every launch's duration
};

Prof& prof() {
    static Prof p;
    return p;
}

cudaEvent_t take(Prof& p) {
    if (!p.pool.empty()) {
        cudaEvent_t e = p.pool.back();
        p.pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Fold finished pairs into the totals; `wait` = block on unfinished ones.
void drain(Prof& p, bool wait) {
    while (!p.pending.empty()) {
        Pending& q = p.pending.front();
        if (wait) {
            cudaEventSynchronize(q.b);
        } else if (cudaEventQuery(q.b) != cudaSuccess) {
            break;
        }
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, q.a, q.b) == cudaSuccess) {
            p.ms[q.kind] += ms;
            p.n[q.kind] += 1;
            p.each[q.kind].push_back(ms);
        }
        p.pool.push_back(q.a);
        p.pool.push_back(q.b);
        p.pending.pop_front();
    }
}
}  // namespace

void prof_begin(cudaStream_t s, int kind) {
    if (t_capturing) {
        ++t_captured;
        return;
    }
    g_launches.fetch_add(1, std::memory_order_relaxed);
    Prof& p = prof();
    if (!p.on) return;
    std::lock_guard<std::mutex> lk(p.m);
    cudaEvent_t e = take(p);
    cudaEventRecord(e, s);
    p.open[kind] = e;
}

void prof_end(cudaStream_t s, int kind) {
    Prof& p = prof();
    if (!p.on || t_capturing) return;
    std::lock_guard<std::mutex> lk(p.m);
    if (!p.open[kind]) return;
    cudaEvent_t e = take(p);
    cudaEventRecord(e, s);
    p.pending.push_back(Pending{p.open[kind], e, kind});
    p.open[kind] = nullptr;
    if (p.pending.size() > 8192) drain(p, false);
}

int64_t prof_capture_begin() {
    t_capturing = true;
    return t_captured;
}

int64_t prof_capture_end() {
    t_capturing = false;
    return t_captured;
}

void prof_add_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

bool graphs_enabled() {
    static const bool env_off = [] {
        const char* v = getenv("PG_NO_GRAPHS");
        return v && v[0] && v[0] != '0';
    }();
    return !env_off && !prof().on;
}

}  // namespace pg

using namespace pg;

extern "C" {

int64_t pg_kernel_launches(void) { return g_launches.load(); }

int pg_profile_enable(int on) {
    Prof& p = prof();
    std::lock_guard<std::mutex> lk(p.m);
    p.on = on != 0;
    return PG_OK;
}

int pg_profile_reset(void) {
    Prof& p = prof();
    std::lock_guard<std::mutex> lk(p.m);
    drain(p, true);
    for (int k = 0; k < KK_COUNT; ++k) {
        p.ms[k] = 0.0;
        p.n[k] = 0;
        p.each[k].clear();
    }
    return PG_OK;
}

int pg_profile_num_kinds(void) { return KK_COUNT; }

const char* pg_profile_kind_name(int kind) {
    if (kind < 0 || kind >= KK_COUNT) return "";
    return kKindNames[kind];
}

int pg_profile_read(int kind, double* total_ms, int64_t* launches) {
    if (kind < 0 || kind >= KK_COUNT) return bad_arg("pg_profile_read: unknown kind");
    Prof& p = prof();
    std::lock_guard<std::mutex> lk(p.m);
    drain(p, true);
    if (total_ms) *total_ms = p.ms[kind];
    if (launches) *launches = p.n[kind];
    return PG_OK;
}

int pg_profile_read_active(int kind, double* total_ms, int64_t* launches) {
    if (kind < 0 || kind >= KK_COUNT) return bad_arg("pg_profile_read_active: unknown kind");
    Prof& p = prof();
    std::lock_guard<std::mutex> lk(p.m);
    drain(p, true);
    // Exit-at-entry launches take a few microseconds, launches that did work
    // are longer: split the two clusters at the smaller of a quarter of the
    // longest launch and the geometric mean of the shortest and the longest.
    float mx = 0.f, mn = 1e30f;
    for (float v : p.each[kind]) {
        mx = std::max(mx, v);
        mn = std::min(mn, v);
    }
    const float cut = std::min(0.25f * mx, std::sqrt(mn * mx));
    double t = 0.0;
    int64_t n = 0;
    for (float v : p.each[kind])
        if (v >= cut) {
            t += v;
            ++n;
        }
    if (total_ms) *total_ms = t;
    if (launches) *launches = n;
    return PG_OK;
}

}  // extern "C"
