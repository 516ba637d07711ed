// Per-kernel timing with CUDA events on the launching stream, and a launch counter.
//
// Off by default.  When enabled (evx_prof_enable(1)) every kernel launch and
// cuFFT execution inside the library is bracketed by a pair of events recorded
// on the stream it runs on; evx_prof_collect() waits for them and accumulates
// the elapsed time per named slot.  The launch counter counts this library's
// own kernel launches (not cuFFT's) and is always on.
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "evx_prof.cuh"

namespace evx {

namespace {

struct Slot {
    std::string name;
    double ms = 0.0;
    long long count = 0;
};

struct Pending {
    int slot;
    cudaEvent_t a, b;
};

std::mutex g_mu;
bool g_on = false;
std::vector<Slot> g_slots;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_pool;
std::atomic<unsigned long long> g_launches{0};

cudaEvent_t take_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

int slot_of(const char* name) {
    for (size_t i = 0; i < g_slots.size(); ++i)
        if (g_slots[i].name == name) return (int)i;
    g_slots.push_back(Slot{name});
    return (int)g_slots.size() - 1;
}

}  // namespace

ProfTok prof_begin(const char* name, cudaStream_t st) {
    ProfTok t{-1, nullptr};
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_on) return t;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return t;
    t.slot = slot_of(name);
    t.ev = take_event();
    cudaEventRecord(t.ev, st);
    return t;
}

void prof_end(const ProfTok& t, cudaStream_t st) {
    if (t.slot < 0) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEvent_t b = take_event();
    cudaEventRecord(b, st);
    g_pending.push_back(Pending{t.slot, t.ev, b});
}

void count_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

unsigned long long launch_counter() { return g_launches.load(std::memory_order_relaxed); }

void uncount_launch(unsigned long long n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }

namespace {
// -1: not yet read from the environment (EVX_GRAPHS=0 turns graph replay off)
std::atomic<int> g_graphs{-1};
std::atomic<unsigned long long> g_config_epoch{0};
}  // namespace

unsigned long long config_epoch() { return g_config_epoch.load(std::memory_order_relaxed); }
void bump_config_epoch() { g_config_epoch.fetch_add(1, std::memory_order_relaxed); }

bool graphs_enabled() {
    int v = g_graphs.load(std::memory_order_relaxed);
    if (v < 0) {
        const char* e = std::getenv("EVX_GRAPHS");
        v = (e && std::strcmp(e, "0") == 0) ? 0 : 1;
        int expect = -1;
        g_graphs.compare_exchange_strong(expect, v);
        v = g_graphs.load(std::memory_order_relaxed);
    }
    if (!v) return false;
    std::lock_guard<std::mutex> lk(g_mu);
    return !g_on;
}

}  // namespace evx

using namespace evx;

extern "C" {

void evx_prof_enable(int on) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_on = on != 0;
}

int evx_prof_collect(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& p : g_pending) {
        if (cudaEventSynchronize(p.b) != cudaSuccess)
            return fail(EVX_ERR_CUDA, "evx_prof_collect: %s", cudaGetErrorString(cudaGetLastError()));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        g_slots[p.slot].ms += ms;
        g_slots[p.slot].count += 1;
        g_pool.push_back(p.a);
        g_pool.push_back(p.b);
    }
    g_pending.clear();
    return EVX_OK;
}

void evx_prof_reset(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& s : g_slots) { s.ms = 0.0; s.count = 0; }
}

int evx_prof_query(int index, char* name, int name_cap, double* total_ms, long long* count) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (index < 0 || index >= (int)g_slots.size()) return -1;
    if (name && name_cap > 0) {
        strncpy(name, g_slots[index].name.c_str(), (size_t)name_cap - 1);
        name[name_cap - 1] = 0;
    }
    if (total_ms) *total_ms = g_slots[index].ms;
    if (count) *count = g_slots[index].count;
    return EVX_OK;
}

unsigned long long evx_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

void evx_set_graphs(int on) { g_graphs.store(on ? 1 : 0, std::memory_order_relaxed); }

int evx_graphs_enabled(void) { return graphs_enabled() ? 1 : 0; }

}  // extern "C"
