// Launch counter and per-launch event timing (see trace.h).
#include "trace.h"
#include "fpm_common.cuh"

#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace fpm_trace {
namespace {
std::atomic<long long> g_launches(0);
std::atomic<bool> g_on(false);
std::mutex g_mu;
struct Rec {
    const char* name;
    cudaEvent_t a, b;
};
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t get_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

Scope::Scope(const char* n, cudaStream_t s) : name(n), st(s), slot(-1) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (!g_on.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lock(g_mu);
    Rec r;
    r.name = n;
    r.a = get_event();
    r.b = get_event();
    cudaEventRecord(r.a, s);
    g_recs.push_back(r);
    slot = (int)g_recs.size() - 1;
}

void add_launches(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

Scope::~Scope() {
    if (slot < 0) return;
    std::lock_guard<std::mutex> lock(g_mu);
    if (slot < (int)g_recs.size()) cudaEventRecord(g_recs[slot].b, st);
}
}  // namespace fpm_trace

extern "C" {

long long fpm_launch_count(void) { return fpm_trace::g_launches.load(); }

int fpm_trace_enable(int on) {
    fpm_trace::g_on.store(on != 0);
    return FPM_OK;
}

int fpm_trace_summary(char* buf, long long len) {
    using namespace fpm_trace;
    if (!buf || len <= 0) return FPM_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_mu);
    std::map<std::string, std::pair<long long, double>> tot;
    std::vector<std::string> order;
    int rc = FPM_OK;
    for (auto& r : g_recs) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess)
            rc = FPM_ERR_CUDA;
        auto it = tot.find(r.name);
        if (it == tot.end()) {
            order.push_back(r.name);
            tot[r.name] = std::make_pair(1LL, (double)ms);
        } else {
            it->second.first += 1;
            it->second.second += ms;
        }
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
    }
    g_recs.clear();
    std::string out;
    char line[256];
    for (auto& name : order) {
        snprintf(line, sizeof(line), "%s %lld %.6f\n", name.c_str(), tot[name].first, tot[name].second);
        out += line;
    }
    if ((long long)out.size() + 1 > len) return FPM_ERR_LIMIT;
    memcpy(buf, out.c_str(), out.size() + 1);
    return rc;
}

}  // extern "C"
