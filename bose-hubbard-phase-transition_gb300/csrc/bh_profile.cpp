// bh_profile.cpp -- optional per-kernel device timing (the library's tracing).
//
// When enabled (bh_profile_enable(1)), every kernel launch of the solver is
// bracketed by a pair of CUDA events recorded on the stream it is launched on,
// and tagged with the launch's algorithmic byte count (bytes the kernel must
// move at minimum: every operand read once, every result written once).
// Pending pairs are resolved after each library call has synchronised its
// stream; totals per kernel name are kept until bh_profile_reset().
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "bh_internal.h"

namespace bh {

namespace {
struct Pending {
    std::string name;
    double bytes;
    cudaEvent_t a, b;
};
struct Total {
    int64_t launches = 0;
    double ms = 0.0;
    double bytes = 0.0;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Pending> g_pending;
std::map<std::string, Total> g_tot;
thread_local cudaEvent_t t_open = nullptr;
}  // namespace

bool profile_on() { return g_on; }

void profile_begin(cudaStream_t st) {
    if (!g_on) return;
    cudaEvent_t a;
    if (cudaEventCreate(&a) != cudaSuccess) return;
    cudaEventRecord(a, st);
    t_open = a;
}

void profile_end(cudaStream_t st, const char* name, double bytes) {
    if (!g_on || !t_open) return;
    cudaEvent_t b;
    if (cudaEventCreate(&b) != cudaSuccess) return;
    cudaEventRecord(b, st);
    std::lock_guard<std::mutex> lk(g_mu);
    g_pending.push_back({name, bytes, t_open, b});
    t_open = nullptr;
}

void profile_flush() {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& p : g_pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            Total& t = g_tot[p.name];
            t.launches += 1;
            t.ms += ms;
            t.bytes += p.bytes;
        }
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    g_pending.clear();
}

}  // namespace bh

extern "C" {

int bh_profile_enable(int on) {
    bh::profile_flush();
    bh::g_on = on != 0;
    return BH_OK;
}

int bh_profile_reset(void) {
    bh::profile_flush();
    std::lock_guard<std::mutex> lk(bh::g_mu);
    bh::g_tot.clear();
    return BH_OK;
}

int bh_profile_count(int* n) {
    if (!n) return BH_ERR_ARG;
    bh::profile_flush();
    std::lock_guard<std::mutex> lk(bh::g_mu);
    *n = (int)bh::g_tot.size();
    return BH_OK;
}

int bh_profile_get(int i, char* name, int name_cap, int64_t* launches, double* ms, double* bytes) {
    std::lock_guard<std::mutex> lk(bh::g_mu);
    if (i < 0 || i >= (int)bh::g_tot.size()) return BH_ERR_ARG;
    auto it = bh::g_tot.begin();
    std::advance(it, i);
    if (name && name_cap > 0) {
        std::strncpy(name, it->first.c_str(), (size_t)name_cap - 1);
        name[name_cap - 1] = '\0';
    }
    if (launches) *launches = it->second.launches;
    if (ms) *ms = it->second.ms;
    if (bytes) *bytes = it->second.bytes;
    return BH_OK;
}

}  // extern "C"
