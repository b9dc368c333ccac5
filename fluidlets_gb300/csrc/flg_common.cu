// flg_common.cu -- library-wide entry points: version and error text.
#include <stdarg.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "flg_common.cuh"

namespace flg {

static thread_local char g_last_error[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

// ---- profiling (measurement aid) -------------------------------------------
struct ProfSlot {
    std::vector<cudaEvent_t> begin, end;
    int64_t launches = 0;
};
static std::atomic<int64_t> g_launches{0};
static std::atomic<bool> g_prof_on{false};
static std::mutex g_prof_mu;
static ProfSlot g_slots[FLG_NUM_SLOTS];

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// while a graph body is being captured on this thread, no timing events are recorded
// (event nodes are not allowed inside conditional graph bodies)
static thread_local int g_prof_suppressed = 0;
ProfSuppress::ProfSuppress() { g_prof_suppressed++; }
ProfSuppress::~ProfSuppress() { g_prof_suppressed--; }

static void prof_reset_locked() {
    for (auto &s : g_slots) {
        for (auto e : s.begin) cudaEventDestroy(e);
        for (auto e : s.end) cudaEventDestroy(e);
        s.begin.clear();
        s.end.clear();
        s.launches = 0;
    }
}

void prof_begin(int slot, cudaStream_t st) {
    if (!g_prof_on.load(std::memory_order_relaxed) || g_prof_suppressed) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecord(e, st);
    g_slots[slot].begin.push_back(e);
}

void prof_end(int slot, cudaStream_t st) {
    if (!g_prof_on.load(std::memory_order_relaxed) || g_prof_suppressed) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecord(e, st);
    g_slots[slot].end.push_back(e);
    g_slots[slot].launches++;
}

}  // namespace flg

extern "C" int flg_profile_enable(int enable) {
    std::lock_guard<std::mutex> lk(flg::g_prof_mu);
    flg::prof_reset_locked();
    flg::g_prof_on.store(enable != 0);
    return FLG_OK;
}

extern "C" int flg_profile_read(int slot, double *total_ms, int64_t *launches) {
    FLG_REQUIRE(slot >= 0 && slot < FLG_NUM_SLOTS, "profile slot %d out of range", slot);
    std::lock_guard<std::mutex> lk(flg::g_prof_mu);
    auto &s = flg::g_slots[slot];
    double tot = 0.0;
    size_t n = s.begin.size() < s.end.size() ? s.begin.size() : s.end.size();
    for (size_t k = 0; k < n; k++) {
        FLG_CUDA(cudaEventSynchronize(s.end[k]));
        float ms = 0.f;
        FLG_CUDA(cudaEventElapsedTime(&ms, s.begin[k], s.end[k]));
        tot += ms;
    }
    if (total_ms) *total_ms = tot;
    if (launches) *launches = s.launches;
    return FLG_OK;
}

extern "C" int64_t flg_launch_count(void) { return flg::g_launches.load(); }

extern "C" int flg_version(void) { return 10000; }  // 1.0.0

extern "C" const char *flg_last_error(void) { return flg::g_last_error; }
