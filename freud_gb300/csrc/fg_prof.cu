// Launch counting and per-kernel event timing behind fg_profile_* (include/freud_gb300.h).
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/freud_gb300.h"
#include "fg_prof.cuh"

namespace fg {
namespace {
std::atomic<uint64_t> g_launches {0};
std::atomic<bool> g_enabled {false};
std::mutex g_mu;
struct Pending
{
    std::string name;
    cudaEvent_t a, b;
};
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_free;
struct Stat
{
    uint64_t count = 0;
    double ms = 0.0;
};
std::map<std::string, Stat> g_stats;
thread_local bool g_capturing = false;
thread_local uint64_t g_captured = 0;

void drain_locked()
{
    for (auto& p : g_pending)
    {
        cudaEventSynchronize(p.b);
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess)
        {
            Stat& s = g_stats[p.name];
            s.count += 1;
            s.ms += ms;
        }
        g_free.push_back(p.a);
        g_free.push_back(p.b);
    }
    g_pending.clear();
}
} // namespace

void prof_count_launch()
{
    if (g_capturing)
        ++g_captured;
    else
        g_launches.fetch_add(1, std::memory_order_relaxed);
}

void prof_begin_capture()
{
    g_capturing = true;
    g_captured = 0;
}

uint64_t prof_end_capture()
{
    g_capturing = false;
    return g_captured;
}

bool prof_capturing()
{
    return g_capturing;
}

void prof_add_launches(uint64_t n)
{
    g_launches.fetch_add(n, std::memory_order_relaxed);
}

bool prof_enabled()
{
    return g_enabled.load(std::memory_order_relaxed);
}

cudaEvent_t prof_event()
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_free.empty())
    {
        cudaEvent_t e = g_free.back();
        g_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void prof_record(const char* name, cudaEvent_t start, cudaEvent_t stop)
{
    std::lock_guard<std::mutex> lock(g_mu);
    g_pending.push_back({name, start, stop});
    if (g_pending.size() > 4096)
    {
        drain_locked();
    }
}

} // namespace fg

extern "C" {

fg_status fg_launch_count(uint64_t* out)
{
    if (out == nullptr)
    {
        return FG_ERR_VALUE;
    }
    *out = fg::g_launches.load();
    return FG_OK;
}

fg_status fg_profile_enable(int enable)
{
    std::lock_guard<std::mutex> lock(fg::g_mu);
    fg::drain_locked();
    fg::g_stats.clear();
    fg::g_enabled.store(enable != 0);
    return FG_OK;
}

fg_status fg_profile_report(char* buf, size_t len)
{
    std::lock_guard<std::mutex> lock(fg::g_mu);
    fg::drain_locked();
    std::string out;
    for (auto& kv : fg::g_stats)
    {
        char line[256];
        std::snprintf(line, sizeof(line), "%s %llu %.6f\n", kv.first.c_str(),
                      static_cast<unsigned long long>(kv.second.count), kv.second.ms);
        out += line;
    }
    if (buf != nullptr && len > 0)
    {
        std::strncpy(buf, out.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return out.size() + 1 > len ? FG_ERR_VALUE : FG_OK;
}

} // extern "C"
