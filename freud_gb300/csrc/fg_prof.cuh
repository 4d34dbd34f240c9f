// Kernel launch accounting: every launch wrapper opens a ProfScope, which counts
// the launch and, while profiling is enabled, brackets it with CUDA events on the
// launch stream so per-kernel device time can be read back (fg_profile_* in the C ABI).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fg {

void prof_count_launch();
bool prof_enabled();
// Stream capture: launches made while capturing are counted for the graph, not
// run; each replay adds the graph's count (prof_add_launches).
void prof_begin_capture();
uint64_t prof_end_capture();
bool prof_capturing();
void prof_add_launches(uint64_t n);
void prof_record(const char* name, cudaEvent_t start, cudaEvent_t stop);
cudaEvent_t prof_event();

struct ProfScope
{
    const char* name;
    cudaStream_t stream;
    cudaEvent_t start = nullptr;
    ProfScope(const char* n, cudaStream_t s, bool count = true) : name(n), stream(s)
    {
        if (count)
            prof_count_launch();
        if (prof_enabled() && !prof_capturing())
        {
            start = prof_event();
            cudaEventRecord(start, stream);
        }
    }
    ~ProfScope()
    {
        if (start != nullptr)
        {
            cudaEvent_t stop = prof_event();
            cudaEventRecord(stop, stream);
            prof_record(name, start, stop);
        }
    }
};

} // namespace fg
