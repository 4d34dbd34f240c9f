// TBB-compatible shim (test infrastructure): parallel_for over 1D and 2D ranges.
#ifndef FG_TBB_SHIM_PARALLEL_FOR_H
#define FG_TBB_SHIM_PARALLEL_FOR_H
#include "blocked_range.h"
#include "blocked_range2d.h"
#include "shim_pool.h"
namespace tbb {
template<typename T, typename Body> void parallel_for(const blocked_range<T>& r, const Body& body)
{
    shim::split_run(static_cast<std::size_t>(r.begin()), static_cast<std::size_t>(r.end()),
                    [&body](std::size_t b, std::size_t e) { body(blocked_range<T>(T(b), T(e))); });
}
template<typename T, typename Body> void parallel_for(const blocked_range2d<T>& r, const Body& body)
{
    const T cb = r.cols().begin();
    const T ce = r.cols().end();
    shim::split_run(static_cast<std::size_t>(r.rows().begin()), static_cast<std::size_t>(r.rows().end()),
                    [&body, cb, ce](std::size_t b, std::size_t e) { body(blocked_range2d<T>(T(b), T(e), cb, ce)); });
}
}; // namespace tbb
#endif
