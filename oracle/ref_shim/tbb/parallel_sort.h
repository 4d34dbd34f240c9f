// TBB-compatible shim (test infrastructure): parallel_sort runs std::sort.
#ifndef FG_TBB_SHIM_PARALLEL_SORT_H
#define FG_TBB_SHIM_PARALLEL_SORT_H
#include <algorithm>
namespace tbb {
template<typename It, typename Cmp> void parallel_sort(It begin, It end, const Cmp& cmp)
{
    std::sort(begin, end, cmp);
}
template<typename It> void parallel_sort(It begin, It end)
{
    std::sort(begin, end);
}
}; // namespace tbb
#endif
