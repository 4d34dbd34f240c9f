// TBB-compatible shim (test infrastructure): blocked_range.
#ifndef FG_TBB_SHIM_BLOCKED_RANGE_H
#define FG_TBB_SHIM_BLOCKED_RANGE_H
#include <cstddef>
namespace tbb {
template<typename T> class blocked_range
{
public:
    blocked_range(T b, T e, std::size_t grain = 1) : m_begin(b), m_end(e), m_grain(grain) {}
    T begin() const { return m_begin; }
    T end() const { return m_end; }
    std::size_t size() const { return static_cast<std::size_t>(m_end - m_begin); }
    bool empty() const { return !(m_begin < m_end); }
    std::size_t grainsize() const { return m_grain; }
private:
    T m_begin;
    T m_end;
    std::size_t m_grain;
};
}; // namespace tbb
#endif
