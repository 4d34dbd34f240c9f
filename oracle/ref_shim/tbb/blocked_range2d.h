// TBB-compatible shim (test infrastructure): blocked_range2d.
#ifndef FG_TBB_SHIM_BLOCKED_RANGE2D_H
#define FG_TBB_SHIM_BLOCKED_RANGE2D_H
#include "blocked_range.h"
namespace tbb {
template<typename T> class blocked_range2d
{
public:
    blocked_range2d(T rb, T re, T cb, T ce) : m_rows(rb, re), m_cols(cb, ce) {}
    blocked_range2d(const blocked_range<T>& r, const blocked_range<T>& c) : m_rows(r), m_cols(c) {}
    const blocked_range<T>& rows() const { return m_rows; }
    const blocked_range<T>& cols() const { return m_cols; }
private:
    blocked_range<T> m_rows;
    blocked_range<T> m_cols;
};
}; // namespace tbb
#endif
