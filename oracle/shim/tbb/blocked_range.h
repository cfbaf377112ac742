// tbb::blocked_range stand-in: a half-open index range.
#ifndef PGX_SHIM_TBB_BLOCKED_RANGE_H
#define PGX_SHIM_TBB_BLOCKED_RANGE_H
namespace tbb
{
template <typename T>
class blocked_range
{
public:
    blocked_range(T b, T e) : m_b(b), m_e(e) {}
    T begin() const { return m_b; }
    T end() const { return m_e; }
    bool empty() const { return !(m_b < m_e); }

private:
    T m_b, m_e;
};
} // namespace tbb
#endif
