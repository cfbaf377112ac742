// Stand-in for Boost.SafeNumerics' safe<T> (Boost is not installed here): an
// integer whose multiplication throws on overflow instead of wrapping, which
// is how the reference's sources use it to size their buffers.
#ifndef PGX_SHIM_BOOST_SAFE_INTEGER_HPP
#define PGX_SHIM_BOOST_SAFE_INTEGER_HPP

#include <limits>
#include <stdexcept>

namespace boost
{
namespace safe_numerics
{

template <typename T>
class safe
{
public:
    safe(T v) : m_v(v) {}
    template <typename U>
    safe operator*(U other) const
    {
        const T b = static_cast<T>(other);
        if (b != 0 && m_v > std::numeric_limits<T>::max() / b) throw std::overflow_error("safe integer overflow");
        return safe(m_v * b);
    }
    operator T() const
    {
        return m_v;
    }

private:
    T m_v;
};

} // namespace safe_numerics
} // namespace boost

#endif
