// Minimal checked numeric_cast stand-in (throws on out-of-range like Boost's).
#ifndef PGX_SHIM_NUMERIC_CAST_HPP
#define PGX_SHIM_NUMERIC_CAST_HPP
#include <limits>
#include <stdexcept>
#include <type_traits>
namespace boost
{
template <typename To, typename From>
inline To numeric_cast(From v)
{
    static_assert(std::is_integral<To>::value && std::is_integral<From>::value, "integral casts only");
    if ((std::is_signed<From>::value && v < From(0) && !std::is_signed<To>::value)
        || static_cast<unsigned long long>(v) > static_cast<unsigned long long>(std::numeric_limits<To>::max())) {
        throw std::overflow_error("numeric_cast: value out of range");
    }
    return static_cast<To>(v);
}
} // namespace boost
#endif
