// Minimal checked numeric_cast stand-in: throws when the value does not fit
// the target type, like Boost's (integral -> integral, floating -> integral
// after truncation toward zero; conversions to a floating type are plain
// casts, which cannot overflow for the integer and double sources pagmo
// converts).
#ifndef PGX_SHIM_NUMERIC_CAST_HPP
#define PGX_SHIM_NUMERIC_CAST_HPP
#include <cmath>
#include <limits>
#include <stdexcept>
#include <type_traits>
namespace boost
{
template <typename To, typename From>
inline To numeric_cast(From v)
{
    static_assert(std::is_arithmetic<To>::value && std::is_arithmetic<From>::value, "arithmetic casts only");
    if constexpr (std::is_floating_point<To>::value) {
        return static_cast<To>(v);
    } else if constexpr (std::is_floating_point<From>::value) {
        // To is integral: NaN and values outside (min - 1, max + 1) do not fit
        const long double t = std::trunc(static_cast<long double>(v));
        if (!(t >= static_cast<long double>(std::numeric_limits<To>::min())
              && t <= static_cast<long double>(std::numeric_limits<To>::max()))) {
            throw std::overflow_error("numeric_cast: value out of range");
        }
        return static_cast<To>(t);
    } else {
        if ((std::is_signed<From>::value && v < From(0) && !std::is_signed<To>::value)
            || (std::is_signed<From>::value && std::is_signed<To>::value
                && static_cast<long long>(v) < static_cast<long long>(std::numeric_limits<To>::min()))
            || (!(std::is_signed<From>::value && v < From(0))
                && static_cast<unsigned long long>(v)
                       > static_cast<unsigned long long>(std::numeric_limits<To>::max()))) {
            throw std::overflow_error("numeric_cast: value out of range");
        }
        return static_cast<To>(v);
    }
}
} // namespace boost
#endif
