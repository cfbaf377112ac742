// boost::math::constants::pi stand-in (gaco.cpp, maco.cpp): pi rounded to T.
#ifndef PGX_SHIM_BOOST_MATH_CONSTANTS_HPP
#define PGX_SHIM_BOOST_MATH_CONSTANTS_HPP
namespace boost
{
namespace math
{
namespace constants
{
template <typename T>
constexpr T pi()
{
    return static_cast<T>(3.14159265358979323846264338327950288L);
}
} // namespace constants
} // namespace math
} // namespace boost
#endif
