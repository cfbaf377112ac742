// boost::optional stand-in for the algorithms' optional bfe member
// (e.g. include/pagmo/algorithms/nsga2.hpp:186): std::optional offers the
// same operations they use (assignment, contextual bool, operator*).
#ifndef PGX_SHIM_BOOST_OPTIONAL_HPP
#define PGX_SHIM_BOOST_OPTIONAL_HPP
#include <optional>
namespace boost
{
template <typename T>
using optional = std::optional<T>;
inline constexpr std::nullopt_t none = std::nullopt;
} // namespace boost
#endif
