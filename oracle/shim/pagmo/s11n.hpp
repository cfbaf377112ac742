// Stand-in for pagmo/s11n.hpp: Boost.Serialization is not installed, and
// checkpointing is not on the batch-evaluation path, so every serialization
// hook the hot-path sources mention becomes a no-op.
#ifndef PAGMO_S11N_HPP
#define PAGMO_S11N_HPP
#include <cstddef>
#include <locale>
#include <random>
#include <sstream>
#include <string>
#include <tuple>
#include <utility>

namespace boost
{
namespace serialization
{
class access
{
};
enum tracking_type { track_never = 0, track_selectively = 1, track_always = 2 };
template <typename Base, typename Derived>
inline Base &base_object(Derived &d)
{
    return d;
}
template <typename Base, typename Derived>
inline const Base &base_object(const Derived &d)
{
    return d;
}
} // namespace serialization
} // namespace boost

#define BOOST_CLASS_EXPORT_KEY2(T, K)
#define BOOST_CLASS_EXPORT_KEY(T)
#define BOOST_CLASS_EXPORT_IMPLEMENT(T)
#define BOOST_CLASS_TRACKING(T, E)
#define BOOST_CLASS_VERSION(T, N)
#define BOOST_SERIALIZATION_SPLIT_MEMBER()

namespace pagmo
{
namespace detail
{
template <typename Archive, typename... Args>
inline void archive(Archive &, Args &&...)
{
}
template <typename Archive, typename... Args>
inline void to_archive(Archive &, Args &&...)
{
}
template <typename Archive, typename... Args>
inline void from_archive(Archive &, Args &&...)
{
}
} // namespace detail
} // namespace pagmo
#endif
