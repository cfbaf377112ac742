// hash_combine stand-in (only used by pagmo's vector hashing helpers).
#ifndef PGX_SHIM_HASH_HPP
#define PGX_SHIM_HASH_HPP
#include <cstddef>
#include <functional>
namespace boost
{
template <typename T>
inline void hash_combine(std::size_t &seed, const T &v)
{
    seed ^= std::hash<T>{}(v) + 0x9e3779b97f4a7c15ull + (seed << 6) + (seed >> 2);
}
} // namespace boost
#endif
