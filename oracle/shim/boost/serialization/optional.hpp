// Serialization of boost::optional: a no-op here (see pagmo/s11n.hpp stand-in).
#ifndef PGX_SHIM_BOOST_SERIALIZATION_OPTIONAL_HPP
#define PGX_SHIM_BOOST_SERIALIZATION_OPTIONAL_HPP
#include <boost/optional.hpp>
#endif
