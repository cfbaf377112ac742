// Stand-in for the CMake-generated pagmo/config.hpp, used only to compile the
// reference's own hot-path sources (problem, bfe, batch evaluators, the three
// UDPs, multi-objective utilities) into the test oracle library.
#ifndef PAGMO_CONFIG_HPP
#define PAGMO_CONFIG_HPP
#include <vector>
#define PAGMO_VERSION "2.19.1"
#define PAGMO_VERSION_MAJOR 2
#define PAGMO_VERSION_MINOR 19
#define PAGMO_VERSION_PATCH 1
#endif
