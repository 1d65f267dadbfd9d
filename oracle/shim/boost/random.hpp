// Stand-in for the two boost::random names the reference CPU_HopHL test code
// uses (CPU_HopHL/include/HBPLL/test.h:56-58,63-66 and
// graph_v_of_v/graph_v_of_v_generate_random_graph.h:14,47,57).
// TEST INFRASTRUCTURE ONLY: it lets the reference headers compile unmodified
// without Boost.  Nothing in this project draws random numbers through it.
#pragma once
#include <random>

namespace boost {
namespace random {
using mt19937 = std::mt19937;
template <class I = int>
using uniform_int_distribution = std::uniform_int_distribution<I>;
}  // namespace random
}  // namespace boost
