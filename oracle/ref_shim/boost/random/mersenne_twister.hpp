// Stand-in: boost::random::mt19937 produces the same stream as std::mt19937.
#pragma once
#include <random>
namespace boost { namespace random { using mt19937 = std::mt19937; } }
