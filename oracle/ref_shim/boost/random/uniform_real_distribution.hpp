// Stand-in: boost::random::uniform_real_distribution mapped to the std one.
// (Only affects random-fill loaders, which no fixture here uses.)
#pragma once
#include <random>
namespace boost { namespace random { template <class T> using uniform_real_distribution = std::uniform_real_distribution<T>; } }
