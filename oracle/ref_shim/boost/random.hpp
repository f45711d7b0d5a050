// Stand-in: the reference declares (but never draws from) a boost::mt19937.
#pragma once
#include <random>
namespace boost {
using mt19937 = std::mt19937;
}
