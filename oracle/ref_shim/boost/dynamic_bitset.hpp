// Stand-in for boost::dynamic_bitset<> backed by std::vector<bool>.
#pragma once
#include <cstddef>
#include <vector>
namespace boost {
template <class Block = unsigned long> class dynamic_bitset : public std::vector<bool> {
public:
    explicit dynamic_bitset(std::size_t n) : std::vector<bool>(n, false) {}
};
}  // namespace boost
