// Stand-in for boost::unordered_map: std::unordered_map hashed through the
// boost::hash_value overload the reference provides for its key type.
#pragma once
#include <cstddef>
#include <unordered_map>
namespace boost {
template <class K> struct shim_hash {
    std::size_t operator()(const K &k) const { return hash_value(k); }
};
template <class K, class V> using unordered_map = std::unordered_map<K, V, shim_hash<K>>;
}  // namespace boost
