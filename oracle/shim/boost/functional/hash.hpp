/* Stand-in for boost::hash, which the reference tree uses only to key
 * perturbed point sets (an incremental-update feature). Test infrastructure. */
#ifndef KI_ORACLE_SHIM_BOOST_HASH_HPP_
#define KI_ORACLE_SHIM_BOOST_HASH_HPP_
#include <cstddef>
#include <functional>
#include <vector>
namespace boost {
template <class T> struct hash {
  std::size_t operator()(const T& v) const { return std::hash<T>()(v); }
};
template <> struct hash<std::vector<double>> {
  std::size_t operator()(const std::vector<double>& v) const {
    std::size_t h = 1469598103934665603ull;
    for (double d : v) h = (h ^ std::hash<double>()(d)) * 1099511628211ull;
    return h;
  }
};
}  // namespace boost
#endif
