// A working stand-in for the parallel-hashmap containers (an un-vendored MeshLib submodule), backed
// by the standard unordered containers, for compiling and running MeshLib's mesher from its own
// sources.  The mesher only looks keys up in its maps (MRMesh/MRSeparationPoint.h), so the
// container's iteration order never reaches its output.
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstddef>
#include <functional>
#include <unordered_map>
#include <unordered_set>

#include <parallel_hashmap/phmap_fwd_decl.h>

namespace phmap {
namespace priv {
// std::hash<T> is named only inside the call operator, so a specialization MeshLib declares after
// a container type is first mentioned (std::hash<MR::Id<T>>, MRMesh/MRId.h) is still the one used
template <class T>
struct hash_default_hash {
    std::size_t operator()(const T& v) const { return std::hash<T>{}(v); }
};
template <class T>
struct hash_default_eq {
    bool operator()(const T& a, const T& b) const { return a == b; }
};
}  // namespace priv

template <class T, class Hash, class Eq, class Alloc>
class flat_hash_set : public std::unordered_set<T, Hash, Eq> {
public:
    using std::unordered_set<T, Hash, Eq>::unordered_set;
};
template <class T, class Hash, class Eq, class Alloc>
class parallel_flat_hash_set : public std::unordered_set<T, Hash, Eq> {
public:
    using std::unordered_set<T, Hash, Eq>::unordered_set;
};
template <class K, class V, class Hash, class Eq, class Alloc>
class flat_hash_map : public std::unordered_map<K, V, Hash, Eq> {
public:
    using std::unordered_map<K, V, Hash, Eq>::unordered_map;
};
// one sub-map: every key hashes to sub-map 0
template <class K, class V, class Hash, class Eq, class Alloc>
class parallel_flat_hash_map : public std::unordered_map<K, V, Hash, Eq> {
public:
    using std::unordered_map<K, V, Hash, Eq>::unordered_map;
    static constexpr std::size_t subcnt() { return 1; }
    std::size_t hash(const K& k) const { return Hash{}(k); }
    static constexpr std::size_t subidx(std::size_t) { return 0; }
};
}  // namespace phmap
