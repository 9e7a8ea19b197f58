// Forward declarations of the parallel-hashmap names that MRMesh/MRMeshFwd.h mentions, so the
// reference's CUDA translation unit MRCuda/MRCudaFastWindingNumber.cu compiles without the
// (un-vendored) parallel-hashmap submodule.  Nothing here is instantiated by that unit.
#pragma once
namespace phmap {
namespace priv {
template <class T> struct hash_default_hash;
template <class T> struct hash_default_eq;
}  // namespace priv
template <class T, class Hash, class Eq, class Alloc = void> class flat_hash_set;
template <class T, class Hash, class Eq, class Alloc = void> class parallel_flat_hash_set;
template <class K, class V, class Hash, class Eq, class Alloc = void> class flat_hash_map;
template <class K, class V, class Hash, class Eq, class Alloc = void> class parallel_flat_hash_map;
}  // namespace phmap
