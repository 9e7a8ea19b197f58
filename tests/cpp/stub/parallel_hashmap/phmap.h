// Stand-in for the parallel-hashmap header (an un-vendored MeshLib submodule): only the names MeshLib's
// headers mention, declared, for a syntax check of the MeshLib-side binding.  Nothing is instantiated.
#pragma once
#include <parallel_hashmap/phmap_fwd_decl.h>
