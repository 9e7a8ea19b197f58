// Stand-in for the parallel-hashmap configuration header (an un-vendored MeshLib submodule), so that
// MeshLib's headers can be syntax-checked against the binding: nothing is configured.
#pragma once
