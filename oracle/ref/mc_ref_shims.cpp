// Definitions standing in for the MeshLib functions that the mesher translation unit references
// but that the golden-vector driver (oracle/ref/mc_ref_driver.cpp) never reaches: the scoped
// timer becomes a no-op, and the OpenVDB grid, the half-edge mesh builder and the point-tree
// accessors (used only by the VDB-volume and Mesh-returning entry points) abort if called.
// TEST INFRASTRUCTURE ONLY.
#include <cstdlib>

#include "MRMesh/MRAABBTreePoints.h"
#include "MRMesh/MRMesh.h"
#include "MRMesh/MRTimer.h"
#include "MRVoxels/MRFloatGrid.h"

namespace MR {

void Timer::start(const char*) {}
void Timer::finish() {}

size_t AABBTreePoints::heapBytes() const { std::abort(); }

FloatGrid::operator bool() const noexcept { std::abort(); }
OpenVdbFloatGrid* FloatGrid::operator->() const noexcept { std::abort(); }

Mesh Mesh::fromTriMesh(TriMesh&&, const MeshBuilder::BuildSettings&, ProgressCallback) { std::abort(); }

}  // namespace MR
