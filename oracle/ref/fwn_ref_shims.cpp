// Definitions standing in for the MeshLib functions that the winding-number library's units
// (Mesh, MeshBuilder) reference but that the golden-vector driver (oracle/ref/fwn_ref_driver.cpp)
// never reaches: the scoped timer becomes a no-op; hole filling, close-vertex search and stream
// sizing (whose units need Eigen, boost or spdlog, absent here) abort if called.
// TEST INFRASTRUCTURE ONLY.
#include <cstdlib>
#include <istream>

#include "MRMesh/MRCloseVertices.h"
#include "MRMesh/MRIOParsing.h"
#include "MRMesh/MRMesh.h"
#include "MRMesh/MRMeshFillHole.h"
#include "MRMesh/MRTimer.h"

namespace MR {

void Timer::start(const char*) {}
void Timer::restart(std::string) {}
void Timer::finish() {}

std::vector<HoleFillPlan> getPlanarHoleFillPlans(const Mesh&, const std::vector<EdgeId>&) { std::abort(); }
void executeHoleFillPlan(Mesh&, EdgeId, HoleFillPlan&, FaceBitSet*) { std::abort(); }
std::optional<VertMap> findSmallestCloseVertices(const Mesh&, float, const ProgressCallback&) { std::abort(); }
std::optional<VertMap> findSmallestCloseVertices(const VertCoords&, float, const VertBitSet*, const ProgressCallback&) {
    std::abort();
}
std::streamoff getStreamSize(std::istream&) { std::abort(); }

}  // namespace MR
