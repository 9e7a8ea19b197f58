// C entry points around MeshLib's own CPU winding-number / signed-distance path
// (MRMesh/MRFastWindingNumber.cpp with the tree, dipoles and projection it uses), compiled from the
// reference sources by oracle/ref/build_cpu_ref.py.  Used to produce golden vectors that pin the
// oracle (oracle/fwn_oracle.cpp) to the reference's own CPU arithmetic, and to time the reference
// code against the oracle's port on one core.
// TEST INFRASTRUCTURE ONLY: nothing in the product loads this.
//
//   fwnref_create                Mesh::fromTriangles (MRMesh/MRMesh.h:29) + FastWindingNumber(mesh)
//                                (MRMesh/MRFastWindingNumber.h:53)
//   fwnref_nodes / _dipoles      mesh.getAABBTree().nodes(), mesh.getDipoles() (MRMesh/MRMesh.h:461,473)
//   fwnref_from_grid_with_distances / _from_grid / _from_vector / _self_intersections
//                                the IFastWindingNumber methods (MRMesh/MRFastWindingNumber.h:26-44)
//   fwnref_grid_voxels           calcWithDistances (:62) at chosen voxels of a grid, as
//                                calcFromGridWithDistances evaluates them (MRFastWindingNumber.cpp:86-93)
//   fwnref_project               findProjection (MRMesh/MRMeshProject.h:56)
// The TBB stand-in runs every parallel loop serially: all timings are one core.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "MRMesh/MRAABBTree.h"
#include "MRMesh/MRAffineXf3.h"
#include "MRMesh/MRBitSet.h"
#include "MRMesh/MRDipole.h"
#include "MRMesh/MRDistanceToMeshOptions.h"
#include "MRMesh/MRFastWindingNumber.h"
#include "MRMesh/MRMesh.h"
#include "MRMesh/MRMeshBuilder.h"
#include "MRMesh/MRMeshProject.h"
#include "MRMesh/MRVolumeIndexer.h"

namespace {

struct Handle {
    MR::Mesh mesh;
    std::unique_ptr<MR::FastWindingNumber> fwn;
};

MR::AffineXf3f xfFrom12(const float* x) {  // row-major 3x3 followed by the translation
    return MR::AffineXf3f(MR::Matrix3f({x[0], x[1], x[2]}, {x[3], x[4], x[5]}, {x[6], x[7], x[8]}),
                          MR::Vector3f(x[9], x[10], x[11]));
}

MR::DistanceToMeshOptions optsFrom(const float* o) {  // minDistSq, maxDistSq, nullOutsideMinMax, threshold, beta
    MR::DistanceToMeshOptions r;
    r.minDistSq = o[0];
    r.maxDistSq = o[1];
    r.nullOutsideMinMax = o[2] != 0.f;
    r.windingNumberThreshold = o[3];
    r.windingNumberBeta = o[4];
    return r;
}

}  // namespace

extern "C" {

void* fwnref_create(const float* verts, int64_t nv, const int32_t* faces, int64_t nf) {
    MR::VertCoords pts;
    pts.resize(size_t(nv));
    for (int64_t i = 0; i < nv; ++i) pts[MR::VertId(int(i))] = MR::Vector3f(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
    MR::Triangulation t;
    t.resize(size_t(nf));
    for (int64_t f = 0; f < nf; ++f)
        t[MR::FaceId(int(f))] = {MR::VertId(faces[3 * f]), MR::VertId(faces[3 * f + 1]), MR::VertId(faces[3 * f + 2])};
    auto* h = new Handle;
    h->mesh = MR::Mesh::fromTriangles(std::move(pts), t);
    h->fwn = std::make_unique<MR::FastWindingNumber>(h->mesh);
    return h;
}

void fwnref_destroy(void* h) { delete static_cast<Handle*>(h); }

int64_t fwnref_num_nodes(void* hp) { return int64_t(static_cast<Handle*>(hp)->mesh.getAABBTree().nodes().size()); }

// 32 bytes per node: box min (3 floats), box max (3 floats), l, r (int32)
void fwnref_nodes(void* hp, void* out) {
    const auto& nodes = static_cast<Handle*>(hp)->mesh.getAABBTree().nodes();
    auto* o = static_cast<uint8_t*>(out);
    for (size_t i = 0; i < nodes.size(); ++i) {
        const auto& n = nodes[MR::NodeId(int(i))];
        const float b[6] = {n.box.min.x, n.box.min.y, n.box.min.z, n.box.max.x, n.box.max.y, n.box.max.z};
        const int32_t lr[2] = {int32_t(int(n.l)), int32_t(int(n.r))};
        std::memcpy(o + 32 * i, b, 24);
        std::memcpy(o + 32 * i + 24, lr, 8);
    }
}

// 8 floats per node: pos, area, dirArea, rr
void fwnref_dipoles(void* hp, float* out) {
    const auto& d = static_cast<Handle*>(hp)->mesh.getDipoles();
    for (size_t i = 0; i < d.size(); ++i) {
        const auto& x = d[MR::NodeId(int(i))];
        const float v[8] = {x.pos.x, x.pos.y, x.pos.z, x.area, x.dirArea.x, x.dirArea.y, x.dirArea.z, x.rr};
        std::memcpy(out + 8 * i, v, sizeof(v));
    }
}

int fwnref_from_grid_with_distances(void* hp, const int32_t* dims, const float* xf12, const float* opts, float* out) {
    auto* h = static_cast<Handle*>(hp);
    std::vector<float> res;
    if (!h->fwn->calcFromGridWithDistances(res, MR::Vector3i(dims[0], dims[1], dims[2]), xfFrom12(xf12), optsFrom(opts), {}))
        return 1;
    std::memcpy(out, res.data(), sizeof(float) * res.size());
    return 0;
}

int fwnref_from_grid(void* hp, const int32_t* dims, const float* xf12, float beta, float* out) {
    auto* h = static_cast<Handle*>(hp);
    std::vector<float> res;
    if (!h->fwn->calcFromGrid(res, MR::Vector3i(dims[0], dims[1], dims[2]), xfFrom12(xf12), beta, {})) return 1;
    std::memcpy(out, res.data(), sizeof(float) * res.size());
    return 0;
}

int fwnref_from_vector(void* hp, const float* pts, int64_t n, float beta, int32_t skipFace, float* out) {
    auto* h = static_cast<Handle*>(hp);
    std::vector<MR::Vector3f> p(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) p[size_t(i)] = MR::Vector3f(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    std::vector<float> res;
    if (!h->fwn->calcFromVector(res, p, beta, skipFace >= 0 ? MR::FaceId(skipFace) : MR::FaceId(), {})) return 1;
    std::memcpy(out, res.data(), sizeof(float) * res.size());
    return 0;
}

// one byte per face: 1 where the reference sets the face's bit
int fwnref_self_intersections(void* hp, float beta, uint8_t* out) {
    auto* h = static_cast<Handle*>(hp);
    MR::FaceBitSet bits;
    if (!h->fwn->calcSelfIntersections(bits, beta, {})) return 1;
    const size_t nf = h->mesh.topology.faceSize();
    for (size_t f = 0; f < nf; ++f) out[f] = (f < bits.size() && bits.test(MR::FaceId(int(f)))) ? 1 : 0;
    return 0;
}

void fwnref_grid_voxels(void* hp, const int32_t* dims, const float* xf12, const float* opts, const int64_t* ids, int64_t n,
                        float* out) {
    auto* h = static_cast<Handle*>(hp);
    const MR::VolumeIndexer indexer(MR::Vector3i(dims[0], dims[1], dims[2]));
    const auto xf = xfFrom12(xf12);
    const auto o = optsFrom(opts);
    for (int64_t i = 0; i < n; ++i)
        out[i] = h->fwn->calcWithDistances(xf(MR::Vector3f(indexer.toPos(MR::VoxelId(size_t(ids[i]))))), o);
}

// per point: distSq, face id (as int32 bits), projection x, y, z, barycentric a, b, edge id (as int32 bits)
void fwnref_project(void* hp, const float* pts, int64_t n, float upDistLimitSq, float* out) {
    auto* h = static_cast<Handle*>(hp);
    for (int64_t i = 0; i < n; ++i) {
        const auto r = MR::findProjection(MR::Vector3f(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]), h->mesh, upDistLimitSq);
        const int32_t face = int32_t(int(r.proj.face)), edge = int32_t(int(r.mtp.e));
        float* o = out + 8 * i;
        o[0] = r.distSq;
        std::memcpy(o + 1, &face, 4);
        o[2] = r.proj.point.x;
        o[3] = r.proj.point.y;
        o[4] = r.proj.point.z;
        o[5] = r.mtp.bary.a;
        o[6] = r.mtp.bary.b;
        std::memcpy(o + 7, &edge, 4);
    }
}

}  // extern "C"
