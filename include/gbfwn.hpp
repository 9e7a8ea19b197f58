// gbfwn.hpp -- header-only C++ adapter over the C ABI (gbfwn.h) with the shape of MeshLib's
// MR::IFastWindingNumber / MR::IFastWindingNumberByParts (MRMesh/MRFastWindingNumber.h:11-107).
//
// It depends on nothing but the C++ standard library, so it compiles inside or outside MeshLib;
// the MeshLib-side class MR::GbFastWindingNumber (include/MRGbFastWindingNumber.h) derives from
// MR::IFastWindingNumberByParts and forwards to this one.  Method names, argument meaning and error behaviour follow the reference:
// results are written to caller-owned std::vector / bitset words that the callee resizes, and
// every call returns an Expected-like value whose error is the library's message.
#pragma once

#include <cstdint>
#include <functional>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "gbfwn.h"

namespace gbfwn {

// Minimal Expected<void>: ok() or an error string ("NVIDIA GPU error: ...", "operation canceled").
class Result {
public:
    Result() = default;
    static Result fromStatus(int st) {
        Result r;
        r.status_ = st;
        if (st != GBFWN_OK) r.error_ = gbfwn_last_error();
        return r;
    }
    explicit operator bool() const { return status_ == GBFWN_OK; }
    int status() const { return status_; }
    const std::string& error() const { return error_; }

private:
    int status_ = GBFWN_OK;
    std::string error_;
};

using ProgressCallback = std::function<bool(float)>;  // MR::ProgressCallback
// MR::IFastWindingNumberByParts::GridByPartsFunc: (slab data, slab dims, zOffset) -> Result
using GridByPartsFunc = std::function<Result(std::vector<float>&& data, const int32_t dims[3], int zOffset)>;

struct DistanceToMeshOptions {  // MR::DistanceToMeshOptions
    float minDistSq = 0.f;
    float maxDistSq = 3.402823466e+38f;
    bool nullOutsideMinMax = true;
    float windingNumberThreshold = 0.5f;
    float windingNumberBeta = 2.f;
    gbfwn_dist_opts c() const {
        return gbfwn_dist_opts{minDistSq, maxDistSq, nullOutsideMinMax ? 1 : 0, windingNumberThreshold, windingNumberBeta};
    }
};

namespace detail {
inline int progressThunk(float p, void* user) { return (*static_cast<const ProgressCallback*>(user))(p) ? 1 : 0; }
struct SlabCtx {
    GridByPartsFunc* fn;
    Result err;
};
inline int slabThunk(const float* data, const int32_t dims[3], int32_t zOffset, void* user) {
    auto* ctx = static_cast<SlabCtx*>(user);
    const size_t n = size_t(dims[0]) * size_t(dims[1]) * size_t(dims[2]);
    std::vector<float> v(data, data + n);
    ctx->err = (*ctx->fn)(std::move(v), dims, zOffset);
    return ctx->err ? 0 : (ctx->err.status() ? ctx->err.status() : GBFWN_CANCELLED);
}
}  // namespace detail

// MR::TriMesh as the mesher returns it: points (3 floats each), triangles (3 vertex ids each) and,
// when requested, the face -> voxel map (MR::Vector<VoxelId, FaceId>).
struct TriMesh {
    std::vector<float> points;
    std::vector<int32_t> tris;
    std::vector<int32_t> faceMap;
};

// MR::MarchingCubesParams (MRVoxels/MRMarchingCubes.h:18-61) for the default linear positioner;
// voxelSize is the volume's (SimpleVolume::voxelSize).
struct MarchingCubesParams {
    float origin[3] = {0.f, 0.f, 0.f};
    float voxelSize[3] = {1.f, 1.f, 1.f};
    float iso = 0.f;
    bool lessInside = false;
    int64_t maxVertices = 2147483647;
    bool outVoxelPerFaceMap = false;
    gbfwn_mc_params c() const {
        gbfwn_mc_params p;
        gbfwn_mc_default_params(&p);
        for (int k = 0; k < 3; ++k) {
            p.origin[k] = origin[k];
            p.voxelSize[k] = voxelSize[k];
        }
        p.iso = iso;
        p.lessInside = lessInside ? 1 : 0;
        p.maxVertices = maxVertices;
        p.wantFaceMap = outVoxelPerFaceMap ? 1 : 0;
        return p;
    }
};

namespace detail {
// copies a device mesh into `out` and frees it
inline Result takeMesh(int st, gbfwn_trimesh m, TriMesh& out) {
    if (st != GBFWN_OK) return Result::fromStatus(st);
    int64_t np = 0, nt = 0;
    gbfwn_trimesh_sizes(m, &np, &nt);
    const int32_t* dFace = nullptr;
    gbfwn_trimesh_device(m, nullptr, nullptr, &dFace);
    out.points.resize(size_t(3 * np));
    out.tris.resize(size_t(3 * nt));
    out.faceMap.resize(dFace ? size_t(nt) : 0);
    st = gbfwn_trimesh_copy(m, out.points.data(), out.tris.data(), dFace ? out.faceMap.data() : nullptr);
    gbfwn_trimesh_destroy(m);
    return Result::fromStatus(st);
}
}  // namespace detail

// MR::marchingCubesAsTriMesh(SimpleVolume, params) (MRVoxels/MRMarchingCubes.h:66) on the GPU:
// the same TriMesh, bit for bit.  volume: dims[0] x dims[1] x dims[2] floats, x fastest.
inline Result marchingCubes(TriMesh& out, const std::vector<float>& volume, const int32_t dims[3],
                            const MarchingCubesParams& params = {}, const ProgressCallback& cb = {}, int device = 0) {
    const gbfwn_mc_params p = params.c();
    gbfwn_trimesh m = nullptr;
    const int st = gbfwn_marching_cubes(volume.data(), dims, &p, nullptr, 0, device, &m,
                                        cb ? &detail::progressThunk : nullptr,
                                        cb ? const_cast<ProgressCallback*>(&cb) : nullptr);
    return detail::takeMesh(st, m, out);
}

// MR::MarchingCubesByParts (MRVoxels/MRMarchingCubes.h:96-122): addPart() volumes of whole XY layers
// starting at nextZ() (the previous part's last layer repeated), then finalize().
class MarchingCubesByParts {
public:
    MarchingCubesByParts(const int32_t dims[3], const MarchingCubesParams& params, int device = 0) {
        const gbfwn_mc_params p = params.c();
        gbfwn_mc_parts h = nullptr;
        created_ = Result::fromStatus(gbfwn_mc_parts_create(dims, &p, device, &h));
        h_.reset(h);
    }
    int nextZ() const { return h_ ? gbfwn_mc_parts_next_z(h_.get()) : 0; }
    Result addPart(const std::vector<float>& part, const int32_t partDims[3]) {
        if (!h_) return created_;
        return Result::fromStatus(gbfwn_mc_parts_add(h_.get(), part.data(), partDims));
    }
    Result finalize(TriMesh& out) {
        if (!h_) return created_;
        gbfwn_trimesh m = nullptr;
        const int st = gbfwn_mc_parts_finalize(h_.get(), &m);
        return detail::takeMesh(st, m, out);
    }

private:
    struct Del {
        void operator()(gbfwn_mc_parts p) const { gbfwn_mc_parts_destroy(p); }
    };
    std::unique_ptr<gbfwn_mc_parts_s, Del> h_;
    Result created_;
};

// GPU fast winding number of one mesh.  Like MR::Cuda::FastWindingNumber it keeps the device data
// (mesh, tree, dipoles) for the lifetime of the object; calls on one object are serialised.
class FastWindingNumber {
public:
    // verts: nv x 3 floats; tris: nt x 3 vertex ids (a face with a negative id is invalid).
    FastWindingNumber(const float* verts, int64_t nv, const int32_t* tris, int64_t nt, int device = 0) {
        gbfwn_handle h = nullptr;
        created_ = Result::fromStatus(gbfwn_create(verts, nv, tris, nt, device, &h));
        h_.reset(h);
    }
    const Result& creation() const { return created_; }
    gbfwn_handle handle() const { return h_.get(); }

    // Knobs of include/gbfwn.h: compensated sums and FP64 near-plane fallbacks (default on); exact
    // signs of closed meshes from column crossings, neighbouring voxels or rays (default on).
    void setPrecise(bool precise) { gbfwn_set_precise(h_.get(), precise ? 1 : 0); }
    void setSignReuse(bool enable) { gbfwn_set_sign_reuse(h_.get(), enable ? 1 : 0); }
    bool isClosed() const { return gbfwn_is_closed(h_.get()) != 0; }

    Result calcFromVector(std::vector<float>& res, const std::vector<float>& points /* 3 per point */, float beta,
                          int32_t skipFace = -1, const ProgressCallback& cb = {}) {
        res.resize(points.size() / 3);
        return Result::fromStatus(gbfwn_from_vector(h_.get(), points.data(), int64_t(res.size()), beta, skipFace, res.data(),
                                                    cb ? &detail::progressThunk : nullptr, cbUser(cb)));
    }

    // res: one bit per face in 64-bit words (MeshLib FaceBitSet blocks)
    Result calcSelfIntersections(std::vector<uint64_t>& res, float beta, const ProgressCallback& cb = {}) {
        res.assign(size_t((gbfwn_num_faces(h_.get()) + 63) / 64), 0);
        return Result::fromStatus(gbfwn_self_intersections(h_.get(), beta, res.data(), nullptr,
                                                           cb ? &detail::progressThunk : nullptr, cbUser(cb)));
    }

    // gridToMeshXf: 3x3 rows then translation (MR::AffineXf3f)
    Result calcFromGrid(std::vector<float>& res, const int32_t dims[3], const float gridToMeshXf[12], float beta,
                        const ProgressCallback& cb = {}) {
        res.resize(size_t(dims[0]) * size_t(dims[1]) * size_t(dims[2]));
        return Result::fromStatus(gbfwn_from_grid(h_.get(), dims, gridToMeshXf, beta, res.data(),
                                                  cb ? &detail::progressThunk : nullptr, cbUser(cb)));
    }

    Result calcFromGridWithDistances(std::vector<float>& res, const int32_t dims[3], const float gridToMeshXf[12],
                                     const DistanceToMeshOptions& options, const ProgressCallback& cb = {}) {
        res.resize(size_t(dims[0]) * size_t(dims[1]) * size_t(dims[2]));
        const gbfwn_dist_opts o = options.c();
        return Result::fromStatus(gbfwn_from_grid_with_distances(h_.get(), dims, gridToMeshXf, &o, res.data(),
                                                                 cb ? &detail::progressThunk : nullptr, cbUser(cb)));
    }

    Result calcFromGridByParts(GridByPartsFunc resFunc, const int32_t dims[3], const float gridToMeshXf[12], float beta,
                               int layerOverlap, const ProgressCallback& cb = {}) {
        detail::SlabCtx ctx{&resFunc, Result{}};
        const int st = gbfwn_from_grid_by_parts(h_.get(), dims, gridToMeshXf, beta, layerOverlap, 0, &detail::slabThunk, &ctx,
                                                cb ? &detail::progressThunk : nullptr, cbUser(cb));
        if (!ctx.err) return ctx.err;
        return Result::fromStatus(st);
    }

    Result calcFromGridWithDistancesByParts(GridByPartsFunc resFunc, const int32_t dims[3], const float gridToMeshXf[12],
                                            const DistanceToMeshOptions& options, int layerOverlap,
                                            const ProgressCallback& cb = {}) {
        detail::SlabCtx ctx{&resFunc, Result{}};
        const gbfwn_dist_opts o = options.c();
        const int st = gbfwn_from_grid_with_distances_by_parts(h_.get(), dims, gridToMeshXf, &o, layerOverlap, 0,
                                                               &detail::slabThunk, &ctx,
                                                               cb ? &detail::progressThunk : nullptr, cbUser(cb));
        if (!ctx.err) return ctx.err;
        return Result::fromStatus(st);
    }

    // mcOffsetMesh's volume step fused on the device: the signed-distance grid of dims voxels centred
    // at origin + (i + 0.5) * voxelSize, meshed by marching cubes without leaving the GPU
    // (gbfwn_grid_to_mesh).  mcOffsetMesh passes mc.origin = origin, mc.iso = offset, lessInside.
    Result gridToMesh(TriMesh& out, const int32_t dims[3], const float origin[3], const float voxelSize[3],
                      const DistanceToMeshOptions& options, const MarchingCubesParams& mc, const ProgressCallback& cb = {}) {
        const gbfwn_dist_opts o = options.c();
        const gbfwn_mc_params p = mc.c();
        gbfwn_trimesh m = nullptr;
        const int st = gbfwn_grid_to_mesh(h_.get(), nullptr, dims, origin, voxelSize, &o, &p, nullptr, 0, &m,
                                          cb ? &detail::progressThunk : nullptr, cbUser(cb));
        return detail::takeMesh(st, m, out);
    }

private:
    static void* cbUser(const ProgressCallback& cb) { return cb ? const_cast<ProgressCallback*>(&cb) : nullptr; }
    struct Del {
        void operator()(gbfwn_handle h) const { gbfwn_destroy(h); }
    };
    std::unique_ptr<gbfwn_mesh_s, Del> h_;
    Result created_;
};

// GPU closest points on one mesh with the shape of MR::IPointsToMeshProjector
// (MRMesh/MRPointsToMeshProjector.h:11-30).  It keeps the mesh's device tree between calls like
// MR::Cuda::PointsToMeshProjector; results are gbfwn_projection records, the memory layout of
// MR::MeshProjectionResult, with edge = -1 for the caller's topology to fill (edgeWithLeft(face)).
class PointsToMeshProjector {
public:
    explicit PointsToMeshProjector(int device = 0) : device_(device) {}

    // verts: nv x 3 floats; tris: nt x 3 vertex ids.  verts == nullptr forgets the mesh.
    Result updateMeshData(const float* verts, int64_t nv, const int32_t* tris, int64_t nt) {
        h_.reset();
        if (!verts) return Result{};
        gbfwn_handle h = nullptr;
        Result r = Result::fromStatus(gbfwn_create(verts, nv, tris, nt, device_, &h));
        h_.reset(h);
        return r;
    }

    // objXf maps the points, refXf the mesh (12 floats each: 3x3 rows then translation; nullptr = none)
    Result findProjections(std::vector<gbfwn_projection>& result, const std::vector<float>& points /* 3 per point */,
                           const float* objXf = nullptr, const float* refXf = nullptr,
                           float upDistLimitSq = 3.402823466e+38f, float loDistLimitSq = 0.f) {
        if (!h_) return Result::fromStatus(GBFWN_INVALID);
        result.resize(points.size() / 3);
        return Result::fromStatus(gbfwn_find_projections(h_.get(), points.data(), int64_t(result.size()), objXf, refXf,
                                                         upDistLimitSq, loDistLimitSq, result.data(), nullptr, nullptr));
    }

    size_t projectionsHeapBytes(size_t numProjections) const { return gbfwn_projections_heap_bytes(int64_t(numProjections)); }

private:
    struct Del {
        void operator()(gbfwn_handle h) const { gbfwn_destroy(h); }
    };
    int device_;
    std::unique_ptr<gbfwn_mesh_s, Del> h_;
};

}  // namespace gbfwn
