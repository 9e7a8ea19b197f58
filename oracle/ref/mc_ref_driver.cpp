// C entry points around MeshLib's own mesher (MRVoxels/MRMarchingCubes.cpp, compiled from the
// reference sources by oracle/ref/build_cpu_ref.py), used only to produce the golden vectors that
// pin the mesher oracle (oracle/mc_oracle.cpp) and, through them, the CUDA mesher.
// TEST INFRASTRUCTURE ONLY: nothing in the product loads this.
//
//   mcref_run  whole volume: marchingCubesAsTriMesh(SimpleVolume, params)
//              (MRVoxels/MRMarchingCubes.h:87) when nParts == 0 and layersPerBlock == 0;
//              otherwise MarchingCubesByParts(dims, params, layersPerBlock) (:104) fed the parts
//              that start at partStarts[] (each part repeats the previous part's last layer).
// Volumes are x-fastest float arrays; params carry origin, iso, lessInside, maxVertices and the
// face -> voxel map (MarchingCubesParams, MRVoxels/MRMarchingCubes.h:17-70).
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "MRVoxels/MRMarchingCubes.h"
#include "MRMesh/MRTriMesh.h"

namespace {

struct Result {
    std::vector<float> points;
    std::vector<int32_t> tris;
    std::vector<int32_t> faceMap;
    std::string error;
};

MR::SimpleVolume makeVolume(const float* vol, int nx, int ny, int z0, int z1, const float* voxelSize) {
    MR::SimpleVolume v;
    v.dims = MR::Vector3i(nx, ny, z1 - z0);
    v.voxelSize = MR::Vector3f(voxelSize[0], voxelSize[1], voxelSize[2]);
    const size_t layer = size_t(nx) * ny;
    v.data.resize(layer * size_t(z1 - z0));
    std::memcpy(v.data.data(), vol + layer * z0, sizeof(float) * v.data.size());
    return v;
}

void take(Result* r, MR::TriMesh&& tm, const MR::Vector<MR::VoxelId, MR::FaceId>& fmap) {
    r->points.reserve(tm.points.size() * 3);
    for (const auto& p : tm.points) {
        r->points.push_back(p.x);
        r->points.push_back(p.y);
        r->points.push_back(p.z);
    }
    r->tris.reserve(tm.tris.size() * 3);
    for (const auto& t : tm.tris)
        for (int k = 0; k < 3; ++k) r->tris.push_back(int32_t(int(t[k])));
    r->faceMap.reserve(fmap.size());
    for (const auto& v : fmap) r->faceMap.push_back(int32_t(size_t(v)));
}

}  // namespace

extern "C" {

void* mcref_run(const float* vol, const int32_t* dims, const float* origin, const float* voxelSize, float iso,
                int lessInside, const int32_t* partStarts, int nParts, int maxVertices, int layersPerBlock) {
    auto* r = new Result;
    MR::Vector<MR::VoxelId, MR::FaceId> fmap;
    MR::MarchingCubesParams params;
    params.origin = MR::Vector3f(origin[0], origin[1], origin[2]);
    params.iso = iso;
    params.lessInside = lessInside != 0;
    params.maxVertices = maxVertices;
    params.outVoxelPerFaceMap = &fmap;
    const int nx = dims[0], ny = dims[1], nz = dims[2];
    MR::Expected<MR::TriMesh> res;
    if (nParts == 0 && layersPerBlock == 0) {
        res = MR::marchingCubesAsTriMesh(makeVolume(vol, nx, ny, 0, nz, voxelSize), params);
    } else {
        MR::MarchingCubesByParts mc(MR::Vector3i(nx, ny, nz), params, layersPerBlock);
        std::vector<int32_t> starts = nParts > 0 ? std::vector<int32_t>(partStarts, partStarts + nParts)
                                                 : std::vector<int32_t>{0};
        MR::Expected<void> ok;
        for (size_t p = 0; p < starts.size() && ok; ++p) {
            const int z1 = p + 1 < starts.size() ? starts[p + 1] + 1 : nz;  // parts overlap by one layer
            ok = mc.addPart(makeVolume(vol, nx, ny, starts[p], z1, voxelSize));
        }
        if (ok)
            res = mc.finalize();
        else
            res = MR::unexpected(ok.error());
    }
    if (!res)
        r->error = res.error();
    else
        take(r, std::move(*res), fmap);
    return r;
}

int64_t mcref_num_points(void* h) { return int64_t(static_cast<Result*>(h)->points.size() / 3); }
int64_t mcref_num_tris(void* h) { return int64_t(static_cast<Result*>(h)->tris.size() / 3); }
const char* mcref_error(void* h) { return static_cast<Result*>(h)->error.c_str(); }
void mcref_get(void* h, float* pts, int32_t* tris, int32_t* faceMap) {
    auto* r = static_cast<Result*>(h);
    std::memcpy(pts, r->points.data(), sizeof(float) * r->points.size());
    std::memcpy(tris, r->tris.data(), sizeof(int32_t) * r->tris.size());
    std::memcpy(faceMap, r->faceMap.data(), sizeof(int32_t) * r->faceMap.size());
}
void mcref_free(void* h) { delete static_cast<Result*>(h); }

}  // extern "C"
