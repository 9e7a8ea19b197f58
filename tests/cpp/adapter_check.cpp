// Exercises include/gbfwn.hpp (the C++ adapter with MeshLib's IFastWindingNumber shape) on a
// small torus and prints one line of results, which tests/test_cpp_adapter.py compares with the
// Python front-end on the same mesh.
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/gbfwn.hpp"

int main() {
    const int nu = 24, nv = 12;
    std::vector<float> verts;
    std::vector<int32_t> tris;
    for (int i = 0; i < nu; ++i)
        for (int j = 0; j < nv; ++j) {
            const double u = 2 * M_PI * i / nu, v = 2 * M_PI * j / nv;
            verts.push_back(float((1 + 0.3 * std::cos(v)) * std::cos(u)));
            verts.push_back(float((1 + 0.3 * std::cos(v)) * std::sin(u)));
            verts.push_back(float(0.3 * std::sin(v)));
        }
    for (int i = 0; i < nu; ++i)
        for (int j = 0; j < nv; ++j) {
            const int a = i * nv + j, b = ((i + 1) % nu) * nv + j, c = ((i + 1) % nu) * nv + (j + 1) % nv,
                      d = i * nv + (j + 1) % nv;
            tris.insert(tris.end(), {a, b, c, a, c, d});
        }
    gbfwn::FastWindingNumber fwn(verts.data(), int64_t(verts.size() / 3), tris.data(), int64_t(tris.size() / 3));
    if (!fwn.creation()) {
        std::printf("ERROR create %s\n", fwn.creation().error().c_str());
        return 1;
    }
    const int32_t dims[3] = {16, 16, 8};
    const float xf[12] = {0.18f, 0, 0, 0, 0.18f, 0, 0, 0, 0.1f, -1.4f, -1.4f, -0.4f};
    std::vector<float> sd, wn;
    if (auto r = fwn.calcFromGridWithDistances(sd, dims, xf, gbfwn::DistanceToMeshOptions{}); !r) {
        std::printf("ERROR sdf %s\n", r.error().c_str());
        return 1;
    }
    if (auto r = fwn.calcFromGrid(wn, dims, xf, 2.f); !r) {
        std::printf("ERROR grid %s\n", r.error().c_str());
        return 1;
    }
    std::vector<float> parts(sd.size(), NAN);
    int slabs = 0;
    auto r = fwn.calcFromGridWithDistancesByParts(
        [&](std::vector<float>&& data, const int32_t d[3], int z0) {
            std::copy(data.begin(), data.end(), parts.begin() + size_t(z0) * dims[0] * dims[1]);
            ++slabs;
            return gbfwn::Result{};
        },
        dims, xf, gbfwn::DistanceToMeshOptions{}, 0);
    if (!r) {
        std::printf("ERROR parts %s\n", r.error().c_str());
        return 1;
    }
    double sumSd = 0, sumWn = 0;
    int neg = 0, same = 1;
    for (size_t i = 0; i < sd.size(); ++i) {
        sumSd += sd[i];
        sumWn += wn[i];
        neg += sd[i] < 0;
        same &= parts[i] == sd[i];
    }
    std::vector<uint64_t> bits;
    fwn.calcSelfIntersections(bits, 2.f);
    int nbits = 0;
    for (auto w : bits) nbits += __builtin_popcountll(w);
    // cancellation through the progress callback
    std::vector<float> tmp;
    auto c = fwn.calcFromGrid(tmp, dims, xf, 2.f, [](float p) { return p < 0.5f; });
    // closest points through the projector adapter: the grid's voxel centres
    gbfwn::PointsToMeshProjector proj;
    if (auto pr = proj.updateMeshData(verts.data(), int64_t(verts.size() / 3), tris.data(), int64_t(tris.size() / 3)); !pr) {
        std::printf("ERROR projector %s\n", pr.error().c_str());
        return 1;
    }
    std::vector<float> pts;
    for (int z = 0; z < dims[2]; ++z)
        for (int y = 0; y < dims[1]; ++y)
            for (int x = 0; x < dims[0]; ++x)
                pts.insert(pts.end(), {xf[0] * x + xf[9], xf[4] * y + xf[10], xf[8] * z + xf[11]});
    std::vector<gbfwn_projection> pj;
    if (auto pr = proj.findProjections(pj, pts); !pr) {
        std::printf("ERROR project %s\n", pr.error().c_str());
        return 1;
    }
    double maxDiff = 0;
    for (size_t i = 0; i < pj.size(); ++i) maxDiff = std::fmax(maxDiff, std::fabs(std::sqrt(double(pj[i].distSq)) - std::fabs(sd[i])));
    // marching cubes on the signed-distance grid, whole and in 2-layer parts, and the fused call
    gbfwn::MarchingCubesParams mp;
    for (int k = 0; k < 3; ++k) {
        mp.voxelSize[k] = xf[4 * k];
        mp.origin[k] = xf[9 + k] - 0.5f * xf[4 * k];
    }
    mp.lessInside = true;
    mp.outVoxelPerFaceMap = true;
    gbfwn::TriMesh whole, byParts, fused;
    if (auto r = gbfwn::marchingCubes(whole, sd, dims, mp); !r) {
        std::printf("ERROR mc %s\n", r.error().c_str());
        return 1;
    }
    gbfwn::MarchingCubesByParts mcp(dims, mp);
    const size_t layer = size_t(dims[0]) * dims[1];
    for (int z = 0; z + 1 < dims[2]; ++z) {
        std::vector<float> part(sd.begin() + layer * z, sd.begin() + layer * (z + 2));
        const int32_t pd[3] = {dims[0], dims[1], 2};
        if (auto r = mcp.addPart(part, pd); !r) {
            std::printf("ERROR mc part %s\n", r.error().c_str());
            return 1;
        }
    }
    if (auto r = mcp.finalize(byParts); !r) {
        std::printf("ERROR mc finalize %s\n", r.error().c_str());
        return 1;
    }
    const float vs[3] = {xf[0], xf[4], xf[8]};
    if (auto r = fwn.gridToMesh(fused, dims, mp.origin, vs, gbfwn::DistanceToMeshOptions{}, mp); !r) {
        std::printf("ERROR grid_to_mesh %s\n", r.error().c_str());
        return 1;
    }
    const int mcSame = whole.tris == byParts.tris && whole.faceMap == byParts.faceMap && whole.tris == fused.tris;
    // the knobs: the torus is closed, and the grid without sign reuse is the same grid
    const int closed = fwn.isClosed() ? 1 : 0;
    fwn.setSignReuse(false);
    std::vector<float> sdPlain;
    if (auto r2 = fwn.calcFromGridWithDistances(sdPlain, dims, xf, gbfwn::DistanceToMeshOptions{}); !r2) {
        std::printf("ERROR sdf plain %s\n", r2.error().c_str());
        return 1;
    }
    fwn.setSignReuse(true);
    const int reuseSame = sdPlain == sd ? 1 : 0;
    std::printf("OK sum_sd=%.6f sum_wn=%.6f neg=%d parts_equal=%d selfint=%d cancel_status=%d proj_max_diff=%.3g "
                "mc_tris=%zu mc_points=%zu mc_same=%d closed=%d reuse_same=%d\n",
                sumSd, sumWn, neg, same, nbits, c.status(), maxDiff, whole.tris.size() / 3, whole.points.size() / 3, mcSame,
                closed, reuseSame);
    return 0;
}
