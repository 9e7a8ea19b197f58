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
    std::printf("OK sum_sd=%.6f sum_wn=%.6f neg=%d parts_equal=%d selfint=%d cancel_status=%d proj_max_diff=%.3g\n", sumSd, sumWn,
                neg, same, nbits, c.status(), maxDiff);
    return 0;
}
