// CPU oracle for marching cubes over a signed-distance volume.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, serially and in plain C++, MeshLib's
// `VolumeMesher` (the engine of `marchingCubes(SimpleVolume)` and `MarchingCubesByParts`) so that
// the CUDA mesher can be checked against it bit for bit.  Only the tests and the CPU-baseline leg
// of the benchmark load it; the product never does.  It is itself pinned to MeshLib's own mesher,
// compiled from the reference sources (oracle/ref/build_cpu_ref.py): tests/test_mc_golden_cpu.py
// compares it with that mesher's outputs in tests/golden/mc_reference.npz, bit for bit.
//
// Reference files restated here (paths inside the MeshLib project):
//   source/MRVoxels/MRMarchingCubes.cpp:25-65     edge -> (corner, direction) map, corner offsets,
//                                                 corner -> configuration bit
//   source/MRVoxels/MRMarchingCubes.cpp:67-323    the triangulation table (256 plans)
//   source/MRVoxels/MRMarchingCubes.cpp:431-546   addPart: part checks, z ranges of the parts
//   source/MRVoxels/MRMarchingCubes.cpp:548-662   addPartBlock_: separation points on +X/+Y/+Z edges
//   source/MRVoxels/MRMarchingCubes.cpp:812-1103  finalize: per-cell configuration with NaN corner
//                                                 substitution, neighbour checks, triangles
//   source/MRMesh/MRSeparationPoint.cpp:13-72     vertex numbering (blocks in z order)
//   source/MRVoxels/MRVoxelsVolumeAccess.h:78     voxel-centre shift 0.5
//
// Numbering.  The reference fills separation points per z-block in voxel order (x fastest, then
// y, then z) and, within a voxel, in X, Y, Z order, then shifts each block by the count of the
// blocks before it: the global vertex id is the rank of (voxel id, direction) over all points,
// whatever the block partition.  Triangles are emitted per cell in voxel order and, within a cell,
// in plan order, and the blocks are concatenated in z order: the same holds for them.  So a
// serial sweep reproduces both orders.
//
// Coordinates.  A part that starts at layer z0 places voxel (x, y, z) at
//   zeroPoint + voxelSize * (x, y, z - z0),  zeroPoint = origin + (0.5, 0.5, 0.5 + z0) * voxelSize,
// each operation rounded to float (compile with -ffp-contract=off); a crossing on the edge to the
// +n neighbour is (1 - r) * p0 + r * p1 with r = (iso - v0) / (v1 - v0) and p1 = p0 + voxelSize[n]
// along n.  The whole volume at once is one part starting at 0.
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

// Edge e of a cell: the corner it starts from and the +direction it runs along
// (MRMarchingCubes.cpp:25-40); corners are numbered x + 2y + 4z.
const int kEdgeCorner[12] = {0, 1, 2, 0, 4, 5, 6, 4, 0, 1, 3, 2};
const int kEdgeDir[12] = {0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2};
// corner -> configuration bit (the polygonise table's vertex numbering, MRMarchingCubes.cpp:52-65)
const int kCornerBit[8] = {0, 1, 3, 2, 4, 5, 7, 6};

// The triangulation table of MRMarchingCubes.cpp:67-323 (256 plans; every three hex digits are the
// edges of one triangle).  The same data as the reference's: the output must list the same
// triangles in the same order.
const char* const kPlans[256] = {
    "", "083", "019", "183981", "12a", "08312a", "92a029", "2832a8a98",
    "3b2", "0b28b0", "19023b", "1b219b98b", "3a1ba3", "0a108a8ba", "3903b9ba9", "98aa8b",
    "478", "430734", "019847", "419471731", "12a847", "34730412a", "92a902847", "2a9297273794",
    "8473b2", "b47b24204", "90184723b", "47b94b9b2921", "3a13ba784", "1ba14b1047b4", "47890b9bab03", "47b4b99ba",
    "954", "954083", "054150", "854835315", "12a954", "30812a495", "52a542402", "2a5325354348",
    "95423b", "0b208b495", "05401523b", "21525828b485", "a3ba13954", "4950818a18ba", "54050b5bab03", "54858aa8b",
    "978579", "930953573", "078017157", "153357", "978957a12", "a12950530573", "802825857a52", "2a5253357",
    "7957893b2", "95797292027b", "23b018178157", "b21b17715", "958857a13a3b", "5705097b010aba0", "ba0b03a50807570", "ba57b5",
    "a65", "0835a6", "9015a6", "1831985a6", "165261", "165126308", "965906026", "598582526328",
    "23ba65", "b08b20a65", "01923b5a6", "5a61929b298b", "63b653513", "08b0b50515b6", "3b6036065059", "65969bb98",
    "5a6478", "43047365a", "1905a6847", "a65197173794", "612651478", "125526304347", "847905065026", "739794329596269",
    "3b2784a65", "5a647242027b", "01947823b5a6", "9219b294b7b45a6", "8473b53515b6", "51b5b610b7b404b", "059065036b63847", "65969b4797b9",
    "a4964a", "4a649a083", "a01a60640", "83181686461a", "149124264", "308129249264", "024426", "832824426",
    "a49a64b23", "08228b49a4a6", "3b201606461a", "64161a48121b8b1", "964936913b63", "8b1810b61914641", "3b6360064", "648b68",
    "7a678a89a", "0730a709a67a", "a671a7178180", "a67a71173", "126168189867", "269291679093739", "780706602", "732672",
    "23ba68a89867", "20727b09767a9a7", "1801781a767a23b", "b21b17a61671", "896867916b63136", "091b67", "7807063b0b60", "7b6",
    "76b", "308b76", "019b76", "819831b76", "a126b7", "12a3086b7", "2902a96b7", "6b72a3a83a98",
    "723627", "708760620", "276237019", "162186198876", "a76a17137", "a7617a187108", "03707a0a96a7", "76a7a88a9",
    "684b86", "36b306046", "86b846901", "946963931b36", "6846b82a1", "12a30b06b046", "4b846b0292a9", "a93a32943b36463",
    "823842462", "042462", "190234246438", "194142246", "8138618466a1", "a10a06604", "4634386a3039a93", "a946a4",
    "49576b", "083495b76", "50154076b", "b76834354315", "954a1276b", "6b712a083495", "76b54a42a402", "348354325a52b76",
    "723762549", "954086062687", "362376150540", "628687218485158", "954a16176137", "16a176107870954", "40a4a503a6a737a", "76a7a854a48a",
    "6956b9b89", "36b063056095", "0b805b01556b", "6b3635531", "12a95b9b8b56", "0b306b09656912a", "b85b56805a52025", "6b36352a3a53",
    "589528562382", "956960062", "158180568382628", "156216", "13616a386569896", "a10a06950560", "03856a", "a56",
    "b5a75b", "b5ab75830", "5b75ab190", "a75ab7981831", "b12b71751", "08312717572b", "9759279022b7", "75272b592328982",
    "25a235375", "820852875a25", "9015a35373a2", "982921872a25752", "135375", "087071175", "903935537", "987597",
    "5845a8ab8", "5045b05abb30", "01984a8aba45", "ab4a45b34941314", "2512852b8458", "04b0b345b2b151b", "0250592b5458b85", "9452b3",
    "25a352345384", "5a2524420", "3a235a385458019", "5a2524192942", "845853351", "045105", "845853905035", "945",
    "4b749b9ab", "0834979b79ab", "1ab1b414074b", "3143481a474bab4", "4b79b492b912", "9749b791b2b1083", "b74b42240", "b74b42834324",
    "29a279237749", "9a7974a27870207", "37a3a274a1a040a", "1a2874", "491417713", "491417081871", "403743", "487",
    "9a8ab8", "30939bb9a", "01a0a88ab", "31ab3a", "12b1b99b8", "30939b1292b9", "02b80b", "32b",
    "23828aa89", "9a2092", "23828a0181a8", "1a2", "138918", "091", "038", "",};

struct McResult {
    std::vector<float> points;     // 3 per vertex
    std::vector<int32_t> tris;     // 3 per triangle
    std::vector<int32_t> faceMap;  // voxel id of each triangle's cell
    std::string error;
};

inline int hexDigit(char c) { return c <= '9' ? c - '0' : c - 'a' + 10; }

}  // namespace

extern "C" {

// partStarts: first layer of each part (parts overlap by one layer, the last layer of a part being
// the first of the next), nParts = 0 for the whole volume at once.
void* orc_mc(const float* vol, const int32_t* dims, const float* origin, const float* voxelSize, float iso,
             int lessInside, const int32_t* partStarts, int nParts, int64_t maxVertices) {
    McResult* R = new McResult;
    const int dx = dims[0], dy = dims[1], dz = dims[2];
    if (dx <= 0 || dy <= 0 || dz <= 0) return R;  // empty mesh (VolumeMesher::run)
    std::vector<int32_t> starts;
    if (nParts <= 0)
        starts.push_back(0);
    else
        starts.assign(partStarts, partStarts + nParts);
    // addPart checks, part by part (MRMarchingCubes.cpp:436-441, 816-817)
    if (starts[0] != 0) {
        R->error = "a part exceeds whole volume in Z dimension";
        return R;
    }
    for (size_t p = 0; p < starts.size(); ++p) {
        const int end = p + 1 < starts.size() ? starts[p + 1] : dz - 1;  // last layer of the part
        if (end - starts[p] + 1 <= 1) {
            R->error = "a part must have at least two Z slices";
            return R;
        }
        if (end > dz - 1) {
            R->error = "a part exceeds whole volume in Z dimension";
            return R;
        }
    }
    const int64_t sx = dx, sxy = int64_t(dx) * dy;
    // separation points: per voxel the vertex ids on its +X/+Y/+Z edges (-1 = none)
    std::unordered_map<int64_t, std::array<int32_t, 3>> sep;
    int64_t nextVid = 0;
    size_t part = 0;
    for (int z = 0; z < dz; ++z) {
        while (part + 1 < starts.size() && z >= starts[part + 1]) ++part;
        const int z0 = starts[part];
        const float zpX = origin[0] + 0.5f * voxelSize[0];
        const float zpY = origin[1] + 0.5f * voxelSize[1];
        const float zpZ = origin[2] + (0.5f + float(z0)) * voxelSize[2];
        const float cz = zpZ + voxelSize[2] * float(z - z0);
        for (int y = 0; y < dy; ++y) {
            const float cy = zpY + voxelSize[1] * float(y);
            for (int x = 0; x < dx; ++x) {
                const int64_t id = z * sxy + y * sx + x;
                const float v = vol[id];
                const bool lower = v < iso, notLower = v >= iso;
                if (!lower && !notLower) continue;  // NaN: no points
                const float c[3] = {zpX + voxelSize[0] * float(x), cy, cz};
                std::array<int32_t, 3> set = {-1, -1, -1};
                bool any = false;
                for (int n = 0; n < 3; ++n) {
                    const bool has = n == 0 ? x + 1 < dx : n == 1 ? y + 1 < dy : z + 1 < dz;
                    if (!has) continue;
                    const float nv = vol[id + (n == 0 ? 1 : n == 1 ? sx : sxy)];
                    if (lower ? !(nv >= iso) : !(nv < iso)) continue;
                    float c1[3] = {c[0], c[1], c[2]};
                    c1[n] = c[n] + voxelSize[n];
                    const float r = (iso - v) / (nv - v);
                    const float w = 1.0f - r;
                    for (int k = 0; k < 3; ++k) R->points.push_back(w * c[k] + r * c1[k]);
                    set[n] = int32_t(nextVid++);
                    any = true;
                }
                if (any) sep.emplace(id, set);
            }
        }
    }
    if (nextVid > maxVertices) {
        R->points.clear();
        R->error = "Vertices number limit exceeded.";
        return R;
    }
    const int64_t cornerAdd[8] = {0, 1, sx, sx + 1, sxy, sxy + 1, sxy + sx, sxy + sx + 1};
    auto lowerAt = [&](int64_t id, bool& invalid) {
        const float v = vol[id];
        invalid = !(v < iso) && !(v >= iso);
        return v < iso;
    };
    for (int z = 0; z + 1 < dz; ++z)
        for (int y = 0; y + 1 < dy; ++y)
            for (int x = 0; x + 1 < dx; ++x) {
                const int64_t id = z * sxy + y * sx + x;
                bool vx[8], ivx[8];
                bool allInvalid = true;
                for (int i = 0; i < 8; ++i) {
                    vx[i] = lowerAt(id + cornerAdd[i], ivx[i]);
                    allInvalid = allInvalid && ivx[i];
                }
                if (allInvalid) continue;
                // an invalid corner takes the side of its first valid neighbour corner, in the
                // order x, y, z, xy, xz, yz, xyz (MRMarchingCubes.cpp:913-951)
                static const int order[7] = {1, 2, 4, 3, 5, 6, 7};
                bool nanCorner = false;
                int config = 0;
                for (int i = 0; i < 8; ++i) {
                    if (ivx[i]) {
                        nanCorner = true;
                        for (int k = 0; k < 7; ++k)
                            if (!ivx[i ^ order[k]]) {
                                vx[i] = vx[i ^ order[k]];
                                break;
                            }
                    }
                    if (vx[i]) config |= 1 << kCornerBit[i];
                }
                if (config == 0 || config == 0xff) continue;
                // the corners whose separation points the cell may use (MRMarchingCubes.cpp:955-1000)
                const std::array<int32_t, 3>* nei[7] = {};
                bool valid = false;
                auto find = [&](int i, int need) {
                    auto it = sep.find(id + cornerAdd[i]);
                    if (it == sep.end()) return;
                    const auto& s = it->second;
                    const bool ok = need == 7 || ((need & 1) && s[0] >= 0) || ((need & 2) && s[1] >= 0) ||
                                    ((need & 4) && s[2] >= 0);
                    if (ok) {
                        nei[i] = &s;
                        valid = true;
                    }
                };
                if (vx[0] != vx[1] || vx[0] != vx[2] || vx[0] != vx[4]) find(0, 7);
                if (vx[1] != vx[3] || vx[1] != vx[5]) find(1, 2 | 4);
                if (vx[2] != vx[3] || vx[2] != vx[6]) find(2, 1 | 4);
                if (vx[3] != vx[7]) find(3, 4);
                if (vx[4] != vx[5] || vx[4] != vx[6]) find(4, 1 | 2);
                if (vx[5] != vx[7]) find(5, 2);
                if (vx[6] != vx[7]) find(6, 1);
                const char* plan = kPlans[config];
                const int len = int(std::strlen(plan));
                auto vid = [&](int e) -> int32_t {
                    const auto* s = nei[kEdgeCorner[e]];
                    return s ? (*s)[kEdgeDir[e]] : -1;
                };
                if (nanCorner && valid)
                    for (int k = 0; k < len && valid; ++k) valid = vid(hexDigit(plan[k])) >= 0;
                if (!valid) continue;
                for (int k = 0; k < len; k += 3) {
                    const int32_t a = vid(hexDigit(plan[k])), b = vid(hexDigit(plan[k + 1])),
                                  c = vid(hexDigit(plan[k + 2]));
                    if (lessInside) {
                        R->tris.push_back(a);
                        R->tris.push_back(c);
                        R->tris.push_back(b);
                    } else {
                        R->tris.push_back(a);
                        R->tris.push_back(b);
                        R->tris.push_back(c);
                    }
                    R->faceMap.push_back(int32_t(id));
                }
            }
    return R;
}

int64_t orc_mc_num_points(void* r) { return int64_t(static_cast<McResult*>(r)->points.size() / 3); }
int64_t orc_mc_num_tris(void* r) { return int64_t(static_cast<McResult*>(r)->tris.size() / 3); }
const char* orc_mc_error(void* r) { return static_cast<McResult*>(r)->error.c_str(); }
void orc_mc_get(void* r, float* points, int32_t* tris, int32_t* faceMap) {
    const McResult* R = static_cast<McResult*>(r);
    if (points) std::memcpy(points, R->points.data(), R->points.size() * sizeof(float));
    if (tris) std::memcpy(tris, R->tris.data(), R->tris.size() * sizeof(int32_t));
    if (faceMap) std::memcpy(faceMap, R->faceMap.data(), R->faceMap.size() * sizeof(int32_t));
}
void orc_mc_free(void* r) { delete static_cast<McResult*>(r); }
// the table, for comparison with the product's packed copy
const char* orc_mc_plan(int config) { return config >= 0 && config < 256 ? kPlans[config] : ""; }

}  // extern "C"
