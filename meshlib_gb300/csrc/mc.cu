// Marching cubes over a device-resident volume: the mesher that MeshLib runs on the signed-distance
// grid in mcOffsetMesh (MRVoxels/MROffset.cpp:185-226), i.e. `VolumeMesher` behind
// marchingCubes(SimpleVolume) and MarchingCubesByParts (MRVoxels/MRMarchingCubes.cpp:328-1103).
//
// The output is the reference's TriMesh bit for bit:
//   * a vertex on the +X/+Y/+Z edge of every voxel whose value and the neighbour's lie on opposite
//     sides of iso (v < iso against v >= iso; NaN on either end: no vertex), at
//     (1 - r) p0 + r p1, r = (iso - v0) / (v1 - v0), every operation rounded to float as the
//     reference's uncontracted code does (MRMarchingCubes.cpp:568-575, 610-646);
//   * vertex ids in the order (voxel id, direction): the reference numbers points per z-block in
//     voxel order and shifts the blocks by the counts before them (MRSeparationPoint.cpp:13-35), which
//     is that order whatever the block size;
//   * per cell (the voxel at its min corner, in voxel order) the plan of its 8-corner configuration,
//     NaN corners replaced by their first valid neighbour corner, a cell dropped when it touches
//     NaN and one of its triangle edges has no vertex (MRMarchingCubes.cpp:870-1054); triangle
//     order = cell order, then plan order; lessInside flips the orientation;
//   * coordinates of part k (MarchingCubesByParts) relative to its first layer z0:
//     zeroPoint = origin + (0.5, 0.5, 0.5 + z0) * voxelSize, p = zeroPoint + voxelSize * (x, y, z - z0)
//     (MRMarchingCubes.cpp:566); the whole volume is one part with z0 = 0.
//
// GB300 design: streaming passes, no hash map.  The reference keeps separation points in per-block
// hash maps keyed by voxel id; here one byte per voxel (crossing bits, below-iso bit, NaN bit) and
// two exclusive scans over 16-voxel chunks give every vertex and triangle its global id: the id of
// the vertex on edge `dir` of voxel u is
//   vertBase[chunk(u)] + popc(crossing bits of the chunk's bytes before u) + popc(u's bits below dir),
// one 16-byte load.  A warp works on 32 voxels of one row at a time (a contiguous run of rows per
// warp, no division per voxel); the flag arrays have a row pitch of whole 32-byte segments so that
// chunks are aligned and numbered in voxel order.
//   classifyKernel     flags + vertices per chunk: the one dense pass over the volume, 4 voxels per
//                      lane (float4 loads when rows allow), two 128-voxel segments in flight per warp
//   cellKernel         triangles per cell + per chunk, 4 cells per lane; segments whose four rows
//                      hold no crossing (by the chunk vertex counts) are skipped
//   two scans          chunk bases (exclusiveScanI32)
//   vertexKernel       crossing positions, only where the chunk counts are nonzero
//   collectCellsKernel the cells that emit triangles, as a list
//   triangleKernel     one thread per listed cell: vertex ids and faceMap
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbfwn.h"
#include "common.cuh"
#include "handle.cuh"

namespace gbfwn {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr unsigned kLower = 8u, kInvalid = 16u;  // flag bits; bits 0..2 = crossing on +X/+Y/+Z

// Edge e of a cell: start corner and +direction (MRMarchingCubes.cpp:25-40); corners x + 2y + 4z.
__device__ const uint8_t kEdgeCorner[12] = {0, 1, 2, 0, 4, 5, 6, 4, 0, 1, 3, 2};
__device__ const uint8_t kEdgeDir[12] = {0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2};
// corner -> configuration bit (MRMarchingCubes.cpp:52-65)
__device__ const uint8_t kCornerBit[8] = {0, 1, 3, 2, 4, 5, 7, 6};
// first valid neighbour corner of a NaN corner: i ^ kNanOrder[k] (MRMarchingCubes.cpp:924-932)
__device__ const uint8_t kNanOrder[7] = {1, 2, 4, 3, 5, 6, 7};

// The triangulation table of MRMarchingCubes.cpp:67-323, the same data re-encoded: edge k of plan c
// is nibble k of kPlan[c] (three per triangle, at most five triangles), kPlanTris[c] triangles.
__device__ const unsigned long long kPlan[256] = {
    0x000000000000000ull, 0x000000000000380ull, 0x000000000000910ull, 0x000000000189381ull,
    0x000000000000a21ull, 0x000000000a21380ull, 0x000000000920a29ull, 0x00000089a8a2382ull,
    0x0000000000002b3ull, 0x0000000000b82b0ull, 0x000000000b32091ull, 0x000000b89b912b1ull,
    0x0000000003ab1a3ull, 0x000000ab8a801a0ull, 0x0000009ab9b3093ull, 0x000000000b8aa89ull,
    0x000000000000874ull, 0x000000000437034ull, 0x000000000748910ull, 0x000000137174914ull,
    0x000000000748a21ull, 0x000000a21403743ull, 0x000000748209a29ull, 0x0004973727929a2ull,
    0x0000000002b3748ull, 0x00000040242b74bull, 0x000000b32748109ull, 0x0001292b9b49b74ull,
    0x000000487ab31a3ull, 0x0004b7401b41ab1ull, 0x00030bab9b09874ull, 0x000000ab99b4b74ull,
    0x000000000000459ull, 0x000000000380459ull, 0x000000000051450ull, 0x000000513538458ull,
    0x000000000459a21ull, 0x000000594a21803ull, 0x000000204245a25ull, 0x0008434535235a2ull,
    0x000000000b32459ull, 0x000000594b802b0ull, 0x000000b32510450ull, 0x000584b82852512ull,
    0x00000045931ab3aull, 0x000ab81a8180594ull, 0x00030bab5b05045ull, 0x000000b8aa85845ull,
    0x000000000975879ull, 0x000000375359039ull, 0x000000751710870ull, 0x000000000753351ull,
    0x00000021a759879ull, 0x00037503505921aull, 0x00025a758528208ull, 0x0000007533525a2ull,
    0x0000002b3987597ull, 0x000b72029279759ull, 0x000751871810b32ull, 0x00000051771b12bull,
    0x000b3a31a758859ull, 0x0aba010b7905075ull, 0x07570805a30b0abull, 0x0000000005b75abull,
    0x00000000000056aull, 0x0000000006a5380ull, 0x0000000006a5109ull, 0x0000006a5891381ull,
    0x000000000162561ull, 0x000000803621561ull, 0x000000620609569ull, 0x000823625285895ull,
    0x00000000056ab32ull, 0x00000056a02b80bull, 0x0000006a5b32910ull, 0x000b892b92916a5ull,
    0x000000315356b36ull, 0x0006b51505b0b80ull, 0x0009505606306b3ull, 0x00000089bb96956ull,
    0x0000000008746a5ull, 0x000000a56374034ull, 0x0000007486a5091ull, 0x00049737179156aull,
    0x000000874156216ull, 0x000743403625521ull, 0x000620560509748ull, 0x962695923497937ull,
    0x00000056a4872b3ull, 0x000b720242746a5ull, 0x0006a5b32874910ull, 0x6a54b7b492b9129ull,
    0x0006b51535b3748ull, 0xb404b7b016b5b15ull, 0x74836b630560950ull, 0x0009b7974b96956ull,
    0x000000000a4694aull, 0x000000380a946a4ull, 0x00000004606a10aull, 0x000a16468618138ull,
    0x000000462421941ull, 0x000462942921803ull, 0x000000000624420ull, 0x000000624428238ull,
    0x00000032b46a94aull, 0x0006a4a94b82280ull, 0x000a164606102b3ull, 0x1b8b12184a16146ull,
    0x00036b319639469ull, 0x14641916b0181b8ull, 0x0000004600636b3ull, 0x00000000086b846ull,
    0x000000a98a876a7ull, 0x000a76a907a0370ull, 0x0000818717a176aull, 0x00000037117a76aull,
    0x000768981861621ull, 0x937390976192962ull, 0x000000206607087ull, 0x000000000276237ull,
    0x00076898a86ab32ull, 0x7a9a76790b72702ull, 0xb32a767a1871081ull, 0x00017616a71b12bull,
    0x63136b619768698ull, 0x00000000076b190ull, 0x00006b0b3607087ull, 0x0000000000006b7ull,
    0x000000000000b67ull, 0x00000000067b803ull, 0x00000000067b910ull, 0x00000067b138918ull,
    0x0000000007b621aull, 0x0000007b6803a21ull, 0x0000007b69a2092ull, 0x00089a38a3a27b6ull,
    0x000000000726327ull, 0x000000026067807ull, 0x000000910732672ull, 0x000678891681261ull,
    0x00000073171a67aull, 0x000801781a7167aull, 0x0007a69a0a70730ull, 0x0000009a88a7a67ull,
    0x00000000068b486ull, 0x000000640603b63ull, 0x000000109648b68ull, 0x00063b139369649ull,
    0x0000001a28b6486ull, 0x000640b60b03a21ull, 0x0009a2920b648b4ull, 0x36463b34923a39aull,
    0x000000264248328ull, 0x000000000264240ull, 0x000834642432091ull, 0x000000642241491ull,
    0x0001a6648168318ull, 0x00000040660a01aull, 0x39a9303a6834364ull, 0x0000000004a649aull,
    0x000000000b67594ull, 0x00000067b594380ull, 0x000000b67045105ull, 0x00051345343867bull,
    0x000000b6721a459ull, 0x000594380a217b6ull, 0x000204a24a45b67ull, 0x67b25a523453843ull,
    0x000000945267327ull, 0x000786260680459ull, 0x000045051673263ull, 0x851584812786826ull,
    0x00073167161a459ull, 0x459078701671a61ull, 0xa737a6a305a4a04ull, 0x000a84a458a7a67ull,
    0x00000098b9b6596ull, 0x000590650360b63ull, 0x000b65510b508b0ull, 0x0000001355363b6ull,
    0x00065b8b9b59a21ull, 0xa21965690b603b0ull, 0x52025a50865b58bull, 0x00035a3a25363b6ull,
    0x000283265825985ull, 0x000000260069659ull, 0x826283865081851ull, 0x000000000612651ull,
    0x698965683a61631ull, 0x00006505960a01aull, 0x000000000a65830ull, 0x00000000000065aull,
    0x000000000b57a5bull, 0x00000003857ba5bull, 0x000000091ba57b5ull, 0x0001381897ba57aull,
    0x00000015717b21bull, 0x000b27571721380ull, 0x0007b2209729579ull, 0x289823295b27257ull,
    0x000000573532a52ull, 0x00052a578258028ull, 0x0002a37353a5109ull, 0x25752a278129289ull,
    0x000000000573531ull, 0x000000571170780ull, 0x000000735539309ull, 0x000000000795789ull,
    0x0000008ba8a5485ull, 0x00003bba50b5405ull, 0x00054aba8a48910ull, 0x41314943b54a4baull,
    0x0008548b2582152ull, 0xb151b2b543b0b40ull, 0x58b8545b2950520ull, 0x0000000003b2549ull,
    0x000483543253a52ull, 0x0000000244252a5ull, 0x910854583a532a3ull, 0x0002492914252a5ull,
    0x000000153358548ull, 0x000000000501540ull, 0x000530509358548ull, 0x000000000000549ull,
    0x000000ba9b947b4ull, 0x000ba97b9794380ull, 0x000b470414b1ba1ull, 0x4bab474a1843413ull,
    0x000219b294b97b4ull, 0x3801b2b197b9479ull, 0x00000004224b47bull, 0x00042343824b47bull,
    0x000947732972a92ull, 0x70207872a4797a9ull, 0xa040a1a472a3a73ull, 0x0000000004782a1ull,
    0x000000317714194ull, 0x000178180714194ull, 0x000000000347304ull, 0x000000000000784ull,
    0x0000000008ba8a9ull, 0x000000a9bb93903ull, 0x000000ba88a0a10ull, 0x000000000a3ba13ull,
    0x0000008b99b1b21ull, 0x0009b2921b93903ull, 0x000000000b08b20ull, 0x000000000000b23ull,
    0x00000098aa82832ull, 0x0000000002902a9ull, 0x0008a1810a82832ull, 0x0000000000002a1ull,
    0x000000000819831ull, 0x000000000000190ull, 0x000000000000830ull, 0x000000000000000ull,};
__device__ const uint8_t kPlanTris[256] = {
    0, 1, 1, 2, 1, 2, 2, 3, 1, 2, 2, 3, 2, 3, 3, 2, 1, 2, 2, 3, 2, 3, 3, 4, 2, 3, 3, 4, 3, 4, 4, 3,
    1, 2, 2, 3, 2, 3, 3, 4, 2, 3, 3, 4, 3, 4, 4, 3, 2, 3, 3, 2, 3, 4, 4, 3, 3, 4, 4, 3, 4, 5, 5, 2,
    1, 2, 2, 3, 2, 3, 3, 4, 2, 3, 3, 4, 3, 4, 4, 3, 2, 3, 3, 4, 3, 4, 4, 5, 3, 4, 4, 5, 4, 5, 5, 4,
    2, 3, 3, 4, 3, 4, 2, 3, 3, 4, 4, 5, 4, 5, 3, 2, 3, 4, 4, 3, 4, 5, 3, 2, 4, 5, 5, 4, 5, 2, 4, 1,
    1, 2, 2, 3, 2, 3, 3, 4, 2, 3, 3, 4, 3, 4, 4, 3, 2, 3, 3, 4, 3, 4, 4, 5, 3, 2, 4, 3, 4, 3, 5, 2,
    2, 3, 3, 4, 3, 4, 4, 5, 3, 4, 4, 5, 4, 5, 5, 4, 3, 4, 4, 3, 4, 5, 5, 4, 4, 3, 5, 2, 5, 4, 2, 1,
    2, 3, 3, 4, 3, 4, 4, 5, 3, 4, 4, 5, 2, 3, 3, 2, 3, 4, 4, 5, 4, 5, 5, 2, 4, 3, 5, 4, 3, 2, 4, 1,
    3, 4, 4, 5, 4, 5, 3, 4, 4, 5, 5, 2, 3, 4, 2, 1, 2, 3, 3, 2, 3, 4, 2, 1, 3, 2, 4, 1, 2, 1, 1, 0,};

struct McDims {
    int32_t dx, dy, dz;
    int64_t sxy;     // dx * dy
    int64_t rows;    // dy * dz
    int32_t xsegs;   // 32-voxel segments per row
    int32_t pitch;   // bytes per row of the flag arrays (xsegs * 32)
    int64_t items;   // rows * xsegs warp work items
    int64_t nChunks; // rows * pitch / 16
    int32_t qsegs;   // 128-voxel segments per row (the classification's work items, 4 voxels per lane)
    int64_t qitems;  // rows * qsegs
};

struct McGeom {
    float zpx, zpy;  // zeroPoint.x, .y
    float vs[3];
    float iso;
};

// A warp work item is 32 consecutive voxels of one row (x fastest): lane = x % 32.  Flag arrays are
// stored with a row pitch of whole 32-byte segments, so every 16-voxel chunk is 16-byte aligned and
// chunks are numbered in voxel order (row-major, then x).  Each warp walks a contiguous run of items
// with an incrementing cursor (no division per item).
struct WarpItem {
    int x, y, z;
    int64_t row;
    bool in;  // x < dx
};

// The contiguous run of items [w0, w1) of this warp out of `items`.
__device__ __forceinline__ void warpRange(int64_t items, int64_t& w0, int64_t& w1) {
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    const int64_t gw = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t per = (items + nw - 1) / nw;
    w0 = gw * per;
    w1 = min(w0 + per, items);
}

// Position of item w (divisions: used once per run, or for the few items a sparse pass visits).
struct Cursor {
    int64_t row;
    int seg, y, z;
    int segs;  // segments per row
    __device__ __forceinline__ void init(const McDims& d, int64_t w, int segsPerRow = 0) {
        segs = segsPerRow ? segsPerRow : d.xsegs;
        row = w / segs;
        seg = int(w - row * segs);
        z = int(row / d.dy);
        y = int(row - int64_t(z) * d.dy);
    }
    __device__ __forceinline__ WarpItem item(const McDims& d, int lane) const {
        WarpItem it;
        it.row = row;
        it.y = y;
        it.z = z;
        it.x = seg * 32 + lane;
        it.in = it.x < d.dx;
        return it;
    }
    __device__ __forceinline__ void advance(const McDims& d) {
        if (++seg == segs) {
            seg = 0;
            ++row;
            if (++y == d.dy) {
                y = 0;
                ++z;
            }
        }
    }
};

// Visits the items of this warp whose two 16-voxel chunks are not both empty by `counts`
// (chunk c of item w is 2w + c): 32 counts per load, a ballot, then only the marked items.
template <typename F>
__device__ __forceinline__ void forEachMarkedItem(const McDims& d, int lane, const int32_t* __restrict__ counts, F&& body) {
    int64_t w0, w1;
    warpRange(d.items, w0, w1);
    for (int64_t g = w0; g < w1; g += 16) {
        const int64_t ch = 2 * g + lane;
        const int cnt = ch < 2 * w1 ? counts[ch] : 0;
        unsigned m = __ballot_sync(FULL, cnt != 0);
        while (m) {
            const int k = (__ffs(m) - 1) >> 1;
            m &= ~(3u << (2 * k));
            Cursor c;
            c.init(d, g + k);
            body(c.item(d, lane));
        }
    }
}

// exclusive prefix of c over the lanes of the chunk before this one
__device__ __forceinline__ int chunkExclusive(int c, int lane) {
    int p = c;
#pragma unroll
    for (int off = 1; off < 16; off <<= 1) {
        const int t = __shfl_up_sync(FULL, p, off, 16);
        if ((lane & 15) >= off) p += t;
    }
    return p - c;
}

// Flag byte of one voxel from its value and its +X/+Y/+Z neighbours' (MRMarchingCubes.cpp:598-646):
// a crossing needs the neighbour on the other side of iso; a NaN neighbour is on neither side.
__device__ __forceinline__ unsigned voxelFlags(float v, float nx, float ny, float nz, bool hx, bool hy, bool hz, float iso) {
    const bool lower = v < iso, notLower = v >= iso;
    if (!lower && !notLower) return kInvalid;
    unsigned f = lower ? kLower : 0u;
    if (hx && (lower ? nx >= iso : nx < iso)) f |= 1u;
    if (hy && (lower ? ny >= iso : ny < iso)) f |= 2u;
    if (hz && (lower ? nz >= iso : nz < iso)) f |= 4u;
    return f;
}

constexpr int kClassifyUnroll = 2;  // 128-voxel segments in flight per warp

// The dense pass: each lane classifies 4 consecutive voxels of a row (a warp 128) and stores their
// flags as one 32-bit word; 16-voxel chunk counts are sums over groups of 4 lanes.  VEC: the
// volume is 16-byte aligned and dx % 4 == 0, so the loads are float4.
template <bool VEC>
__global__ void __launch_bounds__(256, 4) classifyKernel(const float* __restrict__ vol, McDims d, float iso,
                                                         uint8_t* __restrict__ flags, int32_t* __restrict__ chunkVerts,
                                                         unsigned long long* __restrict__ total) {
    const int lane = threadIdx.x & 31;
    unsigned long long mine = 0;
    int64_t w0, w1;
    warpRange(d.qitems, w0, w1);
    Cursor cur;
    if (w0 < w1) cur.init(d, w0, d.qsegs);
    for (int64_t w = w0; w < w1; w += kClassifyUnroll) {
        int x[kClassifyUnroll], y[kClassifyUnroll], z[kClassifyUnroll];
        int64_t row[kClassifyUnroll];
        float v[kClassifyUnroll][5], ny[kClassifyUnroll][4], nz[kClassifyUnroll][4];
        // all loads of the group first: they do not depend on one another
#pragma unroll
        for (int k = 0; k < kClassifyUnroll; ++k) {
            x[k] = cur.seg * 128 + 4 * lane;
            y[k] = cur.y;
            z[k] = cur.z;
            row[k] = cur.row;
            cur.advance(d);
            const bool ok = w + k < w1;
            const int64_t id = row[k] * d.dx + x[k];
            const bool hy = y[k] + 1 < d.dy, hz = z[k] + 1 < d.dz;
            if (VEC && ok && x[k] < d.dx) {  // x % 4 == 0 and dx % 4 == 0: all four in the row
                const float4 a = __ldg(reinterpret_cast<const float4*>(vol + id));
                v[k][0] = a.x; v[k][1] = a.y; v[k][2] = a.z; v[k][3] = a.w;
                v[k][4] = x[k] + 4 < d.dx ? vol[id + 4] : 0.f;
                const float4 b = hy ? __ldg(reinterpret_cast<const float4*>(vol + id + d.dx)) : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 c = hz ? __ldg(reinterpret_cast<const float4*>(vol + id + d.sxy)) : make_float4(0.f, 0.f, 0.f, 0.f);
                ny[k][0] = b.x; ny[k][1] = b.y; ny[k][2] = b.z; ny[k][3] = b.w;
                nz[k][0] = c.x; nz[k][1] = c.y; nz[k][2] = c.z; nz[k][3] = c.w;
            } else {
#pragma unroll
                for (int j = 0; j < 5; ++j) v[k][j] = ok && x[k] + j < d.dx ? vol[id + j] : 0.f;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    ny[k][j] = ok && hy && x[k] + j < d.dx ? vol[id + d.dx + j] : 0.f;
                    nz[k][j] = ok && hz && x[k] + j < d.dx ? vol[id + d.sxy + j] : 0.f;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kClassifyUnroll; ++k) {
            if (w + k >= w1) break;  // warp-uniform
            const bool hy = y[k] + 1 < d.dy, hz = z[k] + 1 < d.dz;
            unsigned word = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (x[k] + j < d.dx)
                    word |= voxelFlags(v[k][j], v[k][j + 1], ny[k][j], nz[k][j], x[k] + j + 1 < d.dx, hy, hz, iso) << (8 * j);
            const int64_t at = row[k] * d.pitch + x[k];
            if (x[k] < d.pitch) reinterpret_cast<uint32_t*>(flags)[at >> 2] = word;
            const int c = __popc(word & 0x07070707u);
            int sum = c + __shfl_xor_sync(FULL, c, 1);
            sum += __shfl_xor_sync(FULL, sum, 2);
            if ((lane & 3) == 0 && x[k] < d.pitch) chunkVerts[at >> 4] = sum;
            mine += c;
        }
    }
    for (int off = 16; off; off >>= 1) mine += __shfl_xor_sync(FULL, mine, off);
    if (lane == 0 && mine) atomicAdd(total, mine);
}

struct CellInfo {
    int config;
    unsigned nei;    // bit i: corner i's separation points may be used (the reference's neis[i] != null)
    unsigned cross;  // crossing bits of corners 0..6, three per corner
};

// offset of corner c of a cell in the pitched flag arrays
__device__ __forceinline__ int64_t cornerOffset(const McDims& d, int c) {
    return int64_t(c & 1) + ((c >> 1) & 1) * int64_t(d.pitch) + ((c >> 2) & 1) * int64_t(d.pitch) * d.dy;
}

// Configuration, neighbour set and triangle count of a cell from the flag bytes of its 8 corners
// (corner i = byte i of c0123 | c4567 << 32) (MRMarchingCubes.cpp:880-1054).  Returns 0 when the cell
// emits nothing.  Corner states are kept as bit masks (bit i = corner i): nothing is indexed at
// run time.
__device__ __forceinline__ int cellCore(unsigned long long corners, CellInfo& ci) {
    unsigned inv = 0, low = 0, cross = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const unsigned f = unsigned(corners >> (8 * i)) & 0xffu;
        inv |= ((f >> 4) & 1u) << i;
        low |= ((f >> 3) & 1u) << i;
        if (i < 7) cross |= (f & 7u) << (3 * i);
    }
    if (inv == 0xffu) return 0;
    if (inv) {
        // a NaN corner takes the side of its first valid neighbour corner (x, y, z, xy, xz, yz, xyz)
        unsigned sub = low;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            if (!((inv >> i) & 1u)) continue;
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const int j = i ^ kNanOrder[k];
                if (!((inv >> j) & 1u)) {
                    sub = (sub & ~(1u << i)) | (((low >> j) & 1u) << i);
                    break;
                }
            }
        }
        low = sub;
    }
    if (low == 0u || low == 0xffu) return 0;
    int config = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i)
        if ((low >> i) & 1u) config |= 1 << kCornerBit[i];
    auto vx = [low](int i) { return (low >> i) & 1u; };
    auto has = [cross](int i, unsigned dirs) { return ((cross >> (3 * i)) & dirs) != 0u; };
    // corner i contributes when its edges inside the cell change sign and its voxel has a point on
    // one of them (the reference's findNei conditions)
    unsigned nei = 0;
    if ((vx(0) != vx(1) || vx(0) != vx(2) || vx(0) != vx(4)) && has(0, 7u)) nei |= 1u;
    if ((vx(1) != vx(3) || vx(1) != vx(5)) && has(1, 6u)) nei |= 2u;
    if ((vx(2) != vx(3) || vx(2) != vx(6)) && has(2, 5u)) nei |= 4u;
    if (vx(3) != vx(7) && has(3, 4u)) nei |= 8u;
    if ((vx(4) != vx(5) || vx(4) != vx(6)) && has(4, 3u)) nei |= 16u;
    if (vx(5) != vx(7) && has(5, 2u)) nei |= 32u;
    if (vx(6) != vx(7) && has(6, 1u)) nei |= 64u;
    if (!nei) return 0;
    const int nt = kPlanTris[config];
    if (inv) {  // a cell touching NaN needs a vertex on every edge of its plan
        const unsigned long long plan = kPlan[config];
        for (int k = 0; k < 3 * nt; ++k) {
            const int e = int((plan >> (4 * k)) & 15u);
            const int c = kEdgeCorner[e];
            if (!((nei >> c) & 1u) || !((cross >> (3 * c + kEdgeDir[e])) & 1u)) return 0;
        }
    }
    ci.config = config;
    ci.nei = nei;
    ci.cross = cross;
    return nt;
}

// The same for the cell whose min corner sits at `at` in the pitched flag array (8 loads).
__device__ __forceinline__ int cellTriangles(const uint8_t* __restrict__ flags, const McDims& d, int64_t at, CellInfo& ci) {
    unsigned long long corners = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) corners |= (unsigned long long)flags[at + cornerOffset(d, i)] << (8 * i);
    return cellCore(corners, ci);
}

// Triangle counts per cell, 4 cells per lane (a warp: 128 cells of a row).  The warp first checks
// the vertex counts of the 16-voxel chunks its cells touch (8 chunks and the next one in each of the
// four rows): with no crossing there, no cell can emit a triangle (a triangle needs a vertex on one
// of its cell's corners) and only the chunk counts are written.  Otherwise each lane reads its four
// flag bytes in each of the four rows as one word; the +x corner of its last cell comes from the next
// lane (lane 31 reads one more byte).
__global__ void __launch_bounds__(256) cellKernel(const uint8_t* __restrict__ flags, const int32_t* __restrict__ chunkVerts,
                                                  McDims d, uint8_t* __restrict__ tcnt, int32_t* __restrict__ chunkTris,
                                                  unsigned long long* __restrict__ total) {
    __shared__ unsigned long long sCorners[8][128];  // per warp: corner bytes of its candidate cells
    __shared__ uint8_t sCounts[8][128];
    const int lane = threadIdx.x & 31;
    unsigned long long mine = 0;
    const int64_t layer = int64_t(d.pitch) * d.dy;
    int64_t w0, w1;
    warpRange(d.qitems, w0, w1);
    Cursor cur;
    if (w0 < w1) cur.init(d, w0, d.qsegs);
    for (int64_t w = w0; w < w1; ++w, cur.advance(d)) {
        const int x0 = cur.seg * 128, x = x0 + 4 * lane;
        const int64_t at = cur.row * d.pitch + x;
        const bool hy = cur.y + 1 < d.dy, hz = cur.z + 1 < d.dz;
        {
            const int r = lane >> 3, k = lane & 7;
            int cnt = 0;
            if (((r & 1) == 0 || hy) && ((r & 2) == 0 || hz)) {
                const int64_t rr = cur.row + (r & 1) + ((r & 2) ? d.dy : 0);
                const int64_t c0 = (rr * d.pitch + x0) >> 4;
                if (x0 + 16 * k < d.pitch) cnt = chunkVerts[c0 + k];
                if (k == 7 && x0 + 128 < d.pitch) cnt |= chunkVerts[c0 + 8];
            }
            if (!__any_sync(FULL, cnt != 0)) {
                if ((lane & 3) == 0 && x < d.pitch) chunkTris[at >> 4] = 0;
                continue;
            }
        }
        const bool inRow = x < d.pitch;
        const uint32_t* fw = reinterpret_cast<const uint32_t*>(flags);
        const unsigned f0 = inRow ? fw[at >> 2] : 0u;
        const unsigned f1 = inRow && hy ? fw[(at + d.pitch) >> 2] : 0u;
        const unsigned f2 = inRow && hz ? fw[(at + layer) >> 2] : 0u;
        const unsigned f3 = inRow && hy && hz ? fw[(at + d.pitch + layer) >> 2] : 0u;
        unsigned n0 = __shfl_down_sync(FULL, f0, 1) & 0xffu, n1 = __shfl_down_sync(FULL, f1, 1) & 0xffu;
        unsigned n2 = __shfl_down_sync(FULL, f2, 1) & 0xffu, n3 = __shfl_down_sync(FULL, f3, 1) & 0xffu;
        if (lane == 31) {  // x + 4 starts the next segment of the same row
            const bool nx = x + 4 < d.pitch;
            n0 = nx ? flags[at + 4] : 0u;
            n1 = nx && hy ? flags[at + d.pitch + 4] : 0u;
            n2 = nx && hz ? flags[at + layer + 4] : 0u;
            n3 = nx && hy && hz ? flags[at + d.pitch + layer + 4] : 0u;
        }
        // row words extended by the next byte: byte j and j + 1 of row r are cell j's corners
        const unsigned long long e0 = f0 | ((unsigned long long)n0 << 32), e1 = f1 | ((unsigned long long)n1 << 32);
        const unsigned long long e2 = f2 | ((unsigned long long)n2 << 32), e3 = f3 | ((unsigned long long)n3 << 32);
        // candidate cells (a corner with a crossing) of this lane, then spread over the warp: lane l
        // evaluates candidates l, l + 32, ... of the warp's list in shared memory, so a run of surface
        // cells held by a few lanes does not serialise their evaluations
        unsigned cand = 0;
        unsigned long long corners[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const unsigned b0 = unsigned(e0 >> (8 * j)) & 0xffffu, b1 = unsigned(e1 >> (8 * j)) & 0xffffu;
            const unsigned b2 = unsigned(e2 >> (8 * j)) & 0xffffu, b3 = unsigned(e3 >> (8 * j)) & 0xffffu;
            corners[j] = (unsigned long long)(b0 | (b1 << 16)) | ((unsigned long long)(b2 | (b3 << 16)) << 32);
            if (x + j + 1 < d.dx && hy && hz && ((b0 | b1 | b2 | b3) & 0x0707u)) cand |= 1u << j;
        }
        const int nc = __popc(cand);
        int excl = nc;  // exclusive prefix of the candidate counts over the lanes
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int t = __shfl_up_sync(FULL, excl, off);
            if (lane >= off) excl += t;
        }
        const int totalC = __shfl_sync(FULL, excl, 31);
        excl -= nc;
        unsigned long long* slots = sCorners[threadIdx.x >> 5];
        uint8_t* counts = sCounts[threadIdx.x >> 5];
        {
            int k = excl;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if ((cand >> j) & 1u) slots[k++] = corners[j];
        }
        __syncwarp();
        for (int g = lane; g < totalC; g += 32) {
            CellInfo ci;
            counts[g] = uint8_t(cellCore(slots[g], ci));
        }
        __syncwarp();
        unsigned word = 0;
        int c = 0;
        {
            int k = excl;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if ((cand >> j) & 1u) {
                    const int nt = counts[k++];
                    word |= unsigned(nt) << (8 * j);
                    c += nt;
                }
        }
        __syncwarp();  // the slots are rewritten by the next item
        if (inRow) reinterpret_cast<uint32_t*>(tcnt)[at >> 2] = word;
        int sum = c + __shfl_xor_sync(FULL, c, 1);
        sum += __shfl_xor_sync(FULL, sum, 2);
        if ((lane & 3) == 0 && inRow) chunkTris[at >> 4] = sum;
        mine += c;
    }
    for (int off = 16; off; off >>= 1) mine += __shfl_xor_sync(FULL, mine, off);
    if (lane == 0 && mine) atomicAdd(total, mine);
}

// Crossing positions: only the items whose chunks hold vertices.
__global__ void __launch_bounds__(256) vertexKernel(const float* __restrict__ vol, const uint8_t* __restrict__ flags,
                                                    const int32_t* __restrict__ chunkVerts, const int32_t* __restrict__ vertBase,
                                                    McDims d, McGeom g, const float* __restrict__ layerZ,
                                                    float* __restrict__ points) {
    const int lane = threadIdx.x & 31;
    forEachMarkedItem(d, lane, chunkVerts, [&](const WarpItem& it) {
        const int64_t at = it.row * d.pitch + it.x;
        const unsigned f = flags[at];  // 0 past the row end
        const int c = __popc(f & 7u);
        const int ex = chunkExclusive(c, lane);
        if (!c) return;
        int64_t v = int64_t(vertBase[at >> 4]) + ex;
        const int64_t id = it.row * d.dx + it.x;
        const float v0 = vol[id];
        const float p0[3] = {__fadd_rn(g.zpx, __fmul_rn(g.vs[0], float(it.x))),
                             __fadd_rn(g.zpy, __fmul_rn(g.vs[1], float(it.y))), layerZ[it.z]};
        const int64_t inc[3] = {1, d.dx, d.sxy};
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            if (!((f >> n) & 1u)) continue;
            const float v1 = vol[id + inc[n]];
            const float r = __fdiv_rn(__fsub_rn(g.iso, v0), __fsub_rn(v1, v0));
            const float wgt = __fsub_rn(1.0f, r);
            float p1[3] = {p0[0], p0[1], p0[2]};
            p1[n] = __fadd_rn(p0[n], g.vs[n]);
            float* o = points + 3 * v;
#pragma unroll
            for (int k = 0; k < 3; ++k) o[k] = __fadd_rn(__fmul_rn(wgt, p0[k]), __fmul_rn(r, p1[k]));
            ++v;
        }
    });
}

// Global id of the vertex on edge `dir` of the voxel at `at` in the pitched flag array (which has it):
// its chunk's base + the crossings of the chunk's voxels before it + its own below `dir`.
__device__ __forceinline__ int32_t vertexId(const uint8_t* __restrict__ flags, const int32_t* __restrict__ vertBase, int64_t at,
                                            int dir) {
    const int64_t chunk = at >> 4;
    const uint4 w = __ldg(reinterpret_cast<const uint4*>(flags) + chunk);
    const int j = int(at & 15);
    const unsigned words[4] = {w.x, w.y, w.z, w.w};
    int p = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int nb = min(max(j - 4 * q, 0), 4);  // bytes of this word before the voxel
        const unsigned m = nb >= 4 ? 0x07070707u : (0x07070707u & ((1u << (8 * nb)) - 1u));
        p += __popc(words[q] & m);
    }
    const unsigned own = (words[j >> 2] >> (8 * (j & 3))) & 0xffu;
    p += __popc(own & ((1u << dir) - 1u));
    return vertBase[chunk] + p;
}

// Positions (in the pitched arrays) of the cells that emit triangles, in any order: a warp counts
// the nonzero cells of its marked items, reserves that many slots with one atomic, then writes them.
__global__ void __launch_bounds__(256) collectCellsKernel(const uint8_t* __restrict__ tcnt, const int32_t* __restrict__ chunkTris,
                                                          McDims d, int64_t* __restrict__ cells,
                                                          unsigned long long* __restrict__ count) {
    const int lane = threadIdx.x & 31;
    unsigned n = 0;
    forEachMarkedItem(d, lane, chunkTris, [&](const WarpItem& it) {
        n += __popc(__ballot_sync(FULL, tcnt[it.row * d.pitch + it.x] != 0));
    });
    unsigned long long base = 0;
    if (lane == 0 && n) base = atomicAdd(count, (unsigned long long)n);
    base = __shfl_sync(FULL, base, 0);
    forEachMarkedItem(d, lane, chunkTris, [&](const WarpItem& it) {
        const int64_t at = it.row * d.pitch + it.x;
        const bool has = tcnt[at] != 0;
        const unsigned m = __ballot_sync(FULL, has);
        if (has) cells[base + __popc(m & ((1u << lane) - 1u))] = at;
        base += __popc(m);
    });
}

// sum of the bytes of w before byte j (values < 64, so no carries between bytes)
__device__ __forceinline__ unsigned bytesBefore(unsigned w, int j) {
    const unsigned m = j >= 4 ? 0xffffffffu : ((1u << (8 * j)) - 1u);
    return ((w & m) * 0x01010101u) >> 24;
}

// Triangles, one thread per listed cell: its first triangle id = the chunk's base + the counts of
// the chunk's cells before it; then the plan's vertex ids and the face map.
__global__ void __launch_bounds__(256) triangleKernel(const uint8_t* __restrict__ flags, const uint8_t* __restrict__ tcnt,
                                                      const int64_t* __restrict__ cells,
                                                      const unsigned long long* __restrict__ cellCount,
                                                      const int32_t* __restrict__ vertBase, const int32_t* __restrict__ triBase,
                                                      McDims d, int lessInside, int32_t* __restrict__ tris,
                                                      int32_t* __restrict__ faceMap) {
    const int64_t nCells = int64_t(*cellCount);
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nCells; i += int64_t(gridDim.x) * blockDim.x) {
        const int64_t at = cells[i];
        const uint4 w = __ldg(reinterpret_cast<const uint4*>(tcnt) + (at >> 4));
        const int j = int(at & 15);
        const unsigned before = bytesBefore(w.x, j) + bytesBefore(w.y, j - 4 < 0 ? 0 : j - 4) +
                                bytesBefore(w.z, j - 8 < 0 ? 0 : j - 8) + bytesBefore(w.w, j - 12 < 0 ? 0 : j - 12);
        int64_t base = int64_t(triBase[at >> 4]) + before;
        CellInfo ci;
        const int nt = cellTriangles(flags, d, at, ci);
        const unsigned long long plan = kPlan[ci.config];
        const int64_t row = at / d.pitch;
        const int32_t voxel = faceMap ? int32_t(row * d.dx + (at - row * d.pitch)) : 0;
        for (int k = 0; k < nt; ++k, ++base) {
            int32_t ids[3];
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                const int e = int((plan >> (4 * (3 * k + m))) & 15u);
                ids[m] = vertexId(flags, vertBase, at + cornerOffset(d, kEdgeCorner[e]), kEdgeDir[e]);
            }
            int32_t* o = tris + 3 * base;
            o[0] = ids[0];
            o[1] = lessInside ? ids[2] : ids[1];
            o[2] = lessInside ? ids[1] : ids[2];
            if (faceMap) faceMap[base] = voxel;
        }
    }
}

}  // namespace
}  // namespace gbfwn

struct gbfwn_trimesh_s {
    int device = 0;
    float* dPoints = nullptr;
    int32_t* dTris = nullptr;
    int32_t* dFaceMap = nullptr;
    int64_t nPoints = 0, nTris = 0;
    ~gbfwn_trimesh_s() {
        gbfwn::DeviceGuard g(device);
        if (dPoints || dTris || dFaceMap) cudaDeviceSynchronize();  // as cudaFree would: no use in flight
        gbfwn::poolFree(dPoints, nullptr);
        gbfwn::poolFree(dTris, nullptr);
        gbfwn::poolFree(dFaceMap, nullptr);
    }
};

struct gbfwn_mc_parts_s {
    int device = 0;
    int32_t dims[3] = {0, 0, 0};
    gbfwn_mc_params params{};
    float* dVol = nullptr;
    int32_t nextZ = 0;
    std::vector<int32_t> starts;
    cudaStream_t stream = nullptr;
    ~gbfwn_mc_parts_s() {
        gbfwn::DeviceGuard g(device);
        if (dVol) cudaDeviceSynchronize();
        gbfwn::poolFree(dVol, stream);
        if (stream) cudaStreamSynchronize(stream);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace gbfwn {
namespace {

int mcError(const char* msg) { return fail(GBFWN_INVALID, msg); }

// Work arrays of the mesher (about 3 bytes per voxel), kept per device between calls so that repeated
// meshing does not pay for cudaMalloc / cudaFree of hundreds of MB; it only grows, and
// gbfwn_mc_release_workspace frees it.
struct McWorkspace {
    std::mutex mu;
    char* buf = nullptr;  // flags, counts, bases, scan scratch, totals, layer z
    size_t cap = 0;
    char* cells = nullptr;  // list of the cells that emit triangles
    size_t cellCap = 0;
    static cudaError_t grow(char*& p, size_t& c, size_t bytes) {
        if (c >= bytes) return cudaSuccess;
        cudaFree(p);
        p = nullptr;
        c = 0;
        cudaError_t e = devMalloc((void**)&p, bytes);
        if (!e) c = bytes;
        return e;
    }
    cudaError_t ensure(size_t bytes) { return grow(buf, cap, bytes); }
    cudaError_t ensureCells(size_t bytes) { return grow(cells, cellCap, bytes); }
};
constexpr int kMaxDevices = 64;
McWorkspace g_workspaces[kMaxDevices];
McWorkspace& workspace(int device) { return g_workspaces[unsigned(device) % kMaxDevices]; }

// Checks the part layout the way MarchingCubesByParts::addPart / finalize do
// (MRMarchingCubes.cpp:436-441, 816-817) and returns the z coordinate of every layer.
int layerCoords(const int32_t dims[3], const gbfwn_mc_params& p, const int32_t* partStarts, int32_t nParts,
                std::vector<float>& lz) {
    std::vector<int32_t> starts;
    if (nParts <= 0)
        starts.push_back(0);
    else
        starts.assign(partStarts, partStarts + nParts);
    if (starts[0] != 0) return mcError("a part exceeds whole volume in Z dimension");
    for (size_t k = 0; k < starts.size(); ++k) {
        const int32_t last = k + 1 < starts.size() ? starts[k + 1] : dims[2] - 1;
        if (last - starts[k] + 1 <= 1) return mcError("a part must have at least two Z slices");
        if (last > dims[2] - 1) return mcError("a part exceeds whole volume in Z dimension");
    }
    lz.resize(size_t(dims[2]));
    size_t k = 0;
    for (int32_t z = 0; z < dims[2]; ++z) {
        while (k + 1 < starts.size() && z >= starts[k + 1]) ++k;
        const int32_t z0 = starts[k];
        // zeroPoint.z = origin.z + (0.5 + z0) * voxelSize.z;  p.z = zeroPoint.z + voxelSize.z * (z - z0)
        const float zp = p.origin[2] + (0.5f + float(z0)) * p.voxelSize[2];
        lz[size_t(z)] = zp + p.voxelSize[2] * float(z - z0);
    }
    return GBFWN_OK;
}

// Blocks of 256 threads: 8 per SM (a one-wave grid sized by occupancy measured no faster), fewer
// for small volumes.
unsigned mcBlocks(const McDims& d) {
    const int64_t want = (d.items + 7) / 8;  // 8 warps per block
    return unsigned(std::max<int64_t>(1, std::min<int64_t>(want, int64_t(numSMs()) * 8)));
}

McDims mcDims(const int32_t dims[3]) {
    McDims d;
    d.dx = dims[0];
    d.dy = dims[1];
    d.dz = dims[2];
    d.sxy = int64_t(dims[0]) * dims[1];
    d.rows = int64_t(dims[1]) * dims[2];
    d.xsegs = (dims[0] + 31) / 32;
    d.pitch = d.xsegs * 32;
    d.items = d.rows * d.xsegs;
    d.nChunks = d.rows * d.pitch / 16;
    d.qsegs = (dims[0] + 127) / 128;
    d.qitems = d.rows * d.qsegs;
    return d;
}

// Bytes of the mesher's work arrays: flags, triangle counts, chunk counts and bases, scan
// scratch, totals, layer z coordinates.
void mcSizes(const McDims& d, size_t sizes[10]) {
    const int64_t nbSums = (d.nChunks + 1023) / 1024 + 1;
    const size_t flagBytes = size_t(d.rows) * size_t(d.pitch) + 16;
    const size_t list[10] = {flagBytes,
                             flagBytes,
                             sizeof(int32_t) * size_t(d.nChunks),
                             sizeof(int32_t) * size_t(d.nChunks),
                             sizeof(int32_t) * size_t(d.nChunks),
                             sizeof(int32_t) * size_t(d.nChunks),
                             sizeof(int32_t) * size_t(nbSums),
                             sizeof(int32_t) * 4,
                             sizeof(unsigned long long) * 3,
                             sizeof(float) * size_t(d.dz)};
    for (int k = 0; k < 10; ++k) sizes[k] = list[k];
}

size_t mcWorkspaceBytes(const McDims& d) {
    size_t sizes[10], need = 0;
    mcSizes(d, sizes);
    for (size_t b : sizes) need += (b + 255) / 256 * 256;
    return need;
}

// The mesher on a device volume; the result is complete when this returns.
int runMarchingCubes(const float* dVol, const int32_t dims[3], const gbfwn_mc_params& p, const int32_t* partStarts,
                     int32_t nParts, int device, cudaStream_t s, gbfwn_trimesh* out, const char* what) {
    auto* m = new gbfwn_trimesh_s;
    m->device = device;
    *out = nullptr;
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) {  // VolumeMesher::run: empty mesh
        *out = m;
        return GBFWN_OK;
    }
    std::vector<float> lz;
    int st = layerCoords(dims, p, partStarts, nParts, lz);
    if (st) {
        delete m;
        return st;
    }
    const McDims d = mcDims(dims);
    if (p.wantFaceMap && d.sxy * dims[2] > INT32_MAX) {
        delete m;
        return mcError("voxel ids of the face map exceed 32 bits");
    }
    McGeom g;
    g.zpx = p.origin[0] + 0.5f * p.voxelSize[0];  // host code is compiled without FMA contraction
    g.zpy = p.origin[1] + 0.5f * p.voxelSize[1];
    for (int k = 0; k < 3; ++k) g.vs[k] = p.voxelSize[k];
    g.iso = p.iso;
    // "if the mesh exceeds this number of vertices, an error returns" (vertex ids are 32-bit either way)
    const int64_t maxVerts = std::min<int64_t>(p.maxVertices, INT32_MAX);

    DeviceGuard guard(device);
    McWorkspace& ws = workspace(device);
    std::lock_guard<std::mutex> lk(ws.mu);
    uint8_t *flags = nullptr, *tcnt = nullptr;
    int32_t *chunkV = nullptr, *chunkT = nullptr, *baseV = nullptr, *baseT = nullptr, *sums = nullptr, *misc = nullptr;
    unsigned long long* totals = nullptr;
    float* dLz = nullptr;
    size_t sizes[10];
    mcSizes(d, sizes);
    void** ptrs[10] = {(void**)&flags, (void**)&tcnt, (void**)&chunkV, (void**)&chunkT, (void**)&baseV,
                       (void**)&baseT, (void**)&sums, (void**)&misc, (void**)&totals, (void**)&dLz};
    cudaError_t e = ws.ensure(mcWorkspaceBytes(d));
    if (!e) {
        size_t off = 0;
        for (int k = 0; k < 10; ++k) {
            *ptrs[k] = ws.buf + off;
            off += (sizes[k] + 255) / 256 * 256;
        }
    }
    if (!e) e = cudaMemsetAsync(totals, 0, sizeof(unsigned long long) * 3, s);
    if (!e) e = cudaMemcpyAsync(dLz, lz.data(), sizeof(float) * lz.size(), cudaMemcpyHostToDevice, s);
    if (!e) {
        const bool vec = (d.dx % 4) == 0 && (reinterpret_cast<uintptr_t>(dVol) % 16) == 0;
        const unsigned nbq = unsigned(std::max<int64_t>(1, std::min<int64_t>((d.qitems + 7) / 8, int64_t(numSMs()) * 8)));
        if (vec)
            classifyKernel<true><<<nbq, 256, 0, s>>>(dVol, d, p.iso, flags, chunkV, totals);
        else
            classifyKernel<false><<<nbq, 256, 0, s>>>(dVol, d, p.iso, flags, chunkV, totals);
        cellKernel<<<nbq, 256, 0, s>>>(flags, chunkV, d, tcnt, chunkT, totals + 1);
        e = cudaGetLastError();
    }
    unsigned long long ht[2] = {0, 0};
    if (!e) e = cudaMemcpyAsync(ht, totals, sizeof(ht), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (e) {
        delete m;
        return cudaFail(e, what);
    }
    if (int64_t(ht[0]) > maxVerts) {
        delete m;
        return mcError("Vertices number limit exceeded.");
    }
    if (ht[1] > INT32_MAX) {
        delete m;
        return mcError("Triangles number limit exceeded.");
    }
    m->nPoints = int64_t(ht[0]);
    m->nTris = int64_t(ht[1]);
    e = exclusiveScanI32(chunkV, baseV, d.nChunks, sums, misc, s);
    if (!e) e = exclusiveScanI32(chunkT, baseT, d.nChunks, sums, misc + 1, s);
    // outputs from the device's pool (reused across calls; returned when the mesh is destroyed)
    if (!e) e = poolMalloc((void**)&m->dPoints, sizeof(float) * 3 * size_t(m->nPoints), device, s);
    if (!e) e = poolMalloc((void**)&m->dTris, sizeof(int32_t) * 3 * size_t(m->nTris), device, s);
    if (!e && p.wantFaceMap) e = poolMalloc((void**)&m->dFaceMap, sizeof(int32_t) * size_t(m->nTris), device, s);
    if (!e) e = ws.ensureCells(sizeof(int64_t) * size_t(std::max<int64_t>(m->nTris, 1)));  // cells <= triangles
    if (!e) {
        int64_t* cellList = reinterpret_cast<int64_t*>(ws.cells);
        vertexKernel<<<mcBlocks(d), 256, 0, s>>>(dVol, flags, chunkV, baseV, d, g, dLz, m->dPoints);
        collectCellsKernel<<<mcBlocks(d), 256, 0, s>>>(tcnt, chunkT, d, cellList, totals + 2);
        const unsigned nbt = unsigned(std::max<int64_t>(1, std::min<int64_t>((m->nTris + 255) / 256, int64_t(numSMs()) * 8)));
        triangleKernel<<<nbt, 256, 0, s>>>(flags, tcnt, cellList, totals + 2, baseV, baseT, d, p.lessInside ? 1 : 0,
                                          m->dTris, m->dFaceMap);
        e = cudaGetLastError();
    }
    if (!e) e = cudaStreamSynchronize(s);
    if (e) {
        delete m;
        return cudaFail(e, what);
    }
    *out = m;
    return GBFWN_OK;
}

}  // namespace
}  // namespace gbfwn

using namespace gbfwn;

namespace {
bool mcProgress(gbfwn_progress_cb cb, void* user, float v) { return !cb || cb(v, user) != 0; }
bool validParams(const gbfwn_mc_params* p) {
    return p && std::isfinite(p->voxelSize[0]) && std::isfinite(p->voxelSize[1]) && std::isfinite(p->voxelSize[2]);
}
}  // namespace

extern "C" {

GBFWN_API void gbfwn_mc_default_params(gbfwn_mc_params* p) {
    if (!p) return;
    *p = gbfwn_mc_params{};
    p->voxelSize[0] = p->voxelSize[1] = p->voxelSize[2] = 1.f;
    p->maxVertices = INT32_MAX;
}

GBFWN_API int gbfwn_marching_cubes_dev(const float* d_volume, const int32_t dims[3], const gbfwn_mc_params* params,
                                       const int32_t* partStarts, int32_t nParts, int device, gbfwn_trimesh* out,
                                       void* stream) {
    if (!out || !dims || !validParams(params) || (nParts > 0 && !partStarts)) return fail(GBFWN_INVALID, "gbfwn_marching_cubes_dev: bad arguments");
    *out = nullptr;
    if (!d_volume && int64_t(dims[0]) * dims[1] * dims[2] > 0 && dims[0] > 0 && dims[1] > 0 && dims[2] > 0)
        return fail(GBFWN_INVALID, "gbfwn_marching_cubes_dev: null volume");
    return runMarchingCubes(d_volume, dims, *params, partStarts, nParts, device, static_cast<cudaStream_t>(stream), out,
                            "gbfwn_marching_cubes_dev");
}

GBFWN_API int gbfwn_marching_cubes(const float* volume, const int32_t dims[3], const gbfwn_mc_params* params,
                                   const int32_t* partStarts, int32_t nParts, int device, gbfwn_trimesh* out,
                                   gbfwn_progress_cb cb, void* user) {
    if (!out || !dims || !validParams(params) || (nParts > 0 && !partStarts)) return fail(GBFWN_INVALID, "gbfwn_marching_cubes: bad arguments");
    *out = nullptr;
    const bool empty = dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0;
    if (!volume && !empty) return fail(GBFWN_INVALID, "gbfwn_marching_cubes: null volume");
    if (!mcProgress(cb, user, 0.f)) return fail(GBFWN_CANCELLED, "Operation was canceled");
    DeviceGuard g(device);
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e) return cudaFail(e, "gbfwn_marching_cubes");
    float* dVol = nullptr;
    const size_t n = empty ? 0 : size_t(dims[0]) * size_t(dims[1]) * size_t(dims[2]);
    e = poolMalloc((void**)&dVol, sizeof(float) * n, device, s);
    if (!e && n) e = cudaMemcpyAsync(dVol, volume, sizeof(float) * n, cudaMemcpyHostToDevice, s);
    int st = e ? cudaFail(e, "gbfwn_marching_cubes") : GBFWN_OK;
    if (!st && !mcProgress(cb, user, 0.3f)) st = fail(GBFWN_CANCELLED, "Operation was canceled");
    if (!st) st = runMarchingCubes(dVol, dims, *params, partStarts, nParts, device, s, out, "gbfwn_marching_cubes");
    poolFree(dVol, s);  // stream-ordered after the copy and the mesher on s
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (!st && !mcProgress(cb, user, 1.f)) {
        gbfwn_trimesh_destroy(*out);
        *out = nullptr;
        st = fail(GBFWN_CANCELLED, "Operation was canceled");
    }
    return st;
}

GBFWN_API int gbfwn_mc_release_workspace(int device) {
    McWorkspace& ws = workspace(device);
    std::lock_guard<std::mutex> lk(ws.mu);
    DeviceGuard g(device);
    cudaFree(ws.buf);
    cudaFree(ws.cells);
    ws.buf = ws.cells = nullptr;
    ws.cap = ws.cellCap = 0;
    return GBFWN_OK;
}

GBFWN_API size_t gbfwn_marching_cubes_memory(const int32_t dims[3], int64_t expectedTriangles) {
    if (!dims || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return 0;
    const McDims d = mcDims(dims);
    const size_t nt = size_t(std::max<int64_t>(expectedTriangles, 0));
    // work arrays + cell list + output (points ~ triangles / 2, 3 floats; triangles 3 ints + face map)
    return mcWorkspaceBytes(d) + 8 * nt + 6 * nt + 16 * nt;
}

GBFWN_API int gbfwn_trimesh_sizes(gbfwn_trimesh m, int64_t* numPoints, int64_t* numTris) {
    if (!m) return fail(GBFWN_INVALID, "gbfwn_trimesh_sizes: null mesh");
    if (numPoints) *numPoints = m->nPoints;
    if (numTris) *numTris = m->nTris;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_trimesh_copy(gbfwn_trimesh m, float* points, int32_t* tris, int32_t* faceMap) {
    if (!m) return fail(GBFWN_INVALID, "gbfwn_trimesh_copy: null mesh");
    if (faceMap && !m->dFaceMap && m->nTris) return fail(GBFWN_INVALID, "gbfwn_trimesh_copy: the face map was not requested");
    DeviceGuard g(m->device);
    cudaError_t e = cudaSuccess;
    if (points && m->nPoints) e = cudaMemcpy(points, m->dPoints, sizeof(float) * 3 * size_t(m->nPoints), cudaMemcpyDeviceToHost);
    if (!e && tris && m->nTris) e = cudaMemcpy(tris, m->dTris, sizeof(int32_t) * 3 * size_t(m->nTris), cudaMemcpyDeviceToHost);
    if (!e && faceMap && m->nTris) e = cudaMemcpy(faceMap, m->dFaceMap, sizeof(int32_t) * size_t(m->nTris), cudaMemcpyDeviceToHost);
    return e ? cudaFail(e, "gbfwn_trimesh_copy") : GBFWN_OK;
}

GBFWN_API int gbfwn_trimesh_device(gbfwn_trimesh m, const float** d_points, const int32_t** d_tris,
                                   const int32_t** d_faceMap) {
    if (!m) return fail(GBFWN_INVALID, "gbfwn_trimesh_device: null mesh");
    if (d_points) *d_points = m->dPoints;
    if (d_tris) *d_tris = m->dTris;
    if (d_faceMap) *d_faceMap = m->dFaceMap;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_trimesh_destroy(gbfwn_trimesh m) {
    delete m;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_mc_parts_create(const int32_t dims[3], const gbfwn_mc_params* params, int device, gbfwn_mc_parts* out) {
    if (!out || !dims || !validParams(params)) return fail(GBFWN_INVALID, "gbfwn_mc_parts_create: bad arguments");
    *out = nullptr;
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return fail(GBFWN_INVALID, "gbfwn_mc_parts_create: non-positive dimensions");
    auto* p = new gbfwn_mc_parts_s;
    p->device = device;
    std::memcpy(p->dims, dims, sizeof(p->dims));
    p->params = *params;
    DeviceGuard g(device);
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (!e) e = poolMalloc((void**)&p->dVol, sizeof(float) * size_t(dims[0]) * size_t(dims[1]) * size_t(dims[2]), device, p->stream);
    if (e) {
        delete p;
        return cudaFail(e, "gbfwn_mc_parts_create");
    }
    *out = p;
    return GBFWN_OK;
}

GBFWN_API int32_t gbfwn_mc_parts_next_z(gbfwn_mc_parts p) { return p ? p->nextZ : 0; }

namespace {
int addPart(gbfwn_mc_parts p, const float* part, const int32_t partDims[3], cudaMemcpyKind kind, cudaStream_t s) {
    if (!p || !part || !partDims) return fail(GBFWN_INVALID, "gbfwn_mc_parts_add: bad arguments");
    // MarchingCubesByParts::addPart checks (MRMarchingCubes.cpp:436-441)
    if (partDims[0] != p->dims[0] || partDims[1] != p->dims[1])
        return mcError("XY dimensions of a part must be equal to XY dimensions of whole volume");
    if (partDims[2] <= 1) return mcError("a part must have at least two Z slices");
    if (int64_t(p->nextZ) + partDims[2] > p->dims[2]) return mcError("a part exceeds whole volume in Z dimension");
    DeviceGuard g(p->device);
    const size_t layer = size_t(p->dims[0]) * size_t(p->dims[1]);
    cudaError_t e = cudaMemcpyAsync(p->dVol + layer * size_t(p->nextZ), part, sizeof(float) * layer * size_t(partDims[2]), kind, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (e) return cudaFail(e, "gbfwn_mc_parts_add");
    p->starts.push_back(p->nextZ);
    p->nextZ += partDims[2] - 1;
    return GBFWN_OK;
}
}  // namespace

GBFWN_API int gbfwn_mc_parts_add(gbfwn_mc_parts p, const float* part, const int32_t partDims[3]) {
    return addPart(p, part, partDims, cudaMemcpyHostToDevice, p ? p->stream : nullptr);
}

GBFWN_API int gbfwn_mc_parts_add_dev(gbfwn_mc_parts p, const float* d_part, const int32_t partDims[3], void* stream) {
    return addPart(p, d_part, partDims, cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream));
}

GBFWN_API int gbfwn_mc_parts_finalize(gbfwn_mc_parts p, gbfwn_trimesh* out) {
    if (!p || !out) return fail(GBFWN_INVALID, "gbfwn_mc_parts_finalize: bad arguments");
    *out = nullptr;
    if (p->nextZ + 1 != p->dims[2]) return mcError("Provided parts do not cover whole volume");
    return runMarchingCubes(p->dVol, p->dims, p->params, p->starts.data(), int32_t(p->starts.size()), p->device, p->stream,
                            out, "gbfwn_mc_parts_finalize");
}

GBFWN_API int gbfwn_mc_parts_destroy(gbfwn_mc_parts p) {
    delete p;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_grid_to_mesh(gbfwn_handle h, gbfwn_surrogate sur, const int32_t dims[3], const float origin[3],
                                 const float voxelSize[3], const gbfwn_dist_opts* opts, const gbfwn_mc_params* mc,
                                 const int32_t* partStarts, int32_t nParts, gbfwn_trimesh* out, gbfwn_progress_cb cb,
                                 void* user) {
    if (!h || !dims || !origin || !voxelSize || !validParams(mc) || !out || (nParts > 0 && !partStarts))
        return fail(GBFWN_INVALID, "gbfwn_grid_to_mesh: bad arguments");
    *out = nullptr;
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return fail(GBFWN_INVALID, "gbfwn_grid_to_mesh: non-positive dimensions");
    if (!mcProgress(cb, user, 0.f)) return fail(GBFWN_CANCELLED, "Operation was canceled");
    // grid basis of mcOffsetMesh: AffineXf3f{ Matrix3f::scale(voxelSize), origin + 0.5f * voxelSize }
    float xf[12] = {voxelSize[0], 0.f, 0.f, 0.f, voxelSize[1], 0.f, 0.f, 0.f, voxelSize[2], 0.f, 0.f, 0.f};
    for (int k = 0; k < 3; ++k) xf[9 + k] = origin[k] + 0.5f * voxelSize[k];
    gbfwn_dist_opts o;
    if (opts) {
        o = *opts;
    } else {
        o = gbfwn_dist_opts{0.f, FLT_MAX, 1, 0.5f, 2.f};
    }
    const bool banded = o.maxDistSq > 0.f && o.maxDistSq < FLT_MAX && o.nullOutsideMinMax;
    DeviceGuard g(h->device);
    float* grid = nullptr;
    cudaError_t e = poolMalloc((void**)&grid, sizeof(float) * size_t(dims[0]) * size_t(dims[1]) * size_t(dims[2]), h->device,
                               h->stream);
    if (e) return cudaFail(e, "gbfwn_grid_to_mesh");
    int st = GBFWN_OK;
    if ((e = h->resetStatus(h->stream))) st = cudaFail(e, "gbfwn_grid_to_mesh");
    if (st) {
    } else if (banded) {
        gbfwn_banded_stats stats;
        st = gbfwn_from_grid_with_distances_banded_dev(h, sur, dims, xf, &o, grid, &stats, h->stream);
    } else {
        st = gbfwn_from_grid_with_distances_dev(h, dims, xf, &o, grid, h->stream);
    }
    if (!st) st = h->checkStatus();  // synchronises; reports a traversal overflow
    if (!st && !mcProgress(cb, user, 0.9f)) st = fail(GBFWN_CANCELLED, "Operation was canceled");
    if (!st) st = runMarchingCubes(grid, dims, *mc, partStarts, nParts, h->device, h->stream, out, "gbfwn_grid_to_mesh");
    poolFree(grid, h->stream);  // the mesher has synchronised h->stream
    if (!st && !mcProgress(cb, user, 1.f)) {
        gbfwn_trimesh_destroy(*out);
        *out = nullptr;
        st = fail(GBFWN_CANCELLED, "Operation was canceled");
    }
    return st;
}

}  // extern "C"
