// Shared definitions of the GB300 winding-number library: device data layout, kernel entry
// points and host helpers.  Everything here is internal; the public surface is include/gbfwn.h.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace gbfwn {

// ---------------------------------------------------------------------------------------------
// Reference tree layout (MRMesh/MRAABBTreeNode.h:29-46): box + l + r, leaf <=> r < 0 with l = face.
// Nodes are in the reference's pre-order: the left child of internal node i is i + 1.
struct RefNode {
    float minx, miny, minz, maxx, maxy, maxz;
    int32_t l, r;
};
static_assert(sizeof(RefNode) == 32, "reference node is 32 bytes");

// ---------------------------------------------------------------------------------------------
// Query layout in HBM ("wide" records: a parent stores both children, so one 64-byte record
// read gives everything a traversal step needs; children are fetched as float4, all lanes of a
// warp read the same record, so each load is a broadcast).
//
//  cp  [internal k] 6 x float4 : the frame of node k (orthonormal t, u, n: the area-weighted normal
//                                of its triangles completed to a basis) and, in that one frame, the
//                                centre c and half extents e of each child's box:
//                                {t.xyz, u.x} {u.yz, n.xy} {n.z, cL} {eL, lLink} {cR, eR.x}
//                                {eR.yz, rLink, 0}
//  dip [internal k] 4 x float4 : {lpos.xyz, l rr}  {l dirArea.xyz, lLink} {rpos.xyz, r rr} {r dirArea.xyz, rLink}
//  tri [leaf slot s] 3 x float4: {a.xyz, face} {b.xyz, 0} {c.xyz, 0}
//
// A link >= 0 is an internal-node index k (internal nodes numbered in pre-order), a link < 0 is
// ~slot of a leaf; leaf slots are the leaves in pre-order.  Root data travels in the kernel
// parameters.
struct QueryTree {
    const float4* __restrict__ cp;
    const float4* __restrict__ dip;
    const float4* __restrict__ tri;
    const int32_t* __restrict__ faceSlot;  // face -> slot, -1 for invalid faces
    const float4* __restrict__ nodes;      // the reference nodes (RefNode: {min.xyz, max.x} {max.yz, l, r})
    float4 rootDip0, rootDip1;             // {pos.xyz, rr} {dirArea.xyz, rootLink}
    float4 rootBox0, rootBox1;             // {min.xyz, rootLink} {max.xyz, 0}
    int32_t nLeaves;
    int32_t nFaces;
    // 1: the faces form a closed oriented surface (every edge used equally often in both
    // directions): a signed-distance voxel may take its sign from the voxel below it when no surface
    // lies between them, and otherwise from the signed count of surface crossings of a ray
    // (gridKernel); 0: every sign comes from its own winding number
    int32_t closed;
};

// Squared-distance level below which the precise triangle distance is re-evaluated in FP64 (the
// query lies within about 1e-4 edge lengths of the triangle): 1e-8 of |b - a|^2 + |c - a|^2, rounded
// the same way wherever it is computed.  Kept in the leaf records (the fourth word of c).
__device__ __forceinline__ float nearPlaneLevel(const float4& a, const float4& b, const float4& c) {
    const float abx = __fsub_rn(b.x, a.x), aby = __fsub_rn(b.y, a.y), abz = __fsub_rn(b.z, a.z);
    const float acx = __fsub_rn(c.x, a.x), acy = __fsub_rn(c.y, a.y), acz = __fsub_rn(c.z, a.z);
    const float s = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(abx, abx), __fmul_rn(aby, aby)), __fmul_rn(abz, abz)),
                              __fadd_rn(__fadd_rn(__fmul_rn(acx, acx), __fmul_rn(acy, acy)), __fmul_rn(acz, acz)));
    return __fmul_rn(1e-8f, s);
}

struct Xf {
    float a[9];  // rows
    float b[3];
};

struct DistOpts {
    float minDistSq, maxDistSq;
    int32_t nullOutsideMinMax;
    float threshold, beta;
};

// Grid sub-range handled by one launch: layers [z0, z1) of a dims grid, written to out with the
// layer z at (z - zOut) * nx * ny.
struct GridRange {
    int32_t nx, ny, nz;
    int32_t z0, z1, zOut;
};

// Device status word bits.
enum : unsigned {
    kStatusStackOverflow = 1u,
    kStatusTimeout = 2u,
};

// ---------------------------------------------------------------------------------------------
// Kernel launchers (query.cu; the column sign pass in columns.cu).  All take a `scratch` pointer to two device words: [0] = work
// queue ticket counter, [1] = status bits.  The launchers reset the ticket counter themselves.
cudaError_t launchGridFwn(const QueryTree& t, const GridRange& g, const Xf& xf, float beta, int precise, float* out,
                          unsigned* scratch, cudaStream_t s);
// colState (optional, colBytes >= gridSdfColumnStateBytes): device words through which the columns of
// the launch hand their top layer's distances, signs and closest triangles to the columns above,
// followed, on a closed mesh whose grid has a vertical z axis (signColumnsApply), by the inside bits
// of the grid's columns and the columns' crossing lists, computed first (launchSignColumns).
cudaError_t launchGridSdf(const QueryTree& t, const GridRange& g, const Xf& xf, const DistOpts& o, int precise,
                          float* out, unsigned* scratch, cudaStream_t s, float* colState = nullptr, size_t colBytes = 0);
size_t gridSdfColumnStateBytes(const QueryTree& t, const GridRange& g, const Xf& xf, const DistOpts& o);
// Signs of a closed mesh's grid from its vertical columns' crossings (columns.cu, signColumnsKernel):
// applicable when signColumnsApply; writes inside bits (one 32-bit word per 32 voxels along x, layout
// (z - zOut, y, x / 32)) or negates `values` where the voxel is inside.
bool signColumnsApply(const QueryTree& t, const Xf& xf, float beta, float threshold);
// work (optional, workBytes >= signColumnsWorkBytes): the columns' crossing lists, filled from the
// triangles first; without it every column casts its own ray.
size_t signColumnsWorkBytes(const GridRange& g);
cudaError_t launchSignColumns(const QueryTree& t, const GridRange& g, const Xf& xf, float beta, float threshold, int precise,
                              uint32_t* bits, float* values, void* work, size_t workBytes, unsigned* scratch, cudaStream_t s);
// One mesh + grid of a batched launch (query.cu batchKernel): its tickets are
// [tileBase, tileBase + batchTiles(...)): columns of up to kBatchSeg tiles of the launch's shape.
struct BatchItem {
    QueryTree t;
    GridRange g;  // whole grid: z0 = 0, z1 = nz, zOut = 0
    Xf xf;
    DistOpts o;
    float* out;
    uint32_t tileBase;
};
constexpr int kBatchShapes = 6;                  // tile shape x block size variants
constexpr int kBatchConfigs = 2 * kBatchShapes;  // each with the one-voxel walk, then with the paired walk
// tiles along z per work item (a column walked by one warp).  64-mesh batch, best configuration, the
// same outputs: 4 tiles 54.9 ms, 8 54.4, 16 52.9, 24 52.4, 32 52.1 (sign reuse makes long columns pay;
// 16 leaves more items for the load balance of batches of small grids)
constexpr int kBatchSeg = 16;
const char* batchConfigName(int config);
uint64_t batchTiles(int config, int32_t nx, int32_t ny, int32_t nz);
// pairOk: every item has minDistSq = 0 (the paired variants need it); fix: the precise paired walk's
// list, batchFixCap(totalTiles) entries after a 16-byte counter.
uint32_t batchFixCap(uint32_t totalTiles);
cudaError_t launchBatchSdf(const BatchItem* items, int nItems, uint32_t totalTiles, int precise, int config, bool pairOk,
                           void* fix, unsigned* scratch, cudaStream_t s);

// Signed distance on runs of 8x8x8-voxel bricks of the grid: runs[i] = (bx, by, bz0, count), the
// `count` bricks (bx, by, bz0 .. bz0 + count - 1), nBricks in all; voxels outside them are not written.
// signBits (optional): the grid's inside bits from launchSignColumns, used for the signs; fix (with
// them, pairFixBytesForRuns bytes): the precise paired walk's fix list, without which precise grids
// take the one-voxel walk.
cudaError_t launchGridSdfBricks(const QueryTree& t, const GridRange& g, const Xf& xf, const DistOpts& o, int precise,
                                float* out, const int4* runs, int32_t nRuns, int32_t nBricks, const uint32_t* signBits,
                                void* fix, unsigned* scratch, cudaStream_t s);
// Bytes of the precise paired walk's fix list for nTiles warp tiles in nItems work items, and for
// brick runs.
size_t pairFixBytes(uint32_t nTiles, uint32_t nItems);
size_t pairFixBytesForRuns(int32_t nRuns, int32_t nBricks);
// Bytes of the inside bits of a grid range (one 32-bit word per 32 voxels along x).
size_t signBitsBytes(const GridRange& g);
// Point queries; `order` (optional) is a permutation of [0, n): points are processed in that order
// (mortonOrder gives a spatially coherent one) and results land at their original indices.
cudaError_t launchVectorFwn(const QueryTree& t, const float* pts, int64_t n, float beta, int32_t skipFace, int precise,
                            float* out, unsigned* scratch, cudaStream_t s, const int32_t* order = nullptr);
cudaError_t launchVectorSdf(const QueryTree& t, const float* pts, int64_t n, const DistOpts& o, int precise, float* out,
                            unsigned* scratch, cudaStream_t s, const int32_t* order = nullptr);
// Closest point on the mesh for n points (MR::IPointsToMeshProjector::findProjections): each point is
// mapped by pointXf (optional), the mesh by treeXf (optional; the non-rigid case).  out holds 2 float4
// per point, the layout of MR::MeshProjectionResult: {face, x, y, z} {edge = -1, a, b, distSq}.
cudaError_t launchProject(const QueryTree& t, const float* pts, int64_t n, const Xf* pointXf, const Xf* treeXf, float upSq,
                          float loSq, int precise, float4* out, unsigned* scratch, cudaStream_t s, const int32_t* order = nullptr);
// Morton order of n points inside the box [lo, hi] (sort.cu); `scratch` holds mortonOrderScratch(n)
// int32 words.
int64_t mortonOrderScratch(int64_t n);
cudaError_t mortonOrder(const float* pts, int64_t n, const float lo[3], const float hi[3], int32_t* order, int32_t* scratch,
                        cudaStream_t s);
cudaError_t launchSelfIntersections(const QueryTree& t, float beta, int precise, uint64_t* bits, float* wn,
                                    unsigned* scratch, cudaStream_t s);

// ---------------------------------------------------------------------------------------------
// Tree/dipole construction (build.cu).
struct DeviceTree {
    int64_t nFaces = 0, nLeaves = 0, nInternal = 0;
    bool closed = false;  // the valid faces form a closed oriented surface (treebuild.cu, validFaces)
    RefNode* nodes = nullptr;   // 2n-1 reference nodes
    float* dip8 = nullptr;      // 2n-1 x 8 reference dipoles
    float4* cp = nullptr;
    float4* dip = nullptr;
    float4* tri = nullptr;
    int32_t* faceSlot = nullptr;
    QueryTree q{};
};

// Builds the tree on the device from device verts / tris (build.cu).  Allocation goes through
// `alloc`, which the caller frees as a whole.
struct Allocator {
    virtual cudaError_t alloc(void** p, size_t bytes) = 0;
    virtual ~Allocator() = default;
};
// P: allocations that live with the handle; T: work arrays the caller frees after the build.
cudaError_t buildDeviceTree(const float* dVerts, int64_t nv, const int32_t* dTris, int64_t nt, DeviceTree& out,
                            Allocator& P, Allocator& T, cudaStream_t s, std::string& err);

// AABBTree::refit + dipole recomputation for moved vertices (build.cu): the tree keeps its
// topology; dVerts holds all vertices at their new positions; dChanged (nv bits in 64-bit words,
// nullable = all) marks the moved ones.  Reuses the tree's arrays; work arrays come from T.
cudaError_t refitDeviceTree(const float* dVerts, int64_t nv, const int32_t* dTris, const uint64_t* dChanged, DeviceTree& out,
                            Allocator& P, Allocator& T, cudaStream_t s);

int numSMs();

// Exclusive prefix sum of n int32 values (treebuild.cu); `sums` holds ceil(n / 1024) + 1 words of
// scratch, `total` receives the sum of all values.
cudaError_t exclusiveScanI32(const int32_t* in, int32_t* out, int64_t n, int32_t* sums, int32_t* total, cudaStream_t s);

// Number of warp tiles a grid of nx x ny x nz voxels is cut into; the work-queue ticket counter is
// 32 bits, so a single launch covers at most 2^32 - 1 tiles.
uint64_t gridTiles(int32_t nx, int32_t ny, int32_t nz);
constexpr uint64_t kMaxTilesPerLaunch = 0xffffffffull;

}  // namespace gbfwn
