// Grid, point, projection, self-intersection and batched kernels and their launchers, over the
// traversal primitives of traverse.cuh.
#include "traverse.cuh"

namespace gbfwn {

namespace {

// True when a voxel at q may take the sign of the voxel at qb, whose squared distance to the surface
// is belowSq (> 0, from a search that ran to the end): qb is farther from the surface than from q, so
// the segment between them meets no surface.  The margin covers the FP32 rounding of both centres and
// of the distance, relative to the coordinates' magnitude.  qb must be computed exactly as that
// voxel's centre was (the same xfPoint call).
__device__ __forceinline__ bool emptyBallCovers(const float3& q, const float3& qb, float belowSq) {
    const float dx = q.x - qb.x, dy = q.y - qb.y, dz = q.z - qb.z;
    const float step = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    const float db = sqrtf(belowSq);
    const float mag = fmaxf(fabsf(q.x), fmaxf(fabsf(q.y), fabsf(q.z)));
    return db > fmaf(step, 1.0001f, 2e-6f * fmaf(3.f, mag, db));
}

// Sign reuse for one tile of TX x TY x TZ voxels (lane = lx + TX (ly + TY lz)) after its closest-point
// searches.  below: the state of the voxel that precedes this lane's voxel (the previous tile's top
// layer for the bottom layer, the lane's own voxel of the previous tile for the others): its squared
// distance with its side in the sign bit, NaN when unknown; zb: that voxel's layer.  A lane above the
// bottom layer may also take the sign of the voxel one layer below it in this tile, once that one's
// sign is settled by reuse.  Returns whether the lane's sign is settled; *inside receives it.
template <int TX, int TY, int TZ>
__device__ __forceinline__ bool reuseSign(const Xf& xf, int x, int y, int z, int zb, int lz, const float3& q, float below,
                                          bool complete, float dsq, bool* inside) {
    bool reuse = fabsf(below) > 0.f && emptyBallCovers(q, xfPoint(xf, x, y, zb), fabsf(below));
    bool in = signbit(below);
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int l = 1; l < TZ; ++l) {
        const float e = __shfl_sync(FULL, (reuse && complete) ? (in ? -dsq : dsq) : __int_as_float(0x7fc00000),
                                    lane >= TX * TY ? lane - TX * TY : lane);
        if (lz == l && !reuse && fabsf(e) > 0.f && emptyBallCovers(q, xfPoint(xf, x, y, z - 1), fabsf(e))) {
            reuse = true;
            in = signbit(e);
        }
    }
    *inside = in;
    return reuse;
}

// A warp takes a column of tiles along z and walks it upwards.  Each lane starts its closest-point
// search from the triangle that was closest to a voxel just below its own: the bottom layer of a
// tile from the voxel one layer below (the previous tile's top layer), the top layer from its own
// voxel of the previous tile, two layers below.  That triangle's distance is an upper bound the
// search would reach anyway, so the minimum is unchanged, but it prunes from the first step (a third
// fewer node visits with an exact bound, in a CPU model of the walk).  On a closed surface the same
// voxel below also lends its sign (signReuseAllowed) when its distance exceeds the step between the
// two voxel centres, and the lane skips its winding-number walk.
template <bool PRECISE, bool DIST, bool BITS = false>
__global__ void __launch_bounds__(kThreads, DIST ? kDistBlocks : 4) gridKernel(QueryTree t, GridRange g, TileGrid tg, Xf xf, DistOpts o,
                                                       float* __restrict__ out, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const int lx = lane % kTX, ly = (lane / kTX) % kTY, lz = lane / (kTX * kTY);
    const float betaSq = __fmul_rn(o.beta, o.beta);
    const size_t sxy = size_t(g.nx) * g.ny;
    const bool reuseOk = DIST && !BITS && signReuseAllowed(t, o);
    const int wordsX = (g.nx + 31) >> 5;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (item >= tg.numItems) break;
        int x0, y0, zBase, nSeg;
        if (tg.runs) {
            const int4 r = tg.runs[item / kBrickCols];
            const int col = int(item % kBrickCols);
            x0 = r.x * 8 + (col % kBrickColsX) * kTX;
            y0 = r.y * 8 + (col / kBrickColsX) * kTY;
            zBase = g.z0 + r.z * 8;
            nSeg = kBrickSeg * r.w;
        } else {
            const int tx = int(item % unsigned(tg.tilesX));
            const unsigned rest = item / unsigned(tg.tilesX);
            const int ty = int(rest % unsigned(tg.tilesY));
            const int sz = int(rest / unsigned(tg.tilesY));
            x0 = tx * kTX;
            y0 = ty * kTY;
            zBase = g.z0 + sz * tg.segLen * kTZ;
            nSeg = min(tg.segLen, tg.tilesZ - sz * tg.segLen);
        }
        const int x = x0 + lx, y = y0 + ly;
        int seed = -1;  // leaf slot closest to the voxel below
        // that voxel's squared distance with its side in the sign bit (negative inside), NaN when
        // its sign is unknown
        float below = __int_as_float(0x7fc00000);
        const uint32_t colsPerSlab = uint32_t(tg.tilesX) * uint32_t(tg.tilesY);
        if (DIST && tg.colState && !tg.runs && item >= colsPerSlab) {
            // the column below ended (its state was written) or not yet (0xff bytes: start cold); the
            // voxel below both layers of the first tile is that column's top-layer voxel
            const float* cs = tg.colState + size_t(item - colsPerSlab) * (2 * kLayer);
            if (!BITS) below = __ldcg(cs + lane % kLayer);
            seed = __float_as_int(__ldcg(cs + kLayer + lane % kLayer));
        }
        for (int j = 0; j < nSeg; ++j) {
            const int z = zBase + j * kTZ + lz;
            const bool active = x < g.nx && y < g.ny && z < g.z1;
            const float3 q = xfPoint(xf, x, y, z);
            float res;
            if (DIST) {
                float up = o.maxDistSq;
                if (active && seed >= 0) {
                    const float4* tr = t.tri + 3 * int64_t(seed);
                    const float ds = triDistSq<PRECISE>(q, ld4(tr), ld4(tr + 1), ld4(tr + 2));
                    if (ds < up) up = ds;
                }
                int best = active ? seed : -1;
                const float dsq = cpPacket<PRECISE, true>(t, q, active, up, o.minDistSq, scratch + 1, &best);
                const bool valid = !(o.nullOutsideMinMax && (dsq < o.minDistSq || dsq >= o.maxDistSq));
                const bool complete = active && valid && dsq >= o.minDistSq;
                bool inside;
                if (BITS) {  // the column rays' signs
                    const uint32_t word = active ? __ldg(tg.signBits + (size_t(z - g.zOut) * g.ny + y) * wordsX + (x >> 5)) : 0u;
                    inside = (word >> (x & 31)) & 1u;
                } else {
                    bool reIn = false;
                    const bool reuse = reuseOk && reuseSign<kTX, kTY, kTZ>(xf, x, y, z, z - (lz == 0 ? 1 : kTZ), lz, q, below,
                                                                          complete, dsq, &reIn);
                    // closed surface: the exact winding number from ray crossings, but the approximated
                    // one (the reference's decision) for a voxel on the surface; otherwise the latter
                    bool onSurface = false;
                    const int cw = reuseOk ? rayWinding(t, q, active && valid && !reuse, scratch + 1, &onSurface) : 0;
                    const bool fwn = reuseOk ? onSurface : (active && valid);
                    const float w = fwnPacket<PRECISE>(t, q, fwn, betaSq, -1, scratch + 1);
                    inside = reuse ? reIn : (fwn ? w > o.threshold : float(cw) > o.threshold);
                }
                const float d = __fsqrt_rn(dsq);
                res = valid ? (inside ? -d : d) : __int_as_float(0x7fc00000);
                // next tile: the bottom layer's lanes take the voxel one layer below them (this tile's
                // top layer), the others their own voxel two layers below.  A distance counts only when
                // the search ran to the end (not cut short below minDistSq): no surface is closer then.
                const int src = lane + (kTZ - 1) * kTX * kTY * (lz == 0);
                seed = __shfl_sync(FULL, best, src);
                if (!BITS) below = __shfl_sync(FULL, complete ? (inside ? -dsq : dsq) : __int_as_float(0x7fc00000), src);
                if (tg.colState && !tg.runs && j == nSeg - 1 && lz == kTZ - 1) {
                    // the column's last tile: the top layer's lanes hold their own voxels' state and
                    // pass on the distances and the seeds at this work item's words (the item
                    // recomputed from the column's position, so no register holds it through the walk)
                    const uint32_t sz = uint32_t(zBase - g.z0) / uint32_t(tg.segLen * kTZ);
                    const uint32_t it = uint32_t(x0) / kTX + uint32_t(tg.tilesX) * (uint32_t(y0) / kTY + uint32_t(tg.tilesY) * sz);
                    float* cs = tg.colState + size_t(it) * (2 * kLayer) + (lane - (kTZ - 1) * kLayer);
                    cs[0] = below;
                    cs[kLayer] = __int_as_float(seed);
                }
            } else {
                res = fwnPacket<PRECISE>(t, q, active, betaSq, -1, scratch + 1);
            }
            if (active) out[size_t(z - g.zOut) * sxy + size_t(y) * g.nx + x] = res;
        }
    }
}

// Signed distances with the column pass's sign bits and no lower distance bound (minDistSq = 0): a
// warp walks its column two tiles at a time, each lane taking its voxel of the lower tile and the one
// two layers above it (a 4x4x4 block of voxels) through one shared packet walk (cpPacket2), so each
// record read and stack step serves 64 voxels.  Both start from the triangle closest to the voxel
// below the lower tile (as gridKernel's seeds); results are the exact minima, as gridKernel's.  In
// precise mode the walk runs in FP32 and the voxels that came within a triangle's near-plane level
// are listed for fixPairKernel, which walks them again with the precise distances.
template <bool PRECISE>
__global__ void __launch_bounds__(kThreads, kPairBlocks) gridPairKernel(QueryTree t, GridRange g, TileGrid tg, Xf xf, DistOpts o,
                                                                        float* __restrict__ out, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const int lx = lane % kTX, ly = (lane / kTX) % kTY, lz = lane / (kTX * kTY);
    const size_t sxy = size_t(g.nx) * g.ny;
    const int wordsX = (g.nx + 31) >> 5;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (item >= tg.numItems) break;
        int x0, y0, zBase, nSeg;
        if (tg.runs) {
            const int4 r = tg.runs[item / kBrickCols];
            const int col = int(item % kBrickCols);
            x0 = r.x * 8 + (col % kBrickColsX) * kTX;
            y0 = r.y * 8 + (col / kBrickColsX) * kTY;
            zBase = g.z0 + r.z * 8;
            nSeg = kBrickSeg * r.w;
        } else {
            const int tx = int(item % unsigned(tg.tilesX));
            const unsigned rest = item / unsigned(tg.tilesX);
            const int ty = int(rest % unsigned(tg.tilesY));
            const int sz = int(rest / unsigned(tg.tilesY));
            x0 = tx * kTX;
            y0 = ty * kTY;
            zBase = g.z0 + sz * tg.segLen * kTZ;
            nSeg = min(tg.segLen, tg.tilesZ - sz * tg.segLen);
        }
        const int x = x0 + lx, y = y0 + ly;
        int seed = -1;
        const uint32_t colsPerSlab = uint32_t(tg.tilesX) * uint32_t(tg.tilesY);
        if (tg.colState && !tg.runs && item >= colsPerSlab)
            seed = __float_as_int(__ldcg(tg.colState + size_t(item - colsPerSlab) * (2 * kLayer) + kLayer + lane % kLayer));
        for (int j = 0; j < nSeg; j += 2) {
            const bool hasB = j + 1 < nSeg;
            const int za = zBase + j * kTZ + lz, zb = za + kTZ;
            const bool inXY = x < g.nx && y < g.ny;
            const bool activeA = inXY && za < g.z1, activeB = inXY && hasB && zb < g.z1;
            const float3 qa = xfPoint(xf, x, y, za), qb = xfPoint(xf, x, y, zb);
            float ra = o.maxDistSq, rb = o.maxDistSq;
            int ba = -1, bb = -1;
            if (PRECISE) {
                if (lane == 0) sPairFix[threadIdx.x >> 5][0] = sPairFix[threadIdx.x >> 5][1] = 0u;
                __syncwarp();
            }
            if (seed >= 0 && (activeA || activeB)) {
                bool da = false, db = false;
                leafDist2<PRECISE>(t, seed, qa, qb, activeA, activeB, ra, rb, ba, bb, da, db);
            }
            cpPacket2<PRECISE>(t, qa, qb, activeA, activeB, ra, rb, ba, bb, scratch + 1);
            if (PRECISE) {
                __syncwarp();
                const unsigned ma = sPairFix[threadIdx.x >> 5][0], mb = sPairFix[threadIdx.x >> 5][1];
                if ((ma | mb) && lane == 0) {  // re-walked with the precise distances by fixPairKernel
                    const uint32_t k = atomicAdd(&tg.fixList[0].x, 1u);
                    if (k < tg.fixCap) tg.fixList[1 + k] = make_uint4(item, uint32_t(j), ma, mb);
                }
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const bool active = h ? activeB : activeA;
                const int z = h ? zb : za;
                const float dsq = h ? rb : ra;
                const bool valid = !(o.nullOutsideMinMax && dsq >= o.maxDistSq);
                const uint32_t word = active ? __ldg(tg.signBits + (size_t(z - g.zOut) * g.ny + y) * wordsX + (x >> 5)) : 0u;
                const bool inside = (word >> (x & 31)) & 1u;
                const float d = __fsqrt_rn(dsq);
                if (active) out[size_t(z - g.zOut) * sxy + size_t(y) * g.nx + x] = valid ? (inside ? -d : d) : __int_as_float(0x7fc00000);
            }
            // next pair: the bottom layer's lanes continue from the voxel one layer below them, the
            // others from their own last voxel (as gridKernel)
            const int src = lane + (kTZ - 1) * kTX * kTY * (lz == 0);
            seed = __shfl_sync(FULL, hasB ? bb : ba, src);
            if (tg.colState && !tg.runs && j + 2 >= nSeg && lz == kTZ - 1) {
                // the column's last tile: its top layer passes its closest triangles to the column above
                const uint32_t sz = uint32_t(zBase - g.z0) / uint32_t(tg.segLen * kTZ);
                const uint32_t it = uint32_t(x0) / kTX + uint32_t(tg.tilesX) * (uint32_t(y0) / kTY + uint32_t(tg.tilesY) * sz);
                float* cs = tg.colState + size_t(it) * (2 * kLayer) + (lane - (kTZ - 1) * kLayer);
                cs[0] = __int_as_float(0x7fc00000);
                cs[kLayer] = __int_as_float(seed);
            }
        }
    }
}

// Winding numbers of a grid two tiles at a time (fwnPacket2): each lane takes its voxel of the lower
// tile and the one kTZ layers above; the same values as gridKernel<PRECISE, false>, bit for bit.
// 4 blocks per SM (64 registers): at 512^3 on 1.31 M triangles 19.7 ms, against 20.7 ms at 3 and
// 29.6 ms at 5 (spills).
template <bool PRECISE>
__global__ void __launch_bounds__(kThreads, 4) gridFwnPairKernel(QueryTree t, GridRange g, TileGrid tg, Xf xf, float beta,
                                                                 float* __restrict__ out, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const int lx = lane % kTX, ly = (lane / kTX) % kTY, lz = lane / (kTX * kTY);
    const float betaSq = __fmul_rn(beta, beta);
    const size_t sxy = size_t(g.nx) * g.ny;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (item >= tg.numItems) break;
        const int tx = int(item % unsigned(tg.tilesX));
        const unsigned rest = item / unsigned(tg.tilesX);
        const int ty = int(rest % unsigned(tg.tilesY));
        const int sz = int(rest / unsigned(tg.tilesY));
        const int x = tx * kTX + lx, y = ty * kTY + ly;
        const int zBase = g.z0 + sz * tg.segLen * kTZ;
        const int nSeg = min(tg.segLen, tg.tilesZ - sz * tg.segLen);
        for (int j = 0; j < nSeg; j += 2) {
            const int za = zBase + j * kTZ + lz, zb = za + kTZ;
            const bool inXY = x < g.nx && y < g.ny;
            const bool activeA = inXY && za < g.z1, activeB = inXY && j + 1 < nSeg && zb < g.z1;
            float wa, wb;
            fwnPacket2<PRECISE>(t, xfPoint(xf, x, y, za), xfPoint(xf, x, y, zb), activeA, activeB, betaSq, scratch + 1, &wa, &wb);
            if (activeA) out[size_t(za - g.zOut) * sxy + size_t(y) * g.nx + x] = wa;
            if (activeB) out[size_t(zb - g.zOut) * sxy + size_t(y) * g.nx + x] = wb;
        }
    }
}

// Winding numbers of spatially ordered points, two tiles of 32 per work item (fwnPacket2): lane i takes
// the i-th point of each tile; the same values as vectorKernel<PRECISE, false>, bit for bit.
template <bool PRECISE>
__global__ void __launch_bounds__(kThreads, 4) vectorFwnPairKernel(QueryTree t, const float* __restrict__ pts, int64_t n,
                                                                   float beta, float* __restrict__ out, unsigned* scratch,
                                                                   const int32_t* __restrict__ order) {
    const int lane = threadIdx.x & 31;
    const float betaSq = __fmul_rn(beta, beta);
    const uint64_t numPairs = (uint64_t(n) + 63) / 64;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (item >= numPairs) break;
        const int64_t ra = int64_t(item) * 64 + lane, rb = ra + 32;  // ranks in processing order
        const bool activeA = ra < n, activeB = rb < n;
        const int64_t ia = activeA ? int64_t(order[ra]) : 0, ib = activeB ? int64_t(order[rb]) : 0;
        float3 qa = make_float3(0.f, 0.f, 0.f), qb = qa;
        if (activeA) qa = make_float3(pts[3 * ia], pts[3 * ia + 1], pts[3 * ia + 2]);
        if (activeB) qb = make_float3(pts[3 * ib], pts[3 * ib + 1], pts[3 * ib + 2]);
        float wa, wb;
        fwnPacket2<PRECISE>(t, qa, qb, activeA, activeB, betaSq, scratch + 1, &wa, &wb);
        if (activeA) out[ia] = wa;
        if (activeB) out[ib] = wb;
    }
}

// The listed pair steps of a precise gridPairKernel launch: each flagged voxel's closest distance by
// the precise walk (cpPacket, from maxDistSq), written with its sign bit.  Voxels never listed kept
// FP32 distances no triangle came near the FP64 re-evaluation for: the precise walk's own.  A list
// that overflowed (more flagged steps than a launch has) cannot happen: one entry per step at most.
__global__ void __launch_bounds__(kThreads) fixPairKernel(QueryTree t, GridRange g, TileGrid tg, Xf xf, DistOpts o,
                                                          float* __restrict__ out, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const int lx = lane % kTX, ly = (lane / kTX) % kTY, lz = lane / (kTX * kTY);
    const size_t sxy = size_t(g.nx) * g.ny;
    const int wordsX = (g.nx + 31) >> 5;
    const uint32_t n = min(__ldcg(&tg.fixList[0].x), tg.fixCap);
    for (;;) {
        const unsigned e = nextTicket(scratch, lane);
        if (e >= n) break;
        const uint4 f = tg.fixList[1 + e];
        const unsigned item = f.x;
        int x0, y0, zBase;
        if (tg.runs) {
            const int4 r = tg.runs[item / kBrickCols];
            const int col = int(item % kBrickCols);
            x0 = r.x * 8 + (col % kBrickColsX) * kTX;
            y0 = r.y * 8 + (col / kBrickColsX) * kTY;
            zBase = g.z0 + r.z * 8;
        } else {
            const unsigned rest = item / unsigned(tg.tilesX);
            x0 = int(item % unsigned(tg.tilesX)) * kTX;
            y0 = int(rest % unsigned(tg.tilesY)) * kTY;
            zBase = g.z0 + int(rest / unsigned(tg.tilesY)) * tg.segLen * kTZ;
        }
        const int x = x0 + lx, y = y0 + ly;
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
            const bool need = ((h ? f.w : f.z) >> lane) & 1u;
            if (!__any_sync(FULL, need)) continue;
            const int z = zBase + (int(f.y) + h) * kTZ + lz;
            const float3 q = xfPoint(xf, x, y, z);
            const float dsq = cpPacket<true>(t, q, need, o.maxDistSq, 0.f, scratch + 1);
            if (need) {
                const bool valid = !(o.nullOutsideMinMax && dsq >= o.maxDistSq);
                const uint32_t word = __ldg(tg.signBits + (size_t(z - g.zOut) * g.ny + y) * wordsX + (x >> 5));
                const float d = __fsqrt_rn(dsq);
                out[size_t(z - g.zOut) * sxy + size_t(y) * g.nx + x] =
                    valid ? (((word >> (x & 31)) & 1u) ? -d : d) : __int_as_float(0x7fc00000);
            }
        }
    }
}

// A warp takes `chunk` consecutive tiles of 32 points; with Morton-ordered points a lane's point in
// one tile is near its point in the previous one, so (as in gridKernel) each lane starts its
// closest-point search from the triangle closest to its previous point.
template <bool PRECISE, bool DIST>
__global__ void __launch_bounds__(kThreads, DIST ? kDistBlocks : 4) vectorKernel(QueryTree t, const float* __restrict__ pts, int64_t n, DistOpts o,
                                                         int32_t skipFace, float* __restrict__ out, unsigned* scratch,
                                                         const int32_t* __restrict__ order, int chunk) {
    const int lane = threadIdx.x & 31;
    const float betaSq = __fmul_rn(o.beta, o.beta);
    const int skipSlot = (skipFace >= 0 && skipFace < t.nFaces) ? t.faceSlot[skipFace] : -1;
    const uint64_t numTiles = (uint64_t(n) + 31) / 32;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (uint64_t(item) * chunk >= numTiles) break;
        int seed = -1;
        for (int j = 0; j < chunk; ++j) {
            const uint64_t tile = uint64_t(item) * chunk + j;
            if (tile >= numTiles) break;
            const int64_t r = int64_t(tile) * 32 + lane;  // rank in processing order
            const bool active = r < n;
            const int64_t i = (order && active) ? int64_t(order[r]) : r;
            float3 q = make_float3(0.f, 0.f, 0.f);
            if (active) q = make_float3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
            float res;
            if (DIST) {
                float up = o.maxDistSq;
                if (active && seed >= 0) {
                    const float4* tr = t.tri + 3 * int64_t(seed);
                    const float ds = triDistSq<PRECISE>(q, ld4(tr), ld4(tr + 1), ld4(tr + 2));
                    if (ds < up) up = ds;
                }
                int best = active ? seed : -1;
                const float dsq = cpPacket<PRECISE, true>(t, q, active, up, o.minDistSq, scratch + 1, &best);
                seed = best;
                const bool valid = !(o.nullOutsideMinMax && (dsq < o.minDistSq || dsq >= o.maxDistSq));
                // closed surfaces: the exact winding number from ray crossings (gridKernel)
                bool onSurface = false;
                const bool rays = signReuseAllowed(t, o);
                const int cw = rays ? rayWinding(t, q, active && valid, scratch + 1, &onSurface) : 0;
                const bool fwn = rays ? onSurface : (active && valid);
                const float w = fwnPacket<PRECISE>(t, q, fwn, betaSq, -1, scratch + 1);
                const bool inside = fwn ? w > o.threshold : float(cw) > o.threshold;
                const float d = __fsqrt_rn(dsq);
                res = valid ? (inside ? -d : d) : __int_as_float(0x7fc00000);
            } else {
                res = fwnPacket<PRECISE>(t, q, active, betaSq, skipSlot, scratch + 1);
            }
            if (active) out[i] = res;
        }
    }
}

// Closest point with barycentric coordinates, FP64 (MRMesh/MRClosestPointInTriangle.h:28-91, in
// double as MRMesh/MRMeshProject.cpp:66-72 calls it): proj = (1 - ba - bb) a + ba b + bb c.
__device__ __noinline__ void closestPointBaryFp64(const float3 p, const float4 A, const float4 B, const float4 C, float3* proj,
                                                  float* ba, float* bb) {
    using V = V3T<double>;
    const V pd{p.x, p.y, p.z}, a{A.x, A.y, A.z}, b{B.x, B.y, B.z}, c{C.x, C.y, C.z};
    const V ab = vsub(b, a), ac = vsub(c, a), ap = vsub(pd, a);
    V r;
    double u = 0, w = 0;
    const double d1 = vdot(ab, ap), d2 = vdot(ac, ap);
    const V bp = vsub(pd, b);
    const double d3 = vdot(ab, bp), d4 = vdot(ac, bp);
    const V cp = vsub(pd, c);
    const double d5 = vdot(ab, cp), d6 = vdot(ac, cp);
    const double vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
    if (d1 <= 0 && d2 <= 0) {
        r = a;
    } else if (d3 >= 0 && d4 <= d3) {
        r = b;
        u = 1;
    } else if (d6 >= 0 && d5 <= d6) {
        r = c;
        w = 1;
    } else if (vc <= 0 && d1 >= 0 && d3 <= 0) {
        u = d1 / (d1 - d3);
        r = vmad(a, u, ab);
    } else if (vb <= 0 && d6 <= 0 && d2 >= 0) {
        w = d2 / (d2 - d6);
        r = vmad(a, w, ac);
    } else if (va <= 0) {
        if (d4 < d3) {
            r = b;
            u = 1;
        } else if (d5 < d6) {
            r = c;
            w = 1;
        } else {
            const double v = (d4 - d3) / ((d4 - d3) + (d5 - d6));
            r = vmad(b, v, vsub(c, b));
            u = 1 - v;
            w = v;
        }
    } else {
        const double denom = 1 / (va + vb + vc);
        u = vb * denom;
        w = vc * denom;
        r = vmad(vmad(a, u, ab), w, ac);
    }
    *proj = make_float3(float(r.x), float(r.y), float(r.z));
    *ba = float(u);
    *bb = float(w);
}

// Points-to-mesh projection (MRMesh/MRPointsToMeshProjector.cpp:17-32 over MRMeshProject.cpp:13-104;
// the GPU counterpart is MRCuda/MRCudaPointsToMeshProjector.cu:6-111).  Each point is mapped by pxf
// (when given), the packet search finds the nearest triangle (FP32, FP64 near the surface in
// precise mode), and the winner's projection, barycentrics and distance are recomputed in FP64 and
// rounded as the reference CPU does.  Output per point, the layout of MR::MeshProjectionResult:
// {face, proj.xyz} {edge = -1, bary a, bary b, distSq}; face = -1 when nothing lies closer than up.
template <bool PRECISE, bool TREEXF>
__global__ void __launch_bounds__(kThreads, kDistBlocks) projectKernel(QueryTree t, const float* __restrict__ pts, int64_t n, Xf pxf,
                                                          int hasPxf, Xf txf, float up, float lo, float4* __restrict__ out,
                                                          unsigned* scratch, const int32_t* __restrict__ order, int chunk) {
    const int lane = threadIdx.x & 31;
    const uint64_t numTiles = (uint64_t(n) + 31) / 32;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (uint64_t(item) * chunk >= numTiles) break;
        int seed = -1;  // leaf slot closest to this lane's previous point (see vectorKernel)
        for (int jt = 0; jt < chunk; ++jt) {
            const uint64_t tile = uint64_t(item) * chunk + jt;
            if (tile >= numTiles) break;
            const int64_t r = int64_t(tile) * 32 + lane;
            const bool active = r < n;
            const int64_t i = (order && active) ? int64_t(order[r]) : r;
            float3 q = make_float3(0.f, 0.f, 0.f);
            if (active) {
                q = make_float3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
                if (hasPxf) q = xfApply(pxf, q.x, q.y, q.z);
            }
            // start from the previous point's triangle when it lies within the limit: its distance is
            // one the search would reach anyway, so the minimum and the reported face are unchanged
            float upS = up;
            bool seeded = false;
            if (active && seed >= 0) {
                const float4* tr = t.tri + 3 * int64_t(seed);
                float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
                if (TREEXF) {
                    xfTri(&txf, A, B, C);
                }
                const float ds = triDistSq<PRECISE>(q, A, B, C);
                if (ds < upS) {
                    upS = ds;
                    seeded = true;
                }
            }
            int best = seeded ? seed : -1;
            const float dsq = cpPacket<PRECISE, true, TREEXF>(t, q, active, upS, lo, scratch + 1, &best, &txf);
            seed = best;
            if (!active) best = -2;
            float4 o0 = make_float4(__int_as_float(-1), 0.f, 0.f, 0.f), o1 = make_float4(__int_as_float(-1), 0.f, 0.f, dsq);
            if (best >= 0) {
                const float4* tr = t.tri + 3 * int64_t(best);
                float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
                if (TREEXF) {
                    xfTri(&txf, A, B, C);
                }
                float3 pr;
                float ba, bb;
                closestPointBaryFp64(q, A, B, C, &pr, &ba, &bb);
                const float dx = pr.x - q.x, dy = pr.y - q.y, dz = pr.z - q.z;
                o0 = make_float4(A.w, pr.x, pr.y, pr.z);
                o1 = make_float4(__int_as_float(-1), ba, bb, dot3rn(dx, dy, dz, dx, dy, dz));
            }
            if (active) {
                out[2 * i] = o0;
                out[2 * i + 1] = o1;
            }
        }
    }
}

// MRMesh/MRFastWindingNumber.cpp:40-52: query = triCenter(f) = (1/3) * (v0 + v1 + v2), skipping f.
// Lanes take consecutive leaf slots, which are spatially coherent.
template <bool PRECISE>
__global__ void __launch_bounds__(kThreads, 4) selfIntKernel(QueryTree t, float beta, uint64_t* __restrict__ bits,
                                                          float* __restrict__ wn, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const float betaSq = __fmul_rn(beta, beta);
    const uint64_t numTiles = (uint64_t(t.nLeaves) + 31) / 32;
    const bool rays = t.closed != 0 && beta >= 2.f && !wn;  // see below
    for (;;) {
        const unsigned tile = nextTicket(scratch, lane);
        if (tile >= numTiles) break;
        const int slot = int(tile) * 32 + lane;
        const bool active = slot < t.nLeaves;
        float3 q = make_float3(0.f, 0.f, 0.f);
        int face = -1;
        if (active) {
            const float4* tr = t.tri + 3 * int64_t(slot);
            const float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
            const float third = 1 / 3.0f;
            q = make_float3(__fmul_rn(third, __fadd_rn(__fadd_rn(A.x, B.x), C.x)),
                            __fmul_rn(third, __fadd_rn(__fadd_rn(A.y, B.y), C.y)),
                            __fmul_rn(third, __fadd_rn(__fadd_rn(A.z, B.z), C.z)));
            face = __float_as_int(A.w);
        }
        // Closed surfaces, bits only: the ray from the centroid that ignores its own face counts the
        // exact winding number on the side of the face the ray leaves into; the other side differs by
        // one, by the face's orientation.  The reference's value (its own face skipped) lies halfway,
        // so the face is flagged when the smaller side is <= -1 or >= 1.  A face whose centroid does
        // not fall strictly inside its own projection (near-vertical or degenerate), or that lies on
        // another face, gets the approximated winding number as before.
        bool fwn = active, flag = false;
        if (rays) {
            int orient = 0;  // the sign of the face normal's z, exact
            if (active) {
                const float4* tr = t.tri + 3 * int64_t(slot);
                const float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
                const float ax = __fsub_rn(A.x, q.x), ay = __fsub_rn(A.y, q.y), bx = __fsub_rn(B.x, q.x),
                            by = __fsub_rn(B.y, q.y), cx = __fsub_rn(C.x, q.x), cy = __fsub_rn(C.y, q.y);
                const int e0 = edgeSign(bx, by, cx, cy), e1 = edgeSign(cx, cy, ax, ay), e2 = edgeSign(ax, ay, bx, by);
                if (e0 != 0 && e0 == e1 && e1 == e2) orient = e0;
            }
            bool onSurface = false, up = true;
            const int wd = rayWinding(t, q, active && orient != 0, scratch + 1, &onSurface, active ? slot : -1, &up);
            fwn = active && (orient == 0 || onSurface);
            if (active && !fwn) {
                const int a = up ? orient : -orient;  // +1: the face's normal points along the ray
                const int m = a > 0 ? wd : wd + a;    // the smaller of the two sides, wd and wd + a
                flag = m <= -1 || m >= 1;
            }
        }
        const float w = fwnPacket<PRECISE>(t, q, fwn, betaSq, active ? slot : -1, scratch + 1);
        if (active) {
            if (wn) wn[face] = w;
            if (fwn ? (w < 0.f || w > 1.f) : flag) atomicOr((unsigned long long*)bits + (face >> 6), 1ull << (face & 63));
        }
    }
}

}  // namespace

int numSMs() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

uint64_t gridTiles(int32_t nx, int32_t ny, int32_t nz) {
    return uint64_t((nx + kTX - 1) / kTX) * uint64_t((ny + kTY - 1) / kTY) * uint64_t((nz + kTZ - 1) / kTZ);
}

static TileGrid tileGridFor(const GridRange& g, int maxSegLen = 16) {
    TileGrid tg;
    tg.tilesX = (g.nx + kTX - 1) / kTX;
    tg.tilesY = (g.ny + kTY - 1) / kTY;
    tg.tilesZ = (g.z1 - g.z0 + kTZ - 1) / kTZ;
    tg.numTiles = uint32_t(uint64_t(tg.tilesX) * tg.tilesY * tg.tilesZ);
    tg.runs = nullptr;
    tg.colState = nullptr;
    tg.signBits = nullptr;
    tg.fixList = nullptr;
    tg.fixCap = 0;
    // Longer columns reuse more seeds; shorter ones leave more items for the tail of the persistent
    // grid.  Measured at 256^3 / 512^3 on 1.3 M triangles: keep >= 25 items per (32-warps-per-SM)
    // resident warp, and columns of at most 32 tiles for unbanded signed distances (512^3: 16 tiles
    // +0.7 %, 64 +1 %) but 16 otherwise (banded requests, where the cost sits in the voxels near the
    // surface: 32 tiles made a 512^3 band 10 % slower).
    const uint64_t cols = uint64_t(tg.tilesX) * tg.tilesY;
    const uint64_t warps = uint64_t(numSMs()) * 4 * (kThreads / 32);
    tg.segLen = maxSegLen;
    while (tg.segLen > 1 && cols * uint64_t((tg.tilesZ + tg.segLen - 1) / tg.segLen) < 25 * warps) tg.segLen /= 2;
    tg.segsZ = (tg.tilesZ + tg.segLen - 1) / tg.segLen;
    tg.numItems = uint32_t(cols * tg.segsZ);
    return tg;
}

// Entries of the precise paired walk's fix list (after its counter): one per pair step at most.
static uint32_t pairFixCap(const TileGrid& tg) { return tg.numTiles / 2 + tg.numItems + 1; }

size_t pairFixBytes(uint32_t nTiles, uint32_t nItems) { return size_t(nTiles / 2 + nItems + 2) * sizeof(uint4); }
size_t pairFixBytesForRuns(int32_t nRuns, int32_t nBricks) {
    return pairFixBytes(uint32_t(nBricks) * 16u, uint32_t(nRuns) * uint32_t(kBrickCols));
}

// The signed distances of a grid (or of brick runs) with the column bits: the paired walk when there
// is no lower distance bound and the work items hold at least four tiles (in precise mode with its
// fix list, when given, and the fix-up pass), else the one-voxel walk.  Small grids get one-tile
// items (enough items for the persistent grid), which leave the pairs nothing to share: measured on
// the 1.31 M-triangle mesh, 128^3 4.8 ms one-voxel against 6.6 ms paired, 256^3 (4-tile items)
// 16.7 against 16.4 ms, 512^3 (32-tile items) 73.6 against 66.1 ms.
static cudaError_t launchWithBits(const QueryTree& t, const GridRange& g, TileGrid tg, const Xf& xf, const DistOpts& o, int precise,
                                  float* out, uint4* fix, unsigned* scratch, cudaStream_t s) {
    if (o.minDistSq <= 0.f && (tg.runs || tg.segLen >= 4) && (!precise || fix)) {
        if (!precise) return launchPersistent(gridPairKernel<false>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
        tg.fixList = fix;
        tg.fixCap = pairFixCap(tg);
        cudaError_t e = cudaMemsetAsync(fix, 0, sizeof(uint4), s);
        if (e || (e = launchPersistent(gridPairKernel<true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch))) return e;
        return launchPersistent(fixPairKernel, tg.fixCap, scratch, s, t, g, tg, xf, o, out, scratch);
    }
    if (precise) return launchPersistent(gridKernel<true, true, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
    return launchPersistent(gridKernel<false, true, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
}

cudaError_t launchGridSdfBricks(const QueryTree& t, const GridRange& g, const Xf& xf, const DistOpts& o, int precise,
                                float* out, const int4* runs, int32_t nRuns, int32_t nBricks, const uint32_t* signBits,
                                void* fix, unsigned* scratch, cudaStream_t s) {
    TileGrid tg = tileGridFor(g);
    tg.runs = runs;
    tg.numTiles = uint32_t(nBricks) * 16u;
    tg.numItems = uint32_t(nRuns) * uint32_t(kBrickCols);
    if (signBits) {
        tg.signBits = signBits;
        return launchWithBits(t, g, tg, xf, o, precise, out, static_cast<uint4*>(fix), scratch, s);
    }
    if (precise)
        return launchPersistent(gridKernel<true, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
    return launchPersistent(gridKernel<false, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
}




cudaError_t launchGridFwn(const QueryTree& t, const GridRange& g, const Xf& xf, float beta, int precise, float* out,
                          unsigned* scratch, cudaStream_t s) {
    const TileGrid tg = tileGridFor(g);
    if (tg.segLen >= 2) {  // work items of two or more tiles: the paired walk
        if (precise) return launchPersistent(gridFwnPairKernel<true>, tg.numItems, scratch, s, t, g, tg, xf, beta, out, scratch);
        return launchPersistent(gridFwnPairKernel<false>, tg.numItems, scratch, s, t, g, tg, xf, beta, out, scratch);
    }
    DistOpts o{0.f, FLT_MAX, 0, 0.5f, beta};
    if (precise)
        return launchPersistent(gridKernel<true, false>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
    return launchPersistent(gridKernel<false, false>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
}

// Column hand-over words, then (when the column rays apply) the inside bits of the range.

size_t gridSdfColumnStateBytes(const QueryTree& t, const GridRange& g, const Xf& xf, const DistOpts& o) {
    const TileGrid tg = tileGridFor(g, o.maxDistSq >= FLT_MAX ? 32 : 16);
    const size_t col = size_t(tg.numItems) * (2 * kLayer) * sizeof(float);
    if (!signColumnsApply(t, xf, o.beta, o.threshold)) return col;
    return col + ((signBitsBytes(g) + 255) & ~size_t(255)) + signColumnsWorkBytes(g) +
           (o.minDistSq <= 0.f ? pairFixBytes(tg.numTiles, tg.numItems) : 0);
}


cudaError_t launchGridSdf(const QueryTree& t, const GridRange& g, const Xf& xf, const DistOpts& o, int precise, float* out,
                          unsigned* scratch, cudaStream_t s, float* colState, size_t colBytes) {
    TileGrid tg = tileGridFor(g, o.maxDistSq >= FLT_MAX ? 32 : 16);
    const size_t need = size_t(tg.numItems) * (2 * kLayer) * sizeof(float);
    if (colState && colBytes >= need && need > 0) {
        cudaError_t e = cudaMemsetAsync(colState, 0xff, need, s);
        if (e) return e;
        tg.colState = colState;
        if (signColumnsApply(t, xf, o.beta, o.threshold) && colBytes >= need + signBitsBytes(g)) {
            // closed surface, vertical z axis: the signs from the columns' crossings first
            char* base = reinterpret_cast<char*>(colState);
            uint32_t* bits = reinterpret_cast<uint32_t*>(base + need);
            const size_t lists = need + ((signBitsBytes(g) + 255) & ~size_t(255));
            void* work = colBytes >= lists + signColumnsWorkBytes(g) ? base + lists : nullptr;
            if ((e = launchSignColumns(t, g, xf, o.beta, o.threshold, precise, bits, nullptr, work, work ? colBytes - lists : 0,
                                       scratch, s)))
                return e;
            tg.signBits = bits;
            const size_t fixAt = lists + signColumnsWorkBytes(g);
            uint4* fix = (work && colBytes >= fixAt + pairFixBytes(tg.numTiles, tg.numItems))
                             ? reinterpret_cast<uint4*>(base + fixAt)
                             : nullptr;
            return launchWithBits(t, g, tg, xf, o, precise, out, fix, scratch, s);
        }
    }
    if (precise)
        return launchPersistent(gridKernel<true, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
    return launchPersistent(gridKernel<false, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
}

// Tiles of 32 points per work item for the seeded point searches: only with a spatial order, and
// while at least 32 items per resident warp remain.  Morton-ordered point sets can hold long runs of
// expensive queries (points far from the surface), so the work items must stay small: with 5 M
// points (4 M near the surface, 1 M spread over the box) and 4 tiles per item the projection took
// 11.8 ms instead of 9.2 ms; at that size the rule below keeps one tile per item.
static int pointChunk(uint64_t tiles, const int32_t* order) {
    if (!order) return 1;
    const uint64_t warps = uint64_t(numSMs()) * 4 * (kThreads / 32);
    int k = 8;
    while (k > 1 && (tiles + k - 1) / k < 32 * warps) k /= 2;
    return k;
}

cudaError_t launchVectorFwn(const QueryTree& t, const float* pts, int64_t n, float beta, int32_t skipFace, int precise,
                            float* out, unsigned* scratch, cudaStream_t s, const int32_t* order) {
    DistOpts o{0.f, FLT_MAX, 0, 0.5f, beta};
    const uint64_t tiles = (uint64_t(n) + 31) / 32;
    if (order && skipFace < 0) {  // spatially ordered points, no face skipped: two tiles per walk
        const uint64_t pairs = (tiles + 1) / 2;
        if (precise) return launchPersistent(vectorFwnPairKernel<true>, pairs, scratch, s, t, pts, n, beta, out, scratch, order);
        return launchPersistent(vectorFwnPairKernel<false>, pairs, scratch, s, t, pts, n, beta, out, scratch, order);
    }
    if (precise)
        return launchPersistent(vectorKernel<true, false>, tiles, scratch, s, t, pts, n, o, skipFace, out, scratch, order, 1);
    return launchPersistent(vectorKernel<false, false>, tiles, scratch, s, t, pts, n, o, skipFace, out, scratch, order, 1);
}

cudaError_t launchVectorSdf(const QueryTree& t, const float* pts, int64_t n, const DistOpts& o, int precise, float* out,
                            unsigned* scratch, cudaStream_t s, const int32_t* order) {
    const uint64_t tiles = (uint64_t(n) + 31) / 32;
    const int k = pointChunk(tiles, order);
    const uint64_t items = (tiles + k - 1) / k;
    if (precise) return launchPersistent(vectorKernel<true, true>, items, scratch, s, t, pts, n, o, -1, out, scratch, order, k);
    return launchPersistent(vectorKernel<false, true>, items, scratch, s, t, pts, n, o, -1, out, scratch, order, k);
}

cudaError_t launchProject(const QueryTree& t, const float* pts, int64_t n, const Xf* pointXf, const Xf* treeXf, float upSq,
                          float loSq, int precise, float4* out, unsigned* scratch, cudaStream_t s, const int32_t* order) {
    const uint64_t tiles = (uint64_t(n) + 31) / 32;
    const int k = pointChunk(tiles, order);
    const uint64_t items = (tiles + k - 1) / k;
    const Xf id{{1, 0, 0, 0, 1, 0, 0, 0, 1}, {0, 0, 0}};
    const Xf px = pointXf ? *pointXf : id, tx = treeXf ? *treeXf : id;
    const int hp = pointXf ? 1 : 0;
    if (treeXf) {
        if (precise)
            return launchPersistent(projectKernel<true, true>, items, scratch, s, t, pts, n, px, hp, tx, upSq, loSq, out, scratch, order, k);
        return launchPersistent(projectKernel<false, true>, items, scratch, s, t, pts, n, px, hp, tx, upSq, loSq, out, scratch, order, k);
    }
    if (precise)
        return launchPersistent(projectKernel<true, false>, items, scratch, s, t, pts, n, px, hp, tx, upSq, loSq, out, scratch, order, k);
    return launchPersistent(projectKernel<false, false>, items, scratch, s, t, pts, n, px, hp, tx, upSq, loSq, out, scratch, order, k);
}

cudaError_t launchSelfIntersections(const QueryTree& t, float beta, int precise, uint64_t* bits, float* wn,
                                    unsigned* scratch, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bits, 0, sizeof(uint64_t) * size_t((t.nFaces + 63) / 64), s);
    if (e) return e;
    if (wn && t.nFaces > 0) {
        fillNan<<<unsigned((t.nFaces + 255) / 256), 256, 0, s>>>(wn, t.nFaces);
        if ((e = cudaGetLastError())) return e;
    }
    const uint64_t tiles = (uint64_t(t.nLeaves) + 31) / 32;
    if (precise) return launchPersistent(selfIntKernel<true>, tiles, scratch, s, t, beta, bits, wn, scratch);
    return launchPersistent(selfIntKernel<false>, tiles, scratch, s, t, beta, bits, wn, scratch);
}

// ------------------------------------------------------------------ batched meshes
// Many meshes, each with its own grid, in one persistent launch: the tiles of all grids form one
// ticket sequence (item i owns tickets [tileBase_i, tileBase_{i+1})); a warp takes a ticket, finds
// its item by binary search, and runs the same packet traversals on that item's tree.  Items are
// ordered by estimated cost, most expensive first, so the long grids start early and the short
// ones fill the tail.  Tile shape (TX x TY x TZ = 32 voxels) and block size are template
// parameters chosen by the autotuner.
namespace {

template <bool PRECISE, int TX, int TY, int TZ, int THREADS>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) batchKernel(const BatchItem* __restrict__ items, int nItems, uint32_t totalTiles,
                                                       unsigned* scratch) {
    static_assert(TX * TY * TZ == 32, "one voxel per lane");
    const int lane = threadIdx.x & 31;
    const int lx = lane % TX, ly = (lane / TX) % TY, lz = lane / (TX * TY);
    for (;;) {
        const unsigned ticket = nextTicket(scratch, lane);
        if (ticket >= totalTiles) break;
        int lo = 0, hi = nItems - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].tileBase <= ticket) lo = mid; else hi = mid - 1;
        }
        // the item (tree, grid, transform, options: ~210 bytes) is staged in this warp's shared-memory
        // slot and read from there, instead of living in registers for the whole column walk
        // (measured 78.1 -> 74.9 ms on the 64-mesh batch)
        __shared__ BatchItem sItem[THREADS / 32];
        BatchItem& it = sItem[threadIdx.x >> 5];
        {
            static_assert(sizeof(BatchItem) % 4 == 0, "copied as 32-bit words");
            const uint32_t* src = reinterpret_cast<const uint32_t*>(items + lo);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&it);
            __syncwarp();  // every lane is done with the previous item
            for (int k = lane; k < int(sizeof(BatchItem) / 4); k += 32) dst[k] = src[k];
            __syncwarp();
        }
        // a ticket is a column of up to kBatchSeg tiles along z, walked upwards with each lane's
        // closest-point search seeded by its previous voxel's triangle (as gridKernel does)
        const unsigned local = ticket - it.tileBase;
        const int tilesX = (it.g.nx + TX - 1) / TX, tilesY = (it.g.ny + TY - 1) / TY;
        const int tx = int(local % unsigned(tilesX));
        const unsigned rest = local / unsigned(tilesX);
        const int ty = int(rest % unsigned(tilesY)), seg = int(rest / unsigned(tilesY));
        const int x = tx * TX + lx, y = ty * TY + ly;
        const QueryTree& t = it.t;  // read through the cache, not copied into registers
        const DistOpts o = it.o;
        const bool reuseOk = signReuseAllowed(t, o);
        int seed = -1;
        float below = __int_as_float(0x7fc00000);  // the preceding voxel's signed squared distance (gridKernel)
        for (int j = 0; j < kBatchSeg; ++j) {
            const int z0 = (seg * kBatchSeg + j) * TZ;
            if (z0 >= it.g.nz) break;
            const int z = z0 + lz;
            const bool active = x < it.g.nx && y < it.g.ny && z < it.g.nz;
            const float3 q = xfPoint(it.xf, x, y, z);
            float up = o.maxDistSq;
            if (active && seed >= 0) {
                const float4* tr = t.tri + 3 * int64_t(seed);
                const float ds = triDistSq<PRECISE>(q, ld4(tr), ld4(tr + 1), ld4(tr + 2));
                if (ds < up) up = ds;
            }
            int best = active ? seed : -1;
            const float dsq = cpPacket<PRECISE, true>(t, q, active, up, o.minDistSq, scratch + 1, &best);
            const bool valid = !(o.nullOutsideMinMax && (dsq < o.minDistSq || dsq >= o.maxDistSq));
            const bool complete = active && valid && dsq >= o.minDistSq;
            bool reIn = false;
            const bool reuse = reuseOk && reuseSign<TX, TY, TZ>(it.xf, x, y, z, z - (lz == 0 ? 1 : TZ), lz, q, below, complete,
                                                                dsq, &reIn);
            bool onSurface = false;  // as gridKernel: ray crossings on closed surfaces
            const int cw = reuseOk ? rayWinding(t, q, active && valid && !reuse, scratch + 1, &onSurface) : 0;
            const bool fwn = reuseOk ? onSurface : (active && valid);
            const float w = fwnPacket<PRECISE>(t, q, fwn, __fmul_rn(o.beta, o.beta), -1, scratch + 1);
            const bool inside = reuse ? reIn : (fwn ? w > o.threshold : float(cw) > o.threshold);
            const float d = __fsqrt_rn(dsq);
            const float res = valid ? (inside ? -d : d) : __int_as_float(0x7fc00000);
            if (active) it.out[(size_t(z) * it.g.ny + y) * it.g.nx + x] = res;
            // the bottom layer's lanes continue from the voxel one layer below (as gridKernel does)
            const int src = lane + (TZ - 1) * TX * TY * (lz == 0);
            seed = __shfl_sync(FULL, best, src);
            below = __shfl_sync(FULL, complete ? (inside ? -dsq : dsq) : __int_as_float(0x7fc00000), src);
        }
    }
}

// The item of a ticket of a batched launch (binary search over the items' first tickets).
__device__ __forceinline__ int batchItemOf(const BatchItem* __restrict__ items, int nItems, unsigned ticket) {
    int lo = 0, hi = nItems - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (items[mid].tileBase <= ticket) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// batchKernel with the paired walk (gridPairKernel's): the column of a ticket two tiles at a time,
// each lane taking its voxel of the lower tile and the one TZ layers above through one packet walk
// (cpPacket2), then the lower voxel's sign and the upper one's from it (the voxel below each, as in
// batchKernel: sign reuse, rays, the winding-number walk).  Only for batches without a lower
// distance bound (minDistSq = 0 in every item).  In precise mode the walk runs in FP32 and the pair
// steps whose voxels came within a triangle's near-plane level are listed ({ticket, first tile, lane
// masks}) for fixBatchKernel.
template <bool PRECISE, int TX, int TY, int TZ, int THREADS>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) batchPairKernel(const BatchItem* __restrict__ items, int nItems,
                                                                           uint32_t totalTiles, uint4* fix, uint32_t fixCap,
                                                                           unsigned* scratch) {
    static_assert(TX * TY * TZ == 32, "one voxel per lane");
    static_assert(THREADS / 32 <= 8, "one sPairFix row per warp");
    const int lane = threadIdx.x & 31;
    const int lx = lane % TX, ly = (lane / TX) % TY, lz = lane / (TX * TY);
    for (;;) {
        const unsigned ticket = nextTicket(scratch, lane);
        if (ticket >= totalTiles) break;
        const int lo = batchItemOf(items, nItems, ticket);
        __shared__ BatchItem sItem[THREADS / 32];
        BatchItem& it = sItem[threadIdx.x >> 5];
        {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(items + lo);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&it);
            __syncwarp();
            for (int k = lane; k < int(sizeof(BatchItem) / 4); k += 32) dst[k] = src[k];
            __syncwarp();
        }
        const unsigned local = ticket - it.tileBase;
        const int tilesX = (it.g.nx + TX - 1) / TX, tilesY = (it.g.ny + TY - 1) / TY;
        const int tx = int(local % unsigned(tilesX));
        const unsigned rest = local / unsigned(tilesX);
        const int ty = int(rest % unsigned(tilesY)), seg = int(rest / unsigned(tilesY));
        const int x = tx * TX + lx, y = ty * TY + ly;
        const QueryTree& t = it.t;
        const DistOpts o = it.o;
        const bool reuseOk = signReuseAllowed(t, o);
        const bool vertical = it.xf.a[2] == 0.f && it.xf.a[5] == 0.f;
        const float betaSq = __fmul_rn(o.beta, o.beta);
        int seed = -1;
        float below = __int_as_float(0x7fc00000);
        for (int j = 0; j < kBatchSeg; j += 2) {
            const int zA0 = (seg * kBatchSeg + j) * TZ;
            if (zA0 >= it.g.nz) break;
            const bool hasB = j + 1 < kBatchSeg && zA0 + TZ < it.g.nz;
            const int za = zA0 + lz, zb = za + TZ;
            const bool inXY = x < it.g.nx && y < it.g.ny;
            const bool activeA = inXY && za < it.g.nz, activeB = inXY && hasB && zb < it.g.nz;
            const float3 qa = xfPoint(it.xf, x, y, za), qb = xfPoint(it.xf, x, y, zb);
            float ra = o.maxDistSq, rb = o.maxDistSq;
            int ba = -1, bb = -1;
            if (PRECISE) {
                if (lane == 0) sPairFix[threadIdx.x >> 5][0] = sPairFix[threadIdx.x >> 5][1] = 0u;
                __syncwarp();
            }
            if (seed >= 0 && (activeA || activeB)) {
                bool da = false, db = false;
                leafDist2<PRECISE>(t, seed, qa, qb, activeA, activeB, ra, rb, ba, bb, da, db);
            }
            cpPacket2<PRECISE>(t, qa, qb, activeA, activeB, ra, rb, ba, bb, scratch + 1, vertical);
            if (PRECISE) {
                __syncwarp();
                const unsigned ma = sPairFix[threadIdx.x >> 5][0], mb = sPairFix[threadIdx.x >> 5][1];
                if ((ma | mb) && lane == 0) {
                    const uint32_t k = atomicAdd(&fix[0].x, 1u);
                    if (k < fixCap) fix[1 + k] = make_uint4(ticket, uint32_t(j), ma, mb);
                }
            }
            const int src = lane + (TZ - 1) * TX * TY * (lz == 0);
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {  // the lower voxel's sign, then the upper one's from it
                const bool active = h ? activeB : activeA;
                if (h && !__any_sync(FULL, active)) break;
                const int z = h ? zb : za;
                const float3& q = h ? qb : qa;
                const float dsq = h ? rb : ra;
                const bool valid = !(o.nullOutsideMinMax && (dsq < o.minDistSq || dsq >= o.maxDistSq));
                const bool complete = active && valid && dsq >= o.minDistSq;
                bool reIn = false;
                const bool reuse = reuseOk && reuseSign<TX, TY, TZ>(it.xf, x, y, z, z - (lz == 0 ? 1 : TZ), lz, q, below, complete,
                                                                    dsq, &reIn);
                bool onSurface = false;
                const int cw = reuseOk ? rayWinding(t, q, active && valid && !reuse, scratch + 1, &onSurface) : 0;
                const bool fwn = reuseOk ? onSurface : (active && valid);
                const float w = fwnPacket<PRECISE>(t, q, fwn, betaSq, -1, scratch + 1);
                const bool inside = reuse ? reIn : (fwn ? w > o.threshold : float(cw) > o.threshold);
                const float d = __fsqrt_rn(dsq);
                if (active) it.out[(size_t(z) * it.g.ny + y) * it.g.nx + x] = valid ? (inside ? -d : d) : __int_as_float(0x7fc00000);
                below = __shfl_sync(FULL, complete ? (inside ? -dsq : dsq) : __int_as_float(0x7fc00000), src);
            }
            seed = __shfl_sync(FULL, hasB ? bb : ba, src);
        }
    }
}

// The listed pair steps of a precise batchPairKernel launch: each flagged voxel's closest distance by
// the precise walk, written with the sign its output already holds (decided by the sign pass, which
// the distance's last bits do not move for a voxel this close to the surface).
template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(kThreads) fixBatchKernel(const BatchItem* __restrict__ items, int nItems, uint4* fix,
                                                           uint32_t fixCap, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const int lx = lane % TX, ly = (lane / TX) % TY, lz = lane / (TX * TY);
    const uint32_t n = min(__ldcg(&fix[0].x), fixCap);
    for (;;) {
        const unsigned e = nextTicket(scratch, lane);
        if (e >= n) break;
        const uint4 f = fix[1 + e];
        const BatchItem& it = items[batchItemOf(items, nItems, f.x)];
        const unsigned local = f.x - it.tileBase;
        const int tilesX = (it.g.nx + TX - 1) / TX, tilesY = (it.g.ny + TY - 1) / TY;
        const unsigned rest = local / unsigned(tilesX);
        const int x = int(local % unsigned(tilesX)) * TX + lx, y = int(rest % unsigned(tilesY)) * TY + ly;
        const int seg = int(rest / unsigned(tilesY));
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
            const bool need = ((h ? f.w : f.z) >> lane) & 1u;
            if (!__any_sync(FULL, need)) continue;
            const int z = (seg * kBatchSeg + int(f.y) + h) * TZ + lz;
            const float3 q = xfPoint(it.xf, x, y, z);
            const float dsq = cpPacket<true>(it.t, q, need, it.o.maxDistSq, 0.f, scratch + 1);
            if (need) {
                float* p = it.out + (size_t(z) * it.g.ny + y) * it.g.nx + x;
                const float old = *p;
                const bool valid = !(it.o.nullOutsideMinMax && dsq >= it.o.maxDistSq);
                if (old == old && valid) *p = copysignf(__fsqrt_rn(dsq), old);
            }
        }
    }
}

template <bool PRECISE, int TX, int TY, int TZ, int THREADS>
cudaError_t launchBatchT(const BatchItem* items, int nItems, uint32_t totalTiles, unsigned* scratch, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned), s);
    if (e || totalTiles == 0) return e;
    auto* k = batchKernel<PRECISE, TX, TY, TZ, THREADS>;
    const int sms = numSMs();
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k, THREADS, 0);
    int blocks = sms * (perSm < 1 ? 1 : perSm);
    const uint64_t maxBlocks = (uint64_t(totalTiles) + THREADS / 32 - 1) / (THREADS / 32);
    if (uint64_t(blocks) > maxBlocks) blocks = int(maxBlocks);
    k<<<blocks, THREADS, 0, s>>>(items, nItems, totalTiles, scratch);
    return cudaGetLastError();
}

template <bool PRECISE, int TX, int TY, int TZ, int THREADS>
cudaError_t launchBatchPairT(const BatchItem* items, int nItems, uint32_t totalTiles, uint4* fix, uint32_t fixCap, unsigned* scratch,
                             cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned), s);
    if (!e && PRECISE) e = cudaMemsetAsync(fix, 0, sizeof(uint4), s);
    if (e || totalTiles == 0) return e;
    auto* k = batchPairKernel<PRECISE, TX, TY, TZ, THREADS>;
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k, THREADS, 0);
    int blocks = numSMs() * (perSm < 1 ? 1 : perSm);
    const uint64_t maxBlocks = (uint64_t(totalTiles) + THREADS / 32 - 1) / (THREADS / 32);
    if (uint64_t(blocks) > maxBlocks) blocks = int(maxBlocks);
    k<<<blocks, THREADS, 0, s>>>(items, nItems, totalTiles, fix, fixCap, scratch);
    if ((e = cudaGetLastError()) || !PRECISE) return e;
    return launchPersistent(fixBatchKernel<TX, TY, TZ>, fixCap, scratch, s, items, nItems, fix, fixCap, scratch);
}

template <bool PRECISE>
cudaError_t launchBatchP(const BatchItem* items, int nItems, uint32_t totalTiles, int config, unsigned* scratch,
                         cudaStream_t s) {
    switch (config) {
        case 0: return launchBatchT<PRECISE, 4, 4, 2, 256>(items, nItems, totalTiles, scratch, s);
        case 1: return launchBatchT<PRECISE, 4, 4, 2, 128>(items, nItems, totalTiles, scratch, s);
        case 2: return launchBatchT<PRECISE, 8, 4, 1, 256>(items, nItems, totalTiles, scratch, s);
        case 3: return launchBatchT<PRECISE, 8, 4, 1, 128>(items, nItems, totalTiles, scratch, s);
        case 4: return launchBatchT<PRECISE, 2, 4, 4, 256>(items, nItems, totalTiles, scratch, s);
        case 5: return launchBatchT<PRECISE, 2, 4, 4, 128>(items, nItems, totalTiles, scratch, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

template <bool PRECISE>
cudaError_t launchBatchPairP(const BatchItem* items, int nItems, uint32_t totalTiles, int config, uint4* fix, uint32_t fixCap,
                             unsigned* scratch, cudaStream_t s) {
    switch (config) {
        case 0: return launchBatchPairT<PRECISE, 4, 4, 2, 256>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        case 1: return launchBatchPairT<PRECISE, 4, 4, 2, 128>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        case 2: return launchBatchPairT<PRECISE, 8, 4, 1, 256>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        case 3: return launchBatchPairT<PRECISE, 8, 4, 1, 128>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        case 4: return launchBatchPairT<PRECISE, 2, 4, 4, 256>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        case 5: return launchBatchPairT<PRECISE, 2, 4, 4, 128>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        default: return cudaErrorInvalidValue;
    }
}

const char* batchConfigName(int config) {
    static const char* names[kBatchConfigs] = {
        "tile 4x4x2, 256 threads",         "tile 4x4x2, 128 threads",         "tile 8x4x1, 256 threads",
        "tile 8x4x1, 128 threads",         "tile 2x4x4, 256 threads",         "tile 2x4x4, 128 threads",
        "tile 4x4x2, 256 threads, paired", "tile 4x4x2, 128 threads, paired", "tile 8x4x1, 256 threads, paired",
        "tile 8x4x1, 128 threads, paired", "tile 2x4x4, 256 threads, paired", "tile 2x4x4, 128 threads, paired"};
    return (config >= 0 && config < kBatchConfigs) ? names[config] : "";
}

uint64_t batchTiles(int config, int32_t nx, int32_t ny, int32_t nz) {
    static const int shape[kBatchShapes][3] = {{4, 4, 2}, {4, 4, 2}, {8, 4, 1}, {8, 4, 1}, {2, 4, 4}, {2, 4, 4}};
    const int* t = shape[(config >= 0 && config < kBatchConfigs) ? config % kBatchShapes : 0];
    const uint64_t tilesZ = uint64_t((nz + t[2] - 1) / t[2]);
    return uint64_t((nx + t[0] - 1) / t[0]) * uint64_t((ny + t[1] - 1) / t[1]) * ((tilesZ + kBatchSeg - 1) / kBatchSeg);
}

uint32_t batchFixCap(uint32_t totalTiles) {  // one entry per pair step at most (kept below 2^31 entries)
    return uint32_t(std::min<uint64_t>(uint64_t(totalTiles) * (kBatchSeg / 2) + 1, 0x7fffffffull));
}

cudaError_t launchBatchSdf(const BatchItem* items, int nItems, uint32_t totalTiles, int precise, int config, bool pairOk,
                           void* fix, unsigned* scratch, cudaStream_t s) {
    // a paired variant needs every item without a lower distance bound, and in precise mode the fix
    // list; otherwise it runs as its one-voxel counterpart (the same grids)
    if (config >= kBatchShapes && pairOk && (!precise || fix)) {
        uint4* f = static_cast<uint4*>(fix);
        const uint32_t cap = batchFixCap(totalTiles);
        if (precise) return launchBatchPairP<true>(items, nItems, totalTiles, config - kBatchShapes, f, cap, scratch, s);
        return launchBatchPairP<false>(items, nItems, totalTiles, config - kBatchShapes, f, cap, scratch, s);
    }
    if (precise) return launchBatchP<true>(items, nItems, totalTiles, config % kBatchShapes, scratch, s);
    return launchBatchP<false>(items, nItems, totalTiles, config % kBatchShapes, scratch, s);
}

}  // namespace gbfwn
