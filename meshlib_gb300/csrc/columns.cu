// The column sign pass of closed meshes on grids with a vertical z axis: the columns' crossing lists
// rasterised from the triangles (columnRasterKernel), the sweep of every column that turns them into
// inside bits or negated values (signColumnsKernel), and its launchers.
#include "traverse.cuh"

namespace gbfwn {
namespace {

// ------------------------------------------------------------------ sign columns (closed surfaces)
// One upward vertical ray per (x, y) column of a grid whose z axis is the world's (xf's third column
// (0, 0, +s)): every voxel of the column lies on that ray, so the exact winding number of a voxel is
// the signed number of the ray's crossings above it.  The crossings' heights come from the exact
// weights in FP64 (error below 1e-15 of the mesh's largest |z|); a voxel within 1e-12 of that of a
// crossing's height (on the surface, up to rounding), and every voxel of a column with more than
// kColumnCrossings crossings above its first voxel, gets the approximated winding number of the
// winding-number walk instead.
constexpr int kColumnCrossings = 24;

// The entry of triangle ABC in the list of the vertical column through q's (x, y): where the column
// crosses the triangle (the same exact, watertight projection test as rayCross), the tolerance
// interval of the crossing's height (FP64, from the exact weights) and its sign, the contribution to
// the winding number below it; where the column passes within sqrt(epsSq) of a vertical triangle
// (flagged in B.w: a voxel there may lie on the surface at any height of the triangle), an interval
// over the triangle's z range, plus zTol.
// The FP32 bounds compare with a voxel centre vz (a float) as the interval does: vz < lo <=> vz below
// it, vz > hi <=> vz above it (rounded outwards where widened).  false: no entry.
__device__ __forceinline__ bool columnEntry(const float3& q, const float4& A, const float4& B, const float4& C, double zTol,
                                            float zTolF, float epsSq, float* lo, float* hi, int* sign) {
    const float ax = __fsub_rn(A.x, q.x), ay = __fsub_rn(A.y, q.y), bx = __fsub_rn(B.x, q.x), by = __fsub_rn(B.y, q.y),
                cx = __fsub_rn(C.x, q.x), cy = __fsub_rn(C.y, q.y);
    const bool near = B.w != 0.f && nearProjection(ax, ay, bx, by, cx, cy, epsSq);
    const int u = edgeSign(bx, by, cx, cy);
    bool cross = u != 0 && edgeSign(cx, cy, ax, ay) == u && edgeSign(ax, ay, bx, by) == u;
    float l = FLT_MAX, h = -FLT_MAX;
    if (cross) {
        const double U = double(bx) * double(cy) - double(by) * double(cx);
        const double V = double(cx) * double(ay) - double(cy) * double(ax);
        const double W = double(ax) * double(by) - double(ay) * double(bx);
        const double det = U + V + W;
        if (det != 0.0) {
            const double z = (U * double(A.z) + V * double(B.z) + W * double(C.z)) / det;
            l = __double2float_ru(z - zTol);
            h = __double2float_rd(z + zTol);
        } else {
            cross = false;
        }
    }
    if (!cross && !near) return false;
    if (near) {
        l = fminf(l, __fsub_rd(fminf(A.z, fminf(B.z, C.z)), zTolF));
        h = fmaxf(h, __fadd_ru(fmaxf(A.z, fmaxf(B.z, C.z)), zTolF));
    }
    *lo = l;
    *hi = h;
    *sign = cross ? u : 0;
    return true;
}

// Crossing lists of the grid's columns, filled by columnRasterKernel: per column the number of
// crossings at or above the range's first voxel (may exceed kColumnSlots: the column then casts its
// own ray), bits 2k, 2k + 1 of signMask the sign of entry k (00: 0, 01: +1, 11: -1), and entry k's
// bounds {lo, hi} (columnEntry) at zz[k * ncols + column].  Index space of the columns:
// (fx, fy) = inv ((X, Y) - org); a column centre's FP32 (X, Y) lies within half of (ex, ey) of the
// exact one.
constexpr int kColumnSlots = 8;
struct ColumnLists {
    uint32_t* count;
    uint32_t* signMask;
    float2* zz;
    int64_t ncols;
    float inv[4], org[2];
    float ex, ey;
};

__device__ __forceinline__ void columnAdd(const ColumnLists& cl, const GridRange& g, const Xf& xf, double zTol, float zTolF,
                                          float epsSq, int ix, int iy, const float4& A, const float4& B, const float4& C) {
    const float3 q0 = xfPoint(xf, ix, iy, g.z0);
    float zl, zh;
    int sgn;
    if (!columnEntry(q0, A, B, C, zTol, zTolF, epsSq, &zl, &zh, &sgn)) return;
    if (q0.z > zh) return;  // below the range's first voxel
    const int64_t col = int64_t(iy) * g.nx + ix;
    const uint32_t k = atomicAdd(cl.count + col, 1u);
    if (k < uint32_t(kColumnSlots)) {
        cl.zz[size_t(k) * size_t(cl.ncols) + size_t(col)] = make_float2(zl, zh);
        if (sgn != 0) atomicOr(cl.signMask + col, (sgn > 0 ? 1u : 3u) << (2 * k));
    }
}

// One lane per triangle: the columns whose centre (x, y) may fall in the triangle's (x, y) bounds
// (the bounds widened by twice the centres' rounding, mapped to index space) are tested
// with columnEntry (the rays' exact crossing test, and the vertical-triangle rule), which adds each
// entry to its column's list.  A triangle
// over more than 16 candidate columns is taken by the whole warp, its lanes striding over them.
__global__ void __launch_bounds__(kThreads) columnRasterKernel(QueryTree t, GridRange g, Xf xf, ColumnLists cl) {
    const int lane = threadIdx.x & 31;
    const double zTol = rayZTol(t);
    const float zTolF = __double2float_ru(zTol), epsSq = rayEpsSq(t);
    const int64_t n = t.nLeaves;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i0 = int64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += stride) {
        const int64_t i = i0 + lane;
        const bool active = i < n;
        float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A, C = A;
        int ix0 = 0, iy0 = 0, w = 0, h = 0;
        if (active) {
            const float4* tr = t.tri + 3 * i;
            A = ld4(tr);
            B = ld4(tr + 1);
            C = ld4(tr + 2);
            // the widened bounds relative to the grid's origin, mapped to index space in FP32 with a
            // margin of 1e-6 of the terms' magnitudes (about 17 ulps, several times the mapping's
            // rounding; FP64 issues far slower)
            const float x0 = __fsub_rn(__fsub_rn(fminf(A.x, fminf(B.x, C.x)), cl.ex), cl.org[0]);
            const float x1 = __fadd_rn(__fsub_rn(fmaxf(A.x, fmaxf(B.x, C.x)), cl.org[0]), cl.ex);
            const float y0 = __fsub_rn(__fsub_rn(fminf(A.y, fminf(B.y, C.y)), cl.ey), cl.org[1]);
            const float y1 = __fadd_rn(__fsub_rn(fmaxf(A.y, fmaxf(B.y, C.y)), cl.org[1]), cl.ey);
            float fx0 = FLT_MAX, fx1 = -FLT_MAX, fy0 = FLT_MAX, fy1 = -FLT_MAX;
            const bool finite = x0 <= x1 && y0 <= y1;  // (no candidates for non-finite bounds)
            for (int c = 0; c < 4 && finite; ++c) {
                const float X = (c & 1) ? x1 : x0, Y = (c & 2) ? y1 : y0;
                const float tx = fabsf(cl.inv[0] * X) + fabsf(cl.inv[1] * Y), ty = fabsf(cl.inv[2] * X) + fabsf(cl.inv[3] * Y);
                const float fx = fmaf(cl.inv[0], X, cl.inv[1] * Y), fy = fmaf(cl.inv[2], X, cl.inv[3] * Y);
                fx0 = fminf(fx0, fx - 1e-6f * tx);
                fx1 = fmaxf(fx1, fx + 1e-6f * tx);
                fy0 = fminf(fy0, fy - 1e-6f * ty);
                fy1 = fmaxf(fy1, fy + 1e-6f * ty);
            }
            // the candidates: ceil(f0) .. floor(f1), clamped to the grid (compared in FP32 before any
            // conversion, so bounds beyond int range convert nothing)
            const float cx0 = fmaxf(0.f, ceilf(fx0)), cx1 = fminf(float(g.nx - 1), floorf(fx1));
            const float cy0 = fmaxf(0.f, ceilf(fy0)), cy1 = fminf(float(g.ny - 1), floorf(fy1));
            if (finite && cx0 <= cx1 && cy0 <= cy1) {
                ix0 = int(cx0);
                iy0 = int(cy0);
                w = int(cx1) - ix0 + 1;
                h = int(cy1) - iy0 + 1;
            }
        }
        const int64_t nc = int64_t(w) * h;
        if (nc <= 16) {
            for (int c = 0; c < int(nc); ++c) columnAdd(cl, g, xf, zTol, zTolF, epsSq, ix0 + c % w, iy0 + c / w, A, B, C);
        }
        unsigned big = __ballot_sync(FULL, nc > 16);
        while (big) {
            const int b = __ffs(big) - 1;
            big &= big - 1;
            // the whole records, flags included (B.w: a vertical triangle)
            const float4 Ab = make_float4(__shfl_sync(FULL, A.x, b), __shfl_sync(FULL, A.y, b), __shfl_sync(FULL, A.z, b),
                                          __shfl_sync(FULL, A.w, b));
            const float4 Bb = make_float4(__shfl_sync(FULL, B.x, b), __shfl_sync(FULL, B.y, b), __shfl_sync(FULL, B.z, b),
                                          __shfl_sync(FULL, B.w, b));
            const float4 Cb = make_float4(__shfl_sync(FULL, C.x, b), __shfl_sync(FULL, C.y, b), __shfl_sync(FULL, C.z, b),
                                          __shfl_sync(FULL, C.w, b));
            const int bx0 = __shfl_sync(FULL, ix0, b), by0 = __shfl_sync(FULL, iy0, b), bw = __shfl_sync(FULL, w, b);
            const int64_t bn = int64_t(bw) * __shfl_sync(FULL, h, b);
            for (int64_t c = lane; c < bn; c += 32)
                columnAdd(cl, g, xf, zTol, zTolF, epsSq, bx0 + int(c % bw), by0 + int(c / bw), Ab, Bb, Cb);
        }
    }
}

// For the grid columns of the launch (32 consecutive x per warp, in segments of kColumnSeg layers;
// the crossings from the columns' lists, or a column's own ray where its list overflowed or there are
// no lists): inside = (winding number of the voxel > threshold), written as bits (one
// word per 32 voxels along x, layout (z - zOut, y, x / 32)) or applied to `values` (negated where
// inside; value index (z - zOut) nx ny + y nx + x).  The range [z0, z1) of dims is covered.
constexpr int kColumnSeg = 128;

// Inside bits (bit k: the voxel at zc + k) of the voxels of a column chunk marked in `amb`, from their
// approximated winding numbers.  Out of line, as columnRay: few voxels take it.
template <bool PRECISE>
__device__ __noinline__ uint32_t columnWalks(const QueryTree& t, const Xf& xf, int xc, int y, int zc, int kn, uint32_t amb,
                                             float betaSq, float threshold, unsigned* status) {
    uint32_t in = 0;
    for (int k = 0; k < kn; ++k) {
        const bool need = (amb >> k) & 1u;
        if (!__any_sync(FULL, need)) continue;
        const float wf = fwnPacket<PRECISE>(t, xfPoint(xf, xc, y, zc + k), need, betaSq, -1, status);
        if (need && wf > threshold) in |= 1u << k;
    }
    return in;
}

// The entries of the columns of the lanes with `ray` from their own vertical ray: a packet walk over
// the reference nodes (a node when the lane's (x, y) lies in its box's footprint and the box reaches
// q0's height) adding each triangle's columnEntry to the lane's list, by lo; past kColumnCrossings
// entries, or when the stack overflows (the whole warp), *overflow is set.  Out of line: only
// columns whose list overflowed, or launches without lists, take it, and its registers stay out of
// the sweep.
__device__ __noinline__ void columnRay(const QueryTree& t, float3 q0, bool ray, double zTol, float zTolF, float epsSq, float* lo,
                                       float* hi, int* sg, int* nOut, bool* overflowOut, unsigned* status) {
    const int lane = threadIdx.x & 31;
    int n = *nOut;
    bool overflow = *overflowOut;
    WarpStack st;
    st.push(lane, 0, __ballot_sync(FULL, ray));
    bool stackFull = false;
    while (st.sp > 0 && t.nLeaves > 0) {
        int node;
        unsigned m;
        st.pop(node, m);
        const float4 n0 = ld4(t.nodes + 2 * int64_t(node)), n1 = ld4(t.nodes + 2 * int64_t(node) + 1);
        const bool hit = ((m >> lane) & 1u) && q0.x >= n0.x && q0.x <= n0.w && q0.y >= n0.y && q0.y <= n1.x && n1.y >= q0.z;
        const unsigned mh = __ballot_sync(FULL, hit);
        if (!mh) continue;
        const int l = __float_as_int(n1.z), r = __float_as_int(n1.w);
        if (r < 0) {
            const float4* tr = t.tri + 3 * int64_t(t.faceSlot[l]);
            const float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
            float zl, zh;
            int sgn;
            if (hit && columnEntry(q0, A, B, C, zTol, zTolF, epsSq, &zl, &zh, &sgn) && !(q0.z > zh)) {
                if (n < kColumnCrossings) {
                    int k = n++;
                    while (k > 0 && lo[k - 1] > zl) {
                        lo[k] = lo[k - 1];
                        hi[k] = hi[k - 1];
                        sg[k] = sg[k - 1];
                        --k;
                    }
                    lo[k] = zl;
                    hi[k] = zh;
                    sg[k] = sgn;
                } else {
                    overflow = true;
                }
            }
        } else if (!st.push(lane, r, mh) || !st.push(lane, l, mh)) {
            stackFull = true;
            break;
        }
    }
    if (stackFull) {
        overflow = true;  // every lane of the warp falls back
        if (lane == 0) atomicOr(status, kStatusStackOverflow);
    }
    *nOut = n;
    *overflowOut = overflow;
}

template <bool PRECISE>
__global__ void __launch_bounds__(kThreads, 4) signColumnsKernel(QueryTree t, GridRange g, Xf xf, float threshold, float beta,
                                                          uint32_t* __restrict__ bits, float* __restrict__ values,
                                                          ColumnLists cl, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const float betaSq = __fmul_rn(beta, beta);
    const int wordsX = (g.nx + 31) >> 5;
    const int segs = (g.z1 - g.z0 + kColumnSeg - 1) / kColumnSeg;
    const uint64_t items = uint64_t(wordsX) * uint64_t(g.ny) * uint64_t(segs);
    const size_t sxy = size_t(g.nx) * g.ny;
    const double zTol = rayZTol(t);
    const float zTolF = __double2float_ru(zTol), epsSq = rayEpsSq(t);
    // per entry (ascending lo; columnEntry): the FP32 bounds of its interval, so that for a voxel
    // centre vz (a float) vz < lo <=> vz below the interval and vz > hi <=> vz above it: the sweep
    // compares in FP32 (FP64 issues at a small fraction of the FP32 rate)
    float lo[kColumnCrossings], hi[kColumnCrossings];
    int sg[kColumnCrossings];
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (item >= items) break;
        const int wx = int(item % unsigned(wordsX));
        const unsigned rest = item / unsigned(wordsX);
        const int y = int(rest % unsigned(g.ny));
        const int zs0 = g.z0 + int(rest / unsigned(g.ny)) * kColumnSeg, zs1 = min(g.z1, zs0 + kColumnSeg);
        const int x = wx * 32 + lane;
        const bool active = x < g.nx;
        const int xc = active ? x : 0;
        const float3 q0 = xfPoint(xf, xc, y, zs0);
        // the column's crossings from its list, or, without lists or when the list overflowed, from
        // the ray: a packet walk over the reference nodes collecting the crossings above q0; by height
        int n = 0;
        bool overflow = false;
        bool ray = active && !cl.count;
        if (cl.count && active) {
            const int64_t col = int64_t(y) * g.nx + x;
            const uint32_t c = __ldg(cl.count + col);
            if (c <= uint32_t(kColumnSlots)) {
                const uint32_t mask = __ldg(cl.signMask + col);
                for (uint32_t e = 0; e < c; ++e) {
                    const float2 zz = __ldg(cl.zz + size_t(e) * size_t(cl.ncols) + size_t(col));
                    int k = n++;
                    while (k > 0 && lo[k - 1] > zz.x) {
                        lo[k] = lo[k - 1];
                        hi[k] = hi[k - 1];
                        sg[k] = sg[k - 1];
                        --k;
                    }
                    lo[k] = zz.x;
                    hi[k] = zz.y;
                    const uint32_t m2 = (mask >> (2 * e)) & 3u;
                    sg[k] = m2 == 1u ? 1 : (m2 == 3u ? -1 : 0);
                }
            } else {
                ray = true;
            }
        }
        if (__any_sync(FULL, ray)) columnRay(t, q0, ray, zTol, zTolF, epsSq, lo, hi, sg, &n, &overflow, scratch + 1);
        // the sweep up the segment, 32 layers at a time: w = signed crossings above the voxel
        int w = 0, p = 0;
        for (int k = 0; k < n; ++k) w += sg[k];
        for (int zc = zs0; zc < zs1; zc += 32) {
            const int kn = min(32, zs1 - zc);
            uint32_t in = 0, amb = 0;  // bit k: the voxel at zc + k
            for (int k = 0; k < kn; ++k) {
                const float vz = xfPoint(xf, xc, y, zc + k).z;
                // entries passed (below the voxel) leave w; the walk stops at the first entry reaching
                // up to vz, and every entry after it starts above lo[p] (ascending lo): so the voxel
                // lies in an interval iff vz >= lo[p], and otherwise every entry left is above it
                while (p < n && vz > hi[p]) {
                    w -= sg[p];
                    ++p;
                }
                if (overflow || (p < n && vz >= lo[p]))  // on the surface, up to rounding: the walk decides
                    amb |= 1u << k;
                else if (float(w) > threshold)
                    in |= 1u << k;
            }
            if (!active) amb = in = 0;
            // on the surface (up to rounding): the winding-number walk
            if (__any_sync(FULL, amb != 0)) in |= columnWalks<PRECISE>(t, xf, xc, y, zc, kn, amb, betaSq, threshold, scratch + 1);
            if (values) {
                float* vp = values + size_t(zc - g.zOut) * sxy + size_t(y) * g.nx + xc;
#pragma unroll 8
                for (int k = 0; k < kn; ++k)
                    if ((in >> k) & 1u) vp[size_t(k) * sxy] = -vp[size_t(k) * sxy];
            } else {
                uint32_t mine = 0;  // lane k stores layer zc + k's word
                for (int k = 0; k < kn; ++k) {
                    const uint32_t word = __ballot_sync(FULL, (in >> k) & 1u);
                    if (lane == k) mine = word;
                }
                if (lane < kn) bits[(size_t(zc + lane - g.zOut) * g.ny + y) * wordsX + wx] = mine;
            }
        }
    }
}

}  // namespace

bool signColumnsApply(const QueryTree& t, const Xf& xf, float beta, float threshold) {
    const float fr = threshold - floorf(threshold);
    // the (x, y) map must be well conditioned: the raster pass maps triangle bounds back to columns
    // through its inverse, in FP32
    const double det = double(xf.a[0]) * xf.a[4] - double(xf.a[1]) * xf.a[3];
    const double scale = (std::fabs(double(xf.a[0])) + std::fabs(double(xf.a[1]))) * (std::fabs(double(xf.a[3])) + std::fabs(double(xf.a[4])));
    return t.closed && beta >= 2.f && fr > 0.25f && fr < 0.75f && xf.a[2] == 0.f && xf.a[5] == 0.f && xf.a[8] > 0.f &&
           std::fabs(det) >= 1e-6 * scale && std::fabs(det) > 1e-30 && scale < 1e30;
}

size_t signColumnsWorkBytes(const GridRange& g) {
    const size_t ncols = size_t(g.nx) * size_t(g.ny);
    return ((2 * sizeof(uint32_t) + kColumnSlots * sizeof(float2)) * ncols + 255) & ~size_t(255);
}

cudaError_t launchSignColumns(const QueryTree& t, const GridRange& g, const Xf& xf, float beta, float threshold, int precise,
                              uint32_t* bits, float* values, void* work, size_t workBytes, unsigned* scratch, cudaStream_t s) {
    ColumnLists cl{};
    const size_t ncols = size_t(g.nx) * size_t(g.ny);
    if (work && workBytes >= signColumnsWorkBytes(g) && t.nLeaves > 0) {
        // zz first (8-byte aligned), then the counts and sign masks, cleared together
        cl.zz = static_cast<float2*>(work);
        cl.count = reinterpret_cast<uint32_t*>(cl.zz + kColumnSlots * ncols);
        cl.signMask = cl.count + ncols;
        cl.ncols = int64_t(ncols);
        const double a0 = xf.a[0], a1 = xf.a[1], a3 = xf.a[3], a4 = xf.a[4], det = a0 * a4 - a1 * a3;
        cl.inv[0] = float(a4 / det);
        cl.inv[1] = float(-a1 / det);
        cl.inv[2] = float(-a3 / det);
        cl.inv[3] = float(a0 / det);
        cl.org[0] = xf.b[0];
        cl.org[1] = xf.b[1];
        // xfPoint's four roundings of x = a0 i + a1 j + 0 k + b0: at most 2 ulps of the largest magnitude
        const auto margin = [](double m) { return float(4.0 * std::ldexp(1.0, std::ilogb(m > 0 ? m : 1e-30) - 23)); };
        cl.ex = margin(std::fabs(a0) * (g.nx - 1) + std::fabs(a1) * (g.ny - 1) + std::fabs(double(xf.b[0])));
        cl.ey = margin(std::fabs(a3) * (g.nx - 1) + std::fabs(a4) * (g.ny - 1) + std::fabs(double(xf.b[1])));
        cudaError_t e = cudaMemsetAsync(cl.count, 0, 2 * sizeof(uint32_t) * ncols, s);
        if (e) return e;
        int blocks = int(std::min<int64_t>((int64_t(t.nLeaves) + kThreads - 1) / kThreads, int64_t(numSMs()) * 16));
        columnRasterKernel<<<blocks, kThreads, 0, s>>>(t, g, xf, cl);
        if ((e = cudaGetLastError())) return e;
    }
    const uint64_t items = uint64_t((g.nx + 31) / 32) * uint64_t(g.ny) * uint64_t((g.z1 - g.z0 + kColumnSeg - 1) / kColumnSeg);
    if (precise)
        return launchPersistent(signColumnsKernel<true>, items, scratch, s, t, g, xf, threshold, beta, bits, values, cl, scratch);
    return launchPersistent(signColumnsKernel<false>, items, scratch, s, t, g, xf, threshold, beta, bits, values, cl, scratch);
}

size_t signBitsBytes(const GridRange& g) {
    return size_t((g.nx + 31) >> 5) * size_t(g.ny) * size_t(g.z1 - g.z0) * sizeof(uint32_t);
}

}  // namespace gbfwn
