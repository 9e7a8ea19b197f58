// CPU oracle for the fast-winding-number / signed-distance path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++, the reference
// algorithm of MeshLib's CPU `MR::FastWindingNumber` so that the CUDA product
// can be checked against it.  Only the test-suite, the smoke check and the
// CPU-baseline leg of the benchmark load it; the product never does.
//
// Every routine is templated on the arithmetic type T:
//   T = float  : the reference's own FP32 arithmetic, operation by operation
//                (compile with -ffp-contract=off so no FMA is formed);
//   T = double : the FP64 oracle that the precision figures are quoted on: the same tree and
//                the reference's own FP32 far-field decisions (so the same set of dipole terms
//                and exact solid angles), every term and sum evaluated in double.  Winding
//                numbers with no approximation at all come from orc_exact_wn.
//
// Reference files restated here (paths inside the MeshLib project):
//   source/MRMesh/MRAABBTree.cpp:15-60          face boxes, tree construction
//   source/MRMesh/MRAABBTreeMaker.hpp:51-165    median split, pre-order layout
//   source/MRMesh/MRAABBTreeMaker.h:23-27       2n-1 nodes
//   source/MRMesh/MRBox.h:122-139,260-270,376-396  include, insignificantlyExpanded, findSortedBoxDims
//   source/MRMesh/MRDipole.h:10-28              Dipole::addIfGoodApprox
//   source/MRMesh/MRDipole.cpp:11-128           calcDipoles, triangleSolidAngle, calcFastWindingNumber
//   source/MRMesh/MRMeshProject.cpp:13-104      findProjectionSubtree
//   source/MRMesh/MRClosestPointInTriangle.h:28-91  closestPointInTriangle
//   source/MRMesh/MRFastWindingNumber.cpp:28-94 calcFromVector/SelfIntersections/Grid/GridWithDistances
//   source/MRMesh/MRVolumeIndexer.h:131-139     voxel linearisation (x fastest)
//   source/MRMesh/MRMeshMath.cpp:119-149        triCenter, leftDirDblArea
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stack>
#include <thread>
#include <type_traits>
#include <vector>

namespace orc {

template <typename T> struct V3 {
    T x = 0, y = 0, z = 0;
    V3() = default;
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <typename T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
// MRVector3.h:118 dot is x*x' + y*y' + z*z' evaluated left to right
template <typename T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> inline T lengthSq(V3<T> a) { return dot(a, a); }
template <typename T> inline T length(V3<T> a) { return std::sqrt(lengthSq(a)); }
template <typename T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T, typename U> inline V3<T> cvt(V3<U> a) { return {T(a.x), T(a.y), T(a.z)}; }

struct Box3f {
    V3<float> min{std::numeric_limits<float>::max(), std::numeric_limits<float>::max(), std::numeric_limits<float>::max()};
    V3<float> max{std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest()};
    // MRBox.h:122-129
    void include(V3<float> p) {
        for (int i = 0; i < 3; ++i) {
            if (p[i] < min[i]) min[i] = p[i];
            if (p[i] > max[i]) max[i] = p[i];
        }
    }
    // MRBox.h:132-139
    void include(const Box3f& b) {
        for (int i = 0; i < 3; ++i) {
            if (b.min[i] < min[i]) min[i] = b.min[i];
            if (b.max[i] > max[i]) max[i] = b.max[i];
        }
    }
};

// Node of the reference tree layout: box + two children; leaf <=> r < 0 and then l = face id
// (MRAABBTreeNode.h:29-46).  32 bytes, the same as the reference.
struct Node {
    Box3f box;
    int32_t l, r;
};
static_assert(sizeof(Node) == 32, "reference node is 32 bytes");

struct Mesh {
    const float* verts;  // nv x 3
    const int32_t* tris; // nt x 3
    int nv, nt;
    V3<float> p(int v) const { return {verts[3 * v], verts[3 * v + 1], verts[3 * v + 2]}; }
    bool valid(int f) const { return tris[3 * f] >= 0 && tris[3 * f + 1] >= 0 && tris[3 * f + 2] >= 0; }
    void tri(int f, V3<float>& a, V3<float>& b, V3<float>& c) const {
        a = p(tris[3 * f]);
        b = p(tris[3 * f + 1]);
        c = p(tris[3 * f + 2]);
    }
};

// ---------------------------------------------------------------- tree build
// MRAABBTree.cpp:15-29 computeFaceBox (+ MRBox.h:260-270 insignificantlyExpanded)
static Box3f computeFaceBox(const Mesh& m, int f) {
    Box3f box;
    V3<float> a, b, c;
    m.tri(f, a, b, c);
    box.include(a);
    box.include(b);
    box.include(c);
    Box3f r;
    for (int i = 0; i < 3; ++i) {
        r.min[i] = std::nextafter(box.min[i], std::numeric_limits<float>::lowest());
        r.max[i] = std::nextafter(box.max[i], std::numeric_limits<float>::max());
    }
    return r;
}

// MRBox.h:376-396 findSortedBoxDims: dims sorted ascending by (extent, index)
static void findSortedBoxDims(const Box3f& box, int out[3]) {
    std::pair<float, int> ps[3];
    for (int i = 0; i < 3; ++i) ps[i] = {box.max[i] - box.min[i], i};
    for (int i = 0; i + 1 < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (ps[j] < ps[i]) std::swap(ps[i], ps[j]);
    for (int i = 0; i < 3; ++i) out[i] = ps[i].second;
}

struct BoxedLeaf {
    int32_t leafId;
    Box3f box;
};

// MRAABBTreeMaker.hpp:51-174, single-threaded (the result does not depend on threading).
static void buildTree(const Mesh& m, std::vector<Node>& nodes) {
    // MRAABBTree.cpp:31-57: leaves are the valid faces (a face with a negative vertex id is not
    // valid), keeping their face ids
    std::vector<BoxedLeaf> leaves;
    for (int f = 0; f < m.nt; ++f)
        if (m.valid(f)) leaves.push_back({f, computeFaceBox(m, f)});
    const int n = int(leaves.size());
    nodes.assign(n > 0 ? 2 * n - 1 : 0, Node{});
    if (n <= 0) return;

    struct Sub {
        int root, first, num;
    };
    std::vector<Sub> st;
    st.push_back({0, 0, n});
    while (!st.empty()) {
        Sub s = st.back();
        st.pop_back();
        Node& node = nodes[s.root];
        if (s.num == 1) {
            node.l = leaves[s.first].leafId;
            node.r = -1;
            node.box = leaves[s.first].box;
            continue;
        }
        // MRAABBTreeMaker.hpp:77-95 makeNode_
        node.box = Box3f{};
        for (int i = 0; i < s.num; ++i) node.box.include(leaves[s.first + i].box);
        int sd[3];
        findSortedBoxDims(node.box, sd);
        auto less = [&](const BoxedLeaf& a, const BoxedLeaf& b) {
            for (int i = 2; i >= 0; --i) {
                const int d = sd[i];
                const float ad = a.box.min[d] + a.box.max[d];
                const float bd = b.box.min[d] + b.box.max[d];
                if (ad != bd) return ad < bd;
            }
            return a.leafId < b.leafId;
        };
        const int mid = s.first + s.num / 2;
        std::nth_element(leaves.begin() + s.first, leaves.begin() + mid, leaves.begin() + s.first + s.num, less);
        const int nl = mid - s.first;
        node.l = s.root + 1;
        node.r = s.root + 1 + (2 * nl - 1);
        st.push_back({node.r, mid, s.num - nl});
        st.push_back({node.l, s.first, nl});
    }
}

// ------------------------------------------------------------------ dipoles
template <typename T> struct Dipole {
    V3<T> pos;
    T area = 0;
    V3<T> dirArea;
    T rr = 0;
    // MRDipole.h:18-27
    bool addIfGoodApprox(const V3<T>& q, T betaSq, T& addTo) const {
        const V3<T> dp = pos - q;
        const T dd = lengthSq(dp);
        if (dd <= betaSq * rr) return false;
        const T d = std::sqrt(dd);
        if (d > 0) addTo += dot(dp, dirArea) / (d * dd);
        return true;
    }
};

// MRDipole.cpp:11-21
template <typename T> static T distToFarthestCornerSq(const Box3f& box, const V3<T>& pos) {
    T res = 0;
    for (int i = 0; i < 3; ++i) {
        const T a = pos[i] - T(box.min[i]);
        const T b = pos[i] - T(box.max[i]);
        res += std::max(a * a, b * b);
    }
    return res;
}

// MRDipole.cpp:23-71 calcDipoles
template <typename T> static void calcDipoles(const Mesh& m, const std::vector<Node>& nodes, std::vector<Dipole<T>>& dip) {
    dip.assign(nodes.size(), Dipole<T>{});
    for (size_t i = 0; i < nodes.size(); ++i) {
        const Node& nd = nodes[i];
        if (nd.r >= 0) continue;
        V3<float> a, b, c;
        m.tri(nd.l, a, b, c);
        const V3<T> A = cvt<T>(a), B = cvt<T>(b), C = cvt<T>(c);
        const V3<T> da = T(0.5) * cross(B - A, C - A);        // 0.5f * dirDblArea (MRMeshMath.cpp:140-149)
        const T ar = length(da);
        const V3<T> ctr = (T(1) / T(3)) * (A + B + C);         // triCenter (MRMeshMath.cpp:119-124)
        dip[i].pos = ar * ctr;
        dip[i].area = ar;
        dip[i].dirArea = da;
    }
    // MRDipole.cpp:47-60: reverse node order down to the root inclusive (NodeId 0 is valid)
    for (size_t i = nodes.size(); i-- > 0;) {
        const Node& nd = nodes[i];
        if (nd.r < 0) continue;
        const Dipole<T>& dl = dip[nd.l];
        const Dipole<T>& dr = dip[nd.r];
        dip[i].pos = dl.pos + dr.pos;
        dip[i].area = dl.area + dr.area;
        dip[i].dirArea = dl.dirArea + dr.dirArea;
    }
    for (size_t i = 0; i < nodes.size(); ++i) {
        Dipole<T>& d = dip[i];
        if (d.area > 0) d.pos = (T(1) / d.area) * d.pos;   // Vector3::operator/= multiplies by 1/a (MRVector3.h:131-137)
        d.rr = distToFarthestCornerSq<T>(nodes[i].box, d.pos);
    }
}

// MRDipole.cpp:81-92 (Jacobson et al. 2013, eq. 6)
template <typename T> static T triangleSolidAngle(const V3<T>& p, const V3<T>& t0, const V3<T>& t1, const V3<T>& t2) {
    const V3<T> mx = t0 - p, my = t1 - p, mz = t2 - p;
    const T x = length(mx), y = length(my), z = length(mz);
    const T den = x * y * z + dot(mx, my) * z + dot(my, mz) * x + dot(mz, mx) * y;
    // Matrix3::det (MRMatrix3.h:227-233) with rows mx, my, mz
    const T det = mx.x * (my.y * mz.z - my.z * mz.y) - mx.y * (my.x * mz.z - my.z * mz.x) + mx.z * (my.x * mz.y - my.y * mz.x);
    return 2 * std::atan2(det, den);
}

struct Counters {
    uint64_t fwnNodes = 0;   // dipole records read by the winding-number DFS
    uint64_t fwnLeaves = 0;  // exact solid angles evaluated
    uint64_t cpNodes = 0;    // AABB boxes read by the closest-point DFS
    uint64_t cpLeaves = 0;   // point-triangle projections evaluated
};

// MRDipole.cpp:94-128 calcFastWindingNumber (stack of 32, right pushed first, left popped first).
// With `decide` (FP64 oracle), the far-field test of every node is the reference's FP32 test on
// the FP32 dipoles and FP32 query `qf`, so the FP64 sum covers exactly the reference's set of
// dipole terms and solid angles -- only the arithmetic differs.
template <typename T>
static T calcFWN(const Mesh& m, const std::vector<Node>& nodes, const std::vector<Dipole<T>>& dip, const V3<T>& q, T beta,
                 int skipFace, Counters* cnt, const std::vector<Dipole<float>>* decide = nullptr, V3<float> qf = {}) {
    if (dip.empty()) return 0;
    const T betaSq = beta * beta;
    const float betaSqF = float(beta) * float(beta);
    int stack[64];
    int sp = 0;
    stack[sp++] = 0;
    T res = 0;
    while (sp > 0) {
        const int i = stack[--sp];
        const Node& node = nodes[i];
        if (cnt) cnt->fwnNodes++;
        if (decide) {
            const Dipole<float>& df = (*decide)[i];
            const V3<float> dpf = df.pos - qf;
            if (lengthSq(dpf) > betaSqF * df.rr) {
                const V3<T> dp = dip[i].pos - q;
                const T dd = lengthSq(dp);
                const T d = std::sqrt(dd);
                if (d > 0) res += dot(dp, dip[i].dirArea) / (d * dd);
                continue;
            }
        } else if (dip[i].addIfGoodApprox(q, betaSq, res)) {
            continue;
        }
        if (node.r >= 0) {
            stack[sp++] = node.r;
            stack[sp++] = node.l;
            continue;
        }
        if (node.l != skipFace) {
            V3<float> a, b, c;
            m.tri(node.l, a, b, c);
            if (cnt) cnt->fwnLeaves++;
            res += triangleSolidAngle<T>(q, cvt<T>(a), cvt<T>(b), cvt<T>(c));
        }
    }
    const T INV_4PI = T(1) / (4 * T(3.14159265358979323846));
    return INV_4PI * res;
}

// MRClosestPointInTriangle.h:28-91 (double in the reference CPU path, MRMeshProject.cpp:68)
template <typename T> static V3<T> closestPointInTriangle(const V3<T>& p, const V3<T>& a, const V3<T>& b, const V3<T>& c) {
    const V3<T> ab = b - a, ac = c - a, ap = p - a;
    const T d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0 && d2 <= 0) return a;
    const V3<T> bp = p - b;
    const T d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) return b;
    const V3<T> cp = p - c;
    const T d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) return c;
    const T vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) {
        const T v = d1 / (d1 - d3);
        return a + v * ab;
    }
    const T vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d6 <= 0 && d2 >= 0) {
        const T v = d2 / (d2 - d6);
        return a + v * ac;
    }
    const T va = d3 * d6 - d5 * d4;
    if (va <= 0) {
        if (d4 < d3) return b;
        if (d5 < d6) return c;
        const T v = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return b + v * (c - b);
    }
    const T denom = 1 / (va + vb + vc);
    const T v = vb * denom, w = vc * denom;
    return a + v * ab + w * ac;
}

// MRBox.h:207-220 Box::getDistanceSq(point)
template <typename T> static T boxDistSq(const Box3f& box, const V3<T>& p) {
    T res = 0;
    for (int i = 0; i < 3; ++i) {
        if (p[i] < T(box.min[i])) {
            const T d = p[i] - T(box.min[i]);
            res += d * d;
        } else if (p[i] > T(box.max[i])) {
            const T d = p[i] - T(box.max[i]);
            res += d * d;
        }
    }
    return res;
}

// MRMeshProject.cpp:13-104 findProjectionSubtree (no xf, no region, no predicates).
// T=float: the reference itself -- FP64 leaf projection, float distance of the float projection.
// T=double: everything in double.
template <typename T>
static T findProjectionDistSq(const Mesh& m, const std::vector<Node>& nodes, const V3<T>& pt, T upDistLimitSq, T loDistLimitSq,
                              Counters* cnt) {
    T resSq = upDistLimitSq;
    if (nodes.empty()) return resSq;
    struct SubTask {
        int n;
        T distSq;
    };
    SubTask st[64];
    int sp = 0;
    auto addSubTask = [&](const SubTask& s) {
        if (s.distSq < resSq) st[sp++] = s;
    };
    auto getSubTask = [&](int n) {
        if (cnt) cnt->cpNodes++;
        return SubTask{n, boxDistSq<T>(nodes[n].box, pt)};
    };
    addSubTask(getSubTask(0));
    while (sp > 0) {
        const SubTask s = st[--sp];
        const Node& node = nodes[s.n];
        if (s.distSq >= resSq) continue;
        if (node.r < 0) {
            V3<float> a, b, c;
            m.tri(node.l, a, b, c);
            if (cnt) cnt->cpLeaves++;
            const V3<double> projD = closestPointInTriangle<double>(cvt<double>(pt), cvt<double>(a), cvt<double>(b), cvt<double>(c));
            const V3<T> proj = cvt<T>(projD);
            const T distSq = lengthSq(proj - pt);
            if (distSq < resSq) {
                resSq = distSq;
                if (resSq <= loDistLimitSq) break;
            }
            continue;
        }
        SubTask s1 = getSubTask(node.l);
        SubTask s2 = getSubTask(node.r);
        if (s1.distSq < s2.distSq) {
            addSubTask(s2);
            addSubTask(s1);
        } else {
            addSubTask(s1);
            addSubTask(s2);
        }
    }
    return resSq;
}

// ---------------------------------------------------------------- points-to-mesh projection
// Affine map in float (MRAffineXf.h): rows of A, then b; x -> A x + b with left-to-right dots.
struct AffF {
    float A[3][3];
    float b[3];
};
static AffF affFrom(const float* x) {
    AffF r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.A[i][j] = x[3 * i + j];
    for (int i = 0; i < 3; ++i) r.b[i] = x[9 + i];
    return r;
}
static V3<float> apply(const AffF& x, V3<float> p) {
    return {(x.A[0][0] * p.x + x.A[0][1] * p.y + x.A[0][2] * p.z) + x.b[0],
            (x.A[1][0] * p.x + x.A[1][1] * p.y + x.A[1][2] * p.z) + x.b[1],
            (x.A[2][0] * p.x + x.A[2][1] * p.y + x.A[2][2] * p.z) + x.b[2]};
}
// MRMatrix3Decompose.h:27-39 isRigid over MRMatrix3.h:272-294 qr (Gram-Schmidt on the columns)
static bool affIsRigid(const AffF& x) {
    V3<float> a0{x.A[0][0], x.A[1][0], x.A[2][0]}, a1{x.A[0][1], x.A[1][1], x.A[2][1]}, a2{x.A[0][2], x.A[1][2], x.A[2][2]};
    const float r00 = length(a0);
    const V3<float> e0 = r00 > 0 ? (1 / r00) * a0 : V3<float>{};
    const float r01 = dot(e0, a1), r02 = dot(e0, a2);
    a1 = a1 - r01 * e0;
    const float r11 = length(a1);
    const V3<float> e1 = r11 > 0 ? (1 / r11) * a1 : V3<float>{};
    const float r12 = dot(e1, a2);
    a2 = a2 - (r02 * e0 + r12 * e1);
    const float r22 = length(a2);
    const float eps = 10 * std::numeric_limits<float>::epsilon();
    return std::abs(r00 - 1) <= eps && std::abs(r11 - 1) <= eps && std::abs(r22 - 1) <= eps;
}
// MRMatrix3.h:227-247 + MRAffineXf.h:51-57
static AffF affInverse(const AffF& x) {
    const auto& m = x.A;
    const float det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                      m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    AffF r{};
    if (det != 0) {
        const float c[3][3] = {
            {m[1][1] * m[2][2] - m[1][2] * m[2][1], m[0][2] * m[2][1] - m[0][1] * m[2][2], m[0][1] * m[1][2] - m[0][2] * m[1][1]},
            {m[1][2] * m[2][0] - m[1][0] * m[2][2], m[0][0] * m[2][2] - m[0][2] * m[2][0], m[0][2] * m[1][0] - m[0][0] * m[1][2]},
            {m[1][0] * m[2][1] - m[1][1] * m[2][0], m[0][1] * m[2][0] - m[0][0] * m[2][1], m[0][0] * m[1][1] - m[0][1] * m[1][0]}};
        const float inv = 1 / det;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.A[i][j] = inv * c[i][j];
    }
    for (int i = 0; i < 3; ++i) r.b[i] = -(r.A[i][0] * x.b[0] + r.A[i][1] * x.b[1] + r.A[i][2] * x.b[2]);
    return r;
}
// MRAffineXf.h:61-62: (u * v)(x) = u(v(x))
static AffF affCompose(const AffF& u, const AffF& v) {
    AffF r;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) r.A[i][j] = u.A[i][0] * v.A[0][j] + u.A[i][1] * v.A[1][j] + u.A[i][2] * v.A[2][j];
        r.b[i] = (u.A[i][0] * v.b[0] + u.A[i][1] * v.b[1] + u.A[i][2] * v.b[2]) + u.b[i];
    }
    return r;
}
// MRBox.h:336-344 transformed(box, xf): the box of the mapped corners
static Box3f transformedBox(const Box3f& box, const AffF& xf) {
    Box3f r;
    for (int k = 0; k < 8; ++k)
        r.include(apply(xf, V3<float>{(k & 1) ? box.max.x : box.min.x, (k & 2) ? box.max.y : box.min.y,
                                       (k & 4) ? box.max.z : box.min.z}));
    return r;
}

// MRClosestPointInTriangle.h:28-91 with the barycentric result: proj = (1 - a - b) A + a B + b C
static void closestPointBary(const V3<double>& p, const V3<double>& a, const V3<double>& b, const V3<double>& c, V3<double>& proj,
                             double& ba, double& bb) {
    const V3<double> ab = b - a, ac = c - a, ap = p - a;
    ba = bb = 0;
    const double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0 && d2 <= 0) { proj = a; return; }
    const V3<double> bp = p - b;
    const double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) { proj = b; ba = 1; return; }
    const V3<double> cp = p - c;
    const double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) { proj = c; bb = 1; return; }
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) { ba = d1 / (d1 - d3); proj = a + ba * ab; return; }
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d6 <= 0 && d2 >= 0) { bb = d2 / (d2 - d6); proj = a + bb * ac; return; }
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0) {
        if (d4 < d3) { proj = b; ba = 1; return; }
        if (d5 < d6) { proj = c; bb = 1; return; }
        const double v = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        proj = b + v * (c - b);
        ba = 1 - v;
        bb = v;
        return;
    }
    const double denom = 1 / (va + vb + vc);
    ba = vb * denom;
    bb = vc * denom;
    proj = a + ba * ab + bb * ac;
}

struct ProjRec {  // MR::MeshProjectionResult layout
    int32_t face;
    float px, py, pz;
    int32_t edge;
    float a, b;
    float distSq;
};
static_assert(sizeof(ProjRec) == 32, "MeshProjectionResult layout");

// MRMeshProject.cpp:13-104 findProjectionSubtree with an optional tree map (no region, no predicates)
static ProjRec findProjectionRef(const Mesh& m, const std::vector<Node>& nodes, const V3<float>& pt, float upDistLimitSq,
                                 const AffF* xf, float loDistLimitSq) {
    ProjRec res{-1, 0, 0, 0, -1, 0, 0, upDistLimitSq};
    if (nodes.empty()) return res;
    struct SubTask {
        int n;
        float distSq;
    };
    SubTask st[64];
    int sp = 0;
    auto boxD = [&](int n) {
        const Box3f b = xf ? transformedBox(nodes[n].box, *xf) : nodes[n].box;
        return boxDistSq<float>(b, pt);
    };
    auto add = [&](const SubTask& s) {
        if (s.distSq < res.distSq) st[sp++] = s;
    };
    add(SubTask{0, boxD(0)});
    while (sp > 0) {
        const SubTask s = st[--sp];
        const Node& node = nodes[s.n];
        if (s.distSq >= res.distSq) continue;
        if (node.r < 0) {
            V3<float> a, b, c;
            m.tri(node.l, a, b, c);
            if (xf) {
                a = apply(*xf, a);
                b = apply(*xf, b);
                c = apply(*xf, c);
            }
            V3<double> projD;
            double ba, bb;
            closestPointBary(cvt<double>(pt), cvt<double>(a), cvt<double>(b), cvt<double>(c), projD, ba, bb);
            const V3<float> proj = cvt<float>(projD);
            const float distSq = lengthSq(proj - pt);
            if (distSq < res.distSq) {
                res = ProjRec{node.l, proj.x, proj.y, proj.z, -1, float(ba), float(bb), distSq};
                if (res.distSq <= loDistLimitSq) break;
            }
            continue;
        }
        const SubTask s1{node.l, boxD(node.l)}, s2{node.r, boxD(node.r)};
        if (s1.distSq < s2.distSq) {
            add(s2);
            add(s1);
        } else {
            add(s1);
            add(s2);
        }
    }
    return res;
}

struct Options {
    float minDistSq, maxDistSq;
    int nullOutsideMinMax;
    float windingNumberThreshold, windingNumberBeta;
};

struct Oracle {
    std::vector<float> verts;
    std::vector<int32_t> tris;
    Mesh mesh;
    std::vector<Node> nodes;
    std::vector<Dipole<float>> dipF;
    std::vector<Dipole<double>> dipD;
};

template <typename F> static void parallelFor(size_t n, int threads, F&& f) {
    if (threads <= 1 || n < 1024) {
        for (size_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    const size_t chunk = 256;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&] {
            for (;;) {
                const size_t b = next.fetch_add(chunk);
                if (b >= n) break;
                const size_t e = std::min(n, b + chunk);
                for (size_t i = b; i < e; ++i) f(i);
            }
        });
    for (auto& th : pool) th.join();
}

// AffineXf3f applied to a voxel position: A*x + b with A given by rows (MRAffineXf.h:46, MRMatrix3.h:127-130)
template <typename T> static V3<T> xfPoint(const float* xf, int x, int y, int z) {
    // xf = [A.x.x A.x.y A.x.z A.y.x A.y.y A.y.z A.z.x A.z.y A.z.z b.x b.y b.z], evaluated in float like the reference
    const V3<float> p{float(x), float(y), float(z)};
    const V3<float> r0{xf[0], xf[1], xf[2]}, r1{xf[3], xf[4], xf[5]}, r2{xf[6], xf[7], xf[8]};
    const V3<float> b{xf[9], xf[10], xf[11]};
    const V3<float> q{dot(r0, p) + b.x, dot(r1, p) + b.y, dot(r2, p) + b.z};
    return cvt<T>(q);
}

// calcWithDistances (MRFastWindingNumber.cpp:69-76) at one point; fwnOut receives the winding number
// (NaN when the distance is outside [min,max) and nullOutsideMinMax is set, as the reference skips it).
template <typename T>
static T withDistances(const Oracle* o, const std::vector<Dipole<T>>& dip, const V3<T>& p, const Options& op, double* fwnOut,
                       Counters* cnt) {
    const T resSq = findProjectionDistSq<T>(o->mesh, o->nodes, p, T(op.maxDistSq), T(op.minDistSq), cnt);
    if (op.nullOutsideMinMax && (resSq < T(op.minDistSq) || resSq >= T(op.maxDistSq))) {
        if (fwnOut) *fwnOut = std::numeric_limits<double>::quiet_NaN();
        return std::numeric_limits<T>::quiet_NaN();
    }
    const std::vector<Dipole<float>>* decide = std::is_same<T, double>::value ? &o->dipF : nullptr;
    const T w = calcFWN<T>(o->mesh, o->nodes, dip, p, T(op.windingNumberBeta), -1, cnt, decide, cvt<float>(p));
    if (fwnOut) *fwnOut = w;
    const T sign = w > T(op.windingNumberThreshold) ? T(-1) : T(1);
    return sign * std::sqrt(resSq);
}

}  // namespace orc

using namespace orc;

extern "C" {

void* orc_create(const float* verts, int nv, const int32_t* tris, int nt) {
    auto* o = new Oracle;
    o->verts.assign(verts, verts + 3 * size_t(nv));
    o->tris.assign(tris, tris + 3 * size_t(nt));
    o->mesh = Mesh{o->verts.data(), o->tris.data(), nv, nt};
    buildTree(o->mesh, o->nodes);
    calcDipoles<float>(o->mesh, o->nodes, o->dipF);
    calcDipoles<double>(o->mesh, o->nodes, o->dipD);
    return o;
}

void orc_destroy(void* h) { delete static_cast<Oracle*>(h); }

int orc_num_nodes(void* h) { return int(static_cast<Oracle*>(h)->nodes.size()); }

// nodes: 8 x 4-byte words per node: min.xyz, max.xyz (float), l, r (int32)
void orc_get_nodes(void* h, void* out) {
    auto* o = static_cast<Oracle*>(h);
    std::memcpy(out, o->nodes.data(), o->nodes.size() * sizeof(Node));
}

// dipoles as float[8]: pos.xyz, area, dirArea.xyz, rr (the reference 32-byte record)
void orc_get_dipoles_f(void* h, float* out) {
    auto* o = static_cast<Oracle*>(h);
    for (size_t i = 0; i < o->dipF.size(); ++i) {
        const auto& d = o->dipF[i];
        float* r = out + 8 * i;
        r[0] = d.pos.x; r[1] = d.pos.y; r[2] = d.pos.z; r[3] = d.area;
        r[4] = d.dirArea.x; r[5] = d.dirArea.y; r[6] = d.dirArea.z; r[7] = d.rr;
    }
}
void orc_get_dipoles_d(void* h, double* out) {
    auto* o = static_cast<Oracle*>(h);
    for (size_t i = 0; i < o->dipD.size(); ++i) {
        const auto& d = o->dipD[i];
        double* r = out + 8 * i;
        r[0] = d.pos.x; r[1] = d.pos.y; r[2] = d.pos.z; r[3] = d.area;
        r[4] = d.dirArea.x; r[5] = d.dirArea.y; r[6] = d.dirArea.z; r[7] = d.rr;
    }
}

float orc_solid_angle_f(const float* p, const float* tri) {
    return triangleSolidAngle<float>(V3<float>{p[0], p[1], p[2]}, V3<float>{tri[0], tri[1], tri[2]},
                                     V3<float>{tri[3], tri[4], tri[5]}, V3<float>{tri[6], tri[7], tri[8]});
}
double orc_solid_angle_d(const double* p, const double* tri) {
    return triangleSolidAngle<double>(V3<double>{p[0], p[1], p[2]}, V3<double>{tri[0], tri[1], tri[2]},
                                      V3<double>{tri[3], tri[4], tri[5]}, V3<double>{tri[6], tri[7], tri[8]});
}
void orc_closest_point_d(const double* p, const double* tri, double* out) {
    auto r = closestPointInTriangle<double>(V3<double>{p[0], p[1], p[2]}, V3<double>{tri[0], tri[1], tri[2]},
                                            V3<double>{tri[3], tri[4], tri[5]}, V3<double>{tri[6], tri[7], tri[8]});
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

// calcFromVector (MRFastWindingNumber.cpp:28-38). prec 0: FP32 reference; 1: FP64 oracle.
void orc_from_vector(void* h, const float* pts, int64_t n, float beta, int skipFace, int prec, int threads, double* out) {
    auto* o = static_cast<Oracle*>(h);
    parallelFor(size_t(n), threads, [&](size_t i) {
        const V3<float> q{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        if (prec == 0)
            out[i] = calcFWN<float>(o->mesh, o->nodes, o->dipF, q, beta, skipFace, nullptr);
        else
            out[i] = calcFWN<double>(o->mesh, o->nodes, o->dipD, cvt<double>(q), double(beta), skipFace, nullptr, &o->dipF, q);
    });
}

// calcSelfIntersections (MRFastWindingNumber.cpp:40-52): also returns the winding number at each centroid.
void orc_self_intersections(void* h, float beta, int prec, int threads, uint8_t* bits, double* wn) {
    auto* o = static_cast<Oracle*>(h);
    parallelFor(size_t(o->mesh.nt), threads, [&](size_t f) {
        if (!o->mesh.valid(int(f))) {  // getValidFaces() only (MRFastWindingNumber.cpp:44)
            if (wn) wn[f] = std::numeric_limits<double>::quiet_NaN();
            bits[f] = 0;
            return;
        }
        V3<float> a, b, c;
        o->mesh.tri(int(f), a, b, c);
        const V3<float> q = (1 / 3.0f) * (a + b + c);
        double w;
        if (prec == 0)
            w = calcFWN<float>(o->mesh, o->nodes, o->dipF, q, beta, int(f), nullptr);
        else
            w = calcFWN<double>(o->mesh, o->nodes, o->dipD, cvt<double>(q), double(beta), int(f), nullptr, &o->dipF, q);
        if (wn) wn[f] = w;
        bits[f] = (w < 0 || w > 1) ? 1 : 0;
    });
}

// calcFromGrid (MRFastWindingNumber.cpp:54-67)
void orc_from_grid(void* h, const int* dims, const float* xf, float beta, int prec, int threads, double* out) {
    auto* o = static_cast<Oracle*>(h);
    const size_t sxy = size_t(dims[0]) * dims[1];
    const size_t total = sxy * dims[2];
    parallelFor(total, threads, [&](size_t i) {
        const int z = int(i / sxy), s = int(i % sxy), y = s / dims[0], x = s % dims[0];
        if (prec == 0)
            out[i] = calcFWN<float>(o->mesh, o->nodes, o->dipF, xfPoint<float>(xf, x, y, z), beta, -1, nullptr);
        else
            out[i] = calcFWN<double>(o->mesh, o->nodes, o->dipD, xfPoint<double>(xf, x, y, z), double(beta), -1, nullptr, &o->dipF,
                                     xfPoint<float>(xf, x, y, z));
    });
}

// calcFromGridWithDistances (MRFastWindingNumber.cpp:78-94); fwn may be null.
void orc_from_grid_with_distances(void* h, const int* dims, const float* xf, const Options* op, int prec, int threads, double* out,
                                  double* fwn) {
    auto* o = static_cast<Oracle*>(h);
    const size_t sxy = size_t(dims[0]) * dims[1];
    const size_t total = sxy * dims[2];
    parallelFor(total, threads, [&](size_t i) {
        const int z = int(i / sxy), s = int(i % sxy), y = s / dims[0], x = s % dims[0];
        double* fo = fwn ? fwn + i : nullptr;
        if (prec == 0)
            out[i] = withDistances<float>(o, o->dipF, xfPoint<float>(xf, x, y, z), *op, fo, nullptr);
        else
            out[i] = withDistances<double>(o, o->dipD, xfPoint<double>(xf, x, y, z), *op, fo, nullptr);
    });
}

// calcFromGridWithDistances / calcFromGrid at n chosen voxels of a dims grid (linear ids, x fastest):
// the same voxel centres and per-voxel computation as the whole-grid calls above, for sampling a
// grid too large to evaluate whole on the CPU.  fwn may be null; distances = 0 gives calcFromGrid.
void orc_grid_voxels(void* h, const int* dims, const float* xf, const int64_t* ids, int64_t n, const Options* op, int distances,
                     int prec, int threads, double* out, double* fwn) {
    auto* o = static_cast<Oracle*>(h);
    const int64_t sxy = int64_t(dims[0]) * dims[1];
    parallelFor(size_t(n), threads, [&](size_t k) {
        const int64_t i = ids[k];
        const int z = int(i / sxy), s = int(i % sxy), y = s / dims[0], x = s % dims[0];
        double* fo = fwn ? fwn + k : nullptr;
        if (distances) {
            if (prec == 0)
                out[k] = withDistances<float>(o, o->dipF, xfPoint<float>(xf, x, y, z), *op, fo, nullptr);
            else
                out[k] = withDistances<double>(o, o->dipD, xfPoint<double>(xf, x, y, z), *op, fo, nullptr);
        } else {
            const float beta = op->windingNumberBeta;
            if (prec == 0)
                out[k] = calcFWN<float>(o->mesh, o->nodes, o->dipF, xfPoint<float>(xf, x, y, z), beta, -1, nullptr);
            else
                out[k] = calcFWN<double>(o->mesh, o->nodes, o->dipD, xfPoint<double>(xf, x, y, z), double(beta), -1, nullptr,
                                         &o->dipF, xfPoint<float>(xf, x, y, z));
            if (fo) *fo = out[k];
        }
    });
}

// calcSelfIntersections at n chosen faces: bit and centroid winding number (skipping the face itself)
// of each, as orc_self_intersections computes them for every face.
void orc_self_intersections_at(void* h, const int32_t* faces, int64_t n, float beta, int prec, int threads, uint8_t* bits,
                               double* wn) {
    auto* o = static_cast<Oracle*>(h);
    parallelFor(size_t(n), threads, [&](size_t k) {
        const int f = faces[k];
        if (!o->mesh.valid(f)) {
            wn[k] = std::numeric_limits<double>::quiet_NaN();
            bits[k] = 0;
            return;
        }
        V3<float> a, b, c;
        o->mesh.tri(f, a, b, c);
        const V3<float> q = (1 / 3.0f) * (a + b + c);
        const double w = prec == 0 ? double(calcFWN<float>(o->mesh, o->nodes, o->dipF, q, beta, f, nullptr))
                                   : calcFWN<double>(o->mesh, o->nodes, o->dipD, cvt<double>(q), double(beta), f, nullptr, &o->dipF, q);
        wn[k] = w;
        bits[k] = (w < 0 || w > 1) ? 1 : 0;
    });
}

// the same at arbitrary points (the CPU-only FastWindingNumber::calcWithDistances, MRFastWindingNumber.h:62)
void orc_vector_with_distances(void* h, const float* pts, int64_t n, const Options* op, int prec, int threads, double* out) {
    auto* o = static_cast<Oracle*>(h);
    parallelFor(size_t(n), threads, [&](size_t i) {
        const V3<float> q{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        if (prec == 0)
            out[i] = withDistances<float>(o, o->dipF, q, *op, nullptr, nullptr);
        else
            out[i] = withDistances<double>(o, o->dipD, cvt<double>(q), *op, nullptr, nullptr);
    });
}

// Unsigned closest distance squared only (FP32 reference arithmetic), for distance-only checks.
void orc_dist_sq(void* h, const float* pts, int64_t n, float maxDistSq, float minDistSq, int threads, float* out) {
    auto* o = static_cast<Oracle*>(h);
    parallelFor(size_t(n), threads, [&](size_t i) {
        const V3<float> q{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        out[i] = findProjectionDistSq<float>(o->mesh, o->nodes, q, maxDistSq, minDistSq, nullptr);
    });
}

// Traversal work of the reference (FP32) signed-distance query at the given points:
// counts[0] = closest-point boxes read, [1] = closest-point leaf projections,
// counts[2] = dipole records read, [3] = exact solid angles.  Summed over all points.
void orc_traversal_counts(void* h, const float* pts, int64_t n, const Options* op, uint64_t* counts) {
    auto* o = static_cast<Oracle*>(h);
    Counters c;
    for (int64_t i = 0; i < n; ++i) {
        const V3<float> q{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        (void)withDistances<float>(o, o->dipF, q, *op, nullptr, &c);
    }
    counts[0] = c.cpNodes;
    counts[1] = c.cpLeaves;
    counts[2] = c.fwnNodes;
    counts[3] = c.fwnLeaves;
}

// Exact generalised winding number: sum of all triangle solid angles in FP64 (no far-field approximation).
void orc_exact_wn(void* h, const float* pts, int64_t n, int threads, double* out) {
    auto* o = static_cast<Oracle*>(h);
    parallelFor(size_t(n), threads, [&](size_t i) {
        const V3<double> q{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        double s = 0;
        for (int f = 0; f < o->mesh.nt; ++f) {
            if (!o->mesh.valid(f)) continue;
            V3<float> a, b, c;
            o->mesh.tri(f, a, b, c);
            s += triangleSolidAngle<double>(q, cvt<double>(a), cvt<double>(b), cvt<double>(c));
        }
        out[i] = s / (4 * 3.14159265358979323846);
    });
}

// PointsToMeshProjector::findProjections (MRPointsToMeshProjector.cpp:17-32) with the transform
// simplification of createProjectionTransforms (MRMeshProject.cpp:105-121); objXf / refXf may be null.
void orc_find_projections(void* h, const float* pts, int64_t n, const float* objXf, const float* refXf, float up, float lo,
                          int threads, void* outv) {
    auto* o = static_cast<Oracle*>(h);
    auto* out = static_cast<ProjRec*>(outv);
    AffF pointXf{}, treeXf{};
    const AffF* pp = nullptr;
    const AffF* tp = nullptr;
    if (refXf && !affIsRigid(affFrom(refXf))) {
        treeXf = affFrom(refXf);
        tp = &treeXf;
    }
    if (tp || !refXf) {
        if (objXf) {
            pointXf = affFrom(objXf);
            pp = &pointXf;
        }
    } else {
        pointXf = affInverse(affFrom(refXf));
        if (objXf) pointXf = affCompose(pointXf, affFrom(objXf));
        pp = &pointXf;
    }
    parallelFor(size_t(n), threads, [&](size_t i) {
        V3<float> q{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        if (pp) q = apply(*pp, q);
        out[i] = findProjectionRef(o->mesh, o->nodes, q, up, tp, lo);
    });
}

int orc_is_rigid(const float* xf) { return affIsRigid(affFrom(xf)) ? 1 : 0; }

// AABBTree::refit (MRAABBTree.cpp:62-94) after the vertices moved, then the dipoles again (Mesh::updateCaches
// drops them, MRMesh.cpp:571-583).  changed: nv bits in 64-bit words, or null for all vertices.
void orc_refit(void* h, const float* verts, const uint64_t* changed) {
    auto* o = static_cast<Oracle*>(h);
    std::copy(verts, verts + o->verts.size(), o->verts.begin());
    auto moved = [&](int v) { return !changed || ((changed[v >> 6] >> (v & 63)) & 1ull); };
    std::vector<char> changedNode(o->nodes.size(), 0);
    for (size_t nid = 0; nid < o->nodes.size(); ++nid) {
        Node& node = o->nodes[nid];
        if (node.r >= 0) continue;
        const int f = node.l;
        const int32_t* t = o->mesh.tris + 3 * size_t(f);
        if (!(moved(t[0]) || moved(t[1]) || moved(t[2]))) continue;
        changedNode[nid] = 1;
        node.box = computeFaceBox(o->mesh, f);
    }
    for (int64_t nid = int64_t(o->nodes.size()) - 1; nid >= 0; --nid) {  // NodeId 0 is valid: the root is included
        Node& node = o->nodes[nid];
        if (node.r < 0) continue;
        if (!changedNode[node.l] && !changedNode[node.r]) continue;
        changedNode[nid] = 1;
        node.box = o->nodes[node.l].box;
        node.box.include(o->nodes[node.r].box);
    }
    calcDipoles<float>(o->mesh, o->nodes, o->dipF);
    calcDipoles<double>(o->mesh, o->nodes, o->dipD);
}

}  // extern "C"
