// Declarations standing in for the few OpenVDB names that MeshLib's mesher translation unit
// (MRVoxels/MRMarchingCubes.cpp) and its headers mention, so the reference mesher compiles from
// its own sources without the un-vendored OpenVDB.  The VDB volume path is compiled but never run:
// the oracle's golden vectors come from dense SimpleVolume inputs only, and every member here that
// would be reached at run time aborts.
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <memory>

namespace openvdb {

using Index = uint32_t;
using Index32 = uint32_t;
using Index64 = uint64_t;

class Coord {
public:
    Coord() = default;
    Coord(int x, int y, int z) : v_{x, y, z} {}
    int x() const { return v_[0]; }
    int y() const { return v_[1]; }
    int z() const { return v_[2]; }
    int operator[](int i) const { return v_[i]; }
    int& operator[](int i) { return v_[i]; }

private:
    int v_[3] = {0, 0, 0};
};

class CoordBBox {
public:
    CoordBBox() = default;
    CoordBBox(const Coord& mn, const Coord& mx) : min_(mn), max_(mx) {}
    const Coord& min() const { return min_; }
    const Coord& max() const { return max_; }

private:
    Coord min_, max_;
};

template <typename T>
class ValueAccessorStub {
public:
    bool probeValue(const Coord&, T&) const { std::abort(); }
    const T& getValue(const Coord&) const { std::abort(); }
};

template <typename T>
class GridStub {
public:
    using Ptr = std::shared_ptr<GridStub>;
    using ConstPtr = std::shared_ptr<const GridStub>;
    using ValueType = T;
    using ConstAccessor = ValueAccessorStub<T>;
    ConstAccessor getConstAccessor() const { return {}; }
    CoordBBox evalActiveVoxelBoundingBox() const { std::abort(); }
    std::size_t memUsage() const { return 0; }
};

using FloatGrid = GridStub<float>;

}  // namespace openvdb
