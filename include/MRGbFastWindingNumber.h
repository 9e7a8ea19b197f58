// MRGbFastWindingNumber.h -- the MeshLib-side class that makes the GB300 library a drop-in
// MR::IFastWindingNumber / MR::IFastWindingNumberByParts (MRMesh/MRFastWindingNumber.h:11-107).
//
// Header-only; it is compiled inside MeshLib (it includes MeshLib's own headers) and links
// libgbfwn.so.  It plays the part of MR::Cuda::FastWindingNumber (MRCuda/MRCudaFastWindingNumber.h:17-39):
// it holds the mesh by reference (the mesh must outlive it), uploads it and builds the tree on first
// use (as prepareData_ does, MRCuda/MRCudaFastWindingNumber.cpp:46-85), resizes the caller's result
// containers, and reports errors as Expected strings ("Operation was canceled" on a cancelled
// progress callback).  Register it in the application's factory slot
// (MRViewer/MRCudaAccessor.h:41):
//
//   MR::CudaAccessor::setCudaFastWindingNumberConstructor(
//       []( const MR::Mesh& mesh ) { return std::make_unique<MR::GbFastWindingNumber>( mesh ); } );
//
// Callers that detect the by-parts interface with dynamic_pointer_cast (MRVoxels/MROffset.cpp:194,
// MRVoxels/MRVDBConversions.cpp:534) find it, as they find it on the reference's GPU class.
#pragma once

#include "MRMesh/MRAffineXf3.h"
#include "MRMesh/MRBitSet.h"
#include "MRMesh/MRDistanceToMeshOptions.h"
#include "MRMesh/MRFastWindingNumber.h"
#include "MRMesh/MRMesh.h"
#include "MRMesh/MRVector3.h"

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "gbfwn.h"

namespace MR
{

class GbFastWindingNumber : public IFastWindingNumber, public IFastWindingNumberByParts
{
public:
    /// the mesh must outlive this object; `device` is the CUDA device ordinal the data lives on
    explicit GbFastWindingNumber( const Mesh& mesh, int device = 0 ) : mesh_( mesh ), device_( device ) {}
    GbFastWindingNumber( const GbFastWindingNumber& ) = delete;
    GbFastWindingNumber& operator=( const GbFastWindingNumber& ) = delete;
    ~GbFastWindingNumber() override { if ( h_ ) gbfwn_destroy( h_ ); }

    Expected<void> calcFromVector( std::vector<float>& res, const std::vector<Vector3f>& points, float beta,
                                   FaceId skipFace, const ProgressCallback& cb ) override
    {
        if ( auto e = prepare_(); !e )
            return e;
        res.resize( points.size() );
        if ( points.empty() )
            return progressDone_( cb );
        static_assert( sizeof( Vector3f ) == 3 * sizeof( float ), "points are read as 3 floats each" );
        return wrap_( gbfwn_from_vector( h_, &points[0].x, std::int64_t( points.size() ), beta,
                                         skipFace.valid() ? int( skipFace ) : -1, res.data(), progress_, (void*)&cb ) );
    }

    Expected<void> calcSelfIntersections( FaceBitSet& res, float beta, const ProgressCallback& cb ) override
    {
        if ( auto e = prepare_(); !e )
            return e;
        const size_t faces = mesh_.topology.faceSize();
        // FaceBitSet keeps 64-bit blocks, bit f of block f / 64: the library's word layout
        std::vector<BitSet::block_type> blocks( ( faces + 63 ) / 64 );
        static_assert( sizeof( BitSet::block_type ) == sizeof( std::uint64_t ), "64-bit blocks" );
        if ( auto e = wrap_( gbfwn_self_intersections( h_, beta, blocks.empty() ? nullptr : blocks.data(), nullptr, progress_,
                                                       (void*)&cb ) ); !e )
            return e;
        res = FaceBitSet( BitSet::fromBlocks( std::move( blocks ) ) );
        res.resize( faces );
        return {};
    }

    Expected<void> calcFromGrid( std::vector<float>& res, const Vector3i& dims, const AffineXf3f& gridToMeshXf, float beta,
                                 const ProgressCallback& cb ) override
    {
        if ( auto e = prepare_(); !e )
            return e;
        res.resize( voxels_( dims ) );
        if ( res.empty() )
            return progressDone_( cb );
        const Grid g( dims, gridToMeshXf );
        return wrap_( gbfwn_from_grid( h_, g.dims, g.xf, beta, res.data(), progress_, (void*)&cb ) );
    }

    Expected<void> calcFromGridWithDistances( std::vector<float>& res, const Vector3i& dims, const AffineXf3f& gridToMeshXf,
                                              const DistanceToMeshOptions& options, const ProgressCallback& cb ) override
    {
        if ( auto e = prepare_(); !e )
            return e;
        res.resize( voxels_( dims ) );
        if ( res.empty() )
            return progressDone_( cb );
        const Grid g( dims, gridToMeshXf );
        const gbfwn_dist_opts o = opts_( options );
        return wrap_( gbfwn_from_grid_with_distances( h_, g.dims, g.xf, &o, res.data(), progress_, (void*)&cb ) );
    }

    Expected<void> calcFromGridByParts( GridByPartsFunc resFunc, const Vector3i& dims, const AffineXf3f& gridToMeshXf,
                                        float beta, int layerOverlap, const ProgressCallback& cb ) override
    {
        if ( auto e = prepare_(); !e )
            return e;
        if ( voxels_( dims ) == 0 )
            return progressDone_( cb );
        const Grid g( dims, gridToMeshXf );
        Slabs s{ &resFunc, {} };
        return byParts_( s, gbfwn_from_grid_by_parts( h_, g.dims, g.xf, beta, layerOverlap, 0, slab_, &s, progress_,
                                                      (void*)&cb ) );
    }

    Expected<void> calcFromGridWithDistancesByParts( GridByPartsFunc resFunc, const Vector3i& dims,
                                                     const AffineXf3f& gridToMeshXf, const DistanceToMeshOptions& options,
                                                     int layerOverlap, const ProgressCallback& cb ) override
    {
        if ( auto e = prepare_(); !e )
            return e;
        if ( voxels_( dims ) == 0 )
            return progressDone_( cb );
        const Grid g( dims, gridToMeshXf );
        const gbfwn_dist_opts o = opts_( options );
        Slabs s{ &resFunc, {} };
        return byParts_( s, gbfwn_from_grid_with_distances_by_parts( h_, g.dims, g.xf, &o, layerOverlap, 0, slab_, &s,
                                                                     progress_, (void*)&cb ) );
    }

private:
    // the grid in the C ABI's form: int32 dims and the 12 floats of the affine map (rows, then b)
    struct Grid
    {
        std::int32_t dims[3];
        float xf[12];
        Grid( const Vector3i& d, const AffineXf3f& x )
            : dims{ d.x, d.y, d.z }
            , xf{ x.A.x.x, x.A.x.y, x.A.x.z, x.A.y.x, x.A.y.y, x.A.y.z, x.A.z.x, x.A.z.y, x.A.z.z, x.b.x, x.b.y, x.b.z }
        {}
    };

    // the by-parts callback's state: the caller's function and the first error it returned
    struct Slabs
    {
        GridByPartsFunc* func;
        std::string error;
    };

    static size_t voxels_( const Vector3i& d )
    {
        return ( d.x > 0 && d.y > 0 && d.z > 0 ) ? size_t( d.x ) * size_t( d.y ) * size_t( d.z ) : 0;
    }

    static gbfwn_dist_opts opts_( const DistanceToMeshOptions& o )
    {
        return gbfwn_dist_opts{ o.minDistSq, o.maxDistSq, o.nullOutsideMinMax ? 1 : 0, o.windingNumberThreshold,
                                o.windingNumberBeta };
    }

    // lazy upload + tree build, like MR::Cuda::FastWindingNumber::prepareData_; deleted faces are
    // passed as (-1, -1, -1), which the library leaves out of the tree (MeshLib's getValidFaces())
    Expected<void> prepare_()
    {
        if ( h_ )
            return {};
        const size_t faces = mesh_.topology.faceSize();
        std::vector<std::int32_t> tris( 3 * faces, -1 );
        for ( FaceId f{ 0 }; f < FaceId( int( faces ) ); ++f )
        {
            if ( !mesh_.topology.hasFace( f ) )
                continue;
            const ThreeVertIds v = mesh_.topology.getTriVerts( f );
            for ( int k = 0; k < 3; ++k )
                tris[3 * size_t( f ) + k] = int( v[k] );
        }
        static_assert( sizeof( Vector3f ) == 3 * sizeof( float ), "vertices are read as 3 floats each" );
        const float* verts = mesh_.points.empty() ? nullptr : &mesh_.points.data()->x;
        return wrap_( gbfwn_create( verts, std::int64_t( mesh_.points.size() ), tris.empty() ? nullptr : tris.data(),
                                    std::int64_t( faces ), device_, &h_ ) );
    }

    Expected<void> byParts_( Slabs& s, int st ) const
    {
        if ( st != GBFWN_OK && !s.error.empty() )
            return unexpected( std::move( s.error ) );  // the caller's own error, passed through
        return wrap_( st );
    }

    static int slab_( const float* data, const std::int32_t dims[3], std::int32_t zOffset, void* user )
    {
        auto& s = *static_cast<Slabs*>( user );
        std::vector<float> v( data, data + size_t( dims[0] ) * size_t( dims[1] ) * size_t( dims[2] ) );
        auto r = ( *s.func )( std::move( v ), Vector3i( dims[0], dims[1], dims[2] ), int( zOffset ) );
        if ( r )
            return 0;
        s.error = r.error();
        return GBFWN_CANCELLED;  // any nonzero status stops the call; the error string above is returned
    }

    static int progress_( float p, void* user )
    {
        const auto& cb = *static_cast<const ProgressCallback*>( user );
        return !cb || cb( p ) ? 1 : 0;
    }

    static Expected<void> progressDone_( const ProgressCallback& cb )
    {
        if ( cb && !cb( 1.0f ) )
            return unexpectedOperationCanceled();
        return {};
    }

    static Expected<void> wrap_( int st )
    {
        if ( st == GBFWN_OK )
            return {};
        if ( st == GBFWN_CANCELLED )
            return unexpectedOperationCanceled();
        return unexpected( std::string( gbfwn_last_error() ) );
    }

    const Mesh& mesh_;
    int device_ = 0;
    gbfwn_handle h_ = nullptr;
};

} // namespace MR
