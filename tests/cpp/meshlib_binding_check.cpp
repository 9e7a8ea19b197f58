// Syntax check of the MeshLib-side binding (include/MRGbFastWindingNumber.h) against MeshLib's own
// headers: the class must be concrete (both interfaces fully overridden), constructible from a
// const Mesh& the way the factory slot of MRViewer/MRCudaAccessor.h:41 calls it, and visible as
// IFastWindingNumberByParts to callers that probe with dynamic_pointer_cast (MRVoxels/MROffset.cpp:194).
#include "MRGbFastWindingNumber.h"

#include <functional>
#include <memory>

std::unique_ptr<MR::IFastWindingNumber> makeGbFastWindingNumber( const MR::Mesh& mesh )
{
    return std::make_unique<MR::GbFastWindingNumber>( mesh );
}

std::shared_ptr<MR::IFastWindingNumberByParts> asByParts( const std::shared_ptr<MR::IFastWindingNumber>& p )
{
    return std::dynamic_pointer_cast<MR::IFastWindingNumberByParts>( p );
}

// the factory type of the application's slot (MRViewer/MRCudaAccessor.h:25)
using Constructor = std::function<std::unique_ptr<MR::IFastWindingNumber>( const MR::Mesh& )>;
const Constructor kFactory = []( const MR::Mesh& mesh ) { return makeGbFastWindingNumber( mesh ); };
