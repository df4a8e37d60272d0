// Link shim for the reference pin library (test infrastructure only).
//
// The pinned arithmetic is the reference's own VolumeRAM::getVoxelNormalizedLinear
// (src/core/datastructures/volume/volumeram.cpp) and VolumeAtomic<T>
// voxel access (include/voreen/core/datastructures/volume/volumeatomic.h),
// compiled from the reference tree. Those objects reference a handful of
// framework symbols that the pinned code paths never call; this file gives
// them trivial definitions so the library links without the rest of the
// framework (serialisation, GL converters, logging back ends).
#include <cstdlib>

#include "voreen/core/datastructures/meta/realworldmappingmetadata.h"
#include "voreen/core/datastructures/volume/volumefactory.h"
#include "voreen/core/datastructures/volume/volumerepresentation.h"

namespace voreen {
const std::string VolumeRepresentation::loggerCat_("pin");
VolumeRepresentation::VolumeRepresentation(const tgt::svec3& d) : dimensions_(d) {
    numVoxels_ = d.x * d.y * d.z;
}
tgt::svec3 VolumeRepresentation::getDimensions() const { return dimensions_; }
size_t VolumeRepresentation::getNumVoxels() const { return numVoxels_; }

// never reached by the pinned paths
std::string RealWorldMapping::getUnit() const { std::abort(); }
float RealWorldMapping::normalizedToRealWorld(float) const { std::abort(); }
const std::string VolumeFactory::loggerCat_("pin");
VolumeFactory::VolumeFactory() {}
VolumeFactory::~VolumeFactory() {}
}  // namespace voreen

namespace tgt {
void LogManager::log(const std::string&, LogLevel, const std::string&, const std::string&) {}
}  // namespace tgt
