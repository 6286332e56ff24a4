// Mixed-precision form, 3D unstructured meshes.
#include "fvc_mixed_impl.cuh"

namespace fvc {
template struct VariantMx<3>;
}  // namespace fvc
