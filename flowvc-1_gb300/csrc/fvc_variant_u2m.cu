// Mixed-precision form, 2D unstructured meshes.
#include "fvc_mixed_impl.cuh"

namespace fvc {
template struct VariantMx<2>;
}  // namespace fvc
