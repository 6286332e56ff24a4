// fvc_variant_u2.cu -- integrator kernels for unstructured 2D meshes.
#include "fvc_advect_impl.cuh"

namespace fvc {
template struct Variant<2, 1>;
}  // namespace fvc
