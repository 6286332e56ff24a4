// fvc_variant_u3.cu -- integrator kernels for unstructured 3D meshes.
#include "fvc_advect_impl.cuh"

namespace fvc {
template struct Variant<3, 1>;
}  // namespace fvc
