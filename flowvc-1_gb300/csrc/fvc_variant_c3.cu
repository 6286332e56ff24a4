// fvc_variant_c3.cu -- integrator kernels for Cartesian 3D meshes.
#include "fvc_advect_impl.cuh"

namespace fvc {
template struct Variant<3, 0>;
}  // namespace fvc
