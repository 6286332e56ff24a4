// fvc_variant_c2.cu -- integrator kernels for Cartesian 2D meshes.
#include "fvc_advect_impl.cuh"

namespace fvc {
template struct Variant<2, 0>;
}  // namespace fvc
