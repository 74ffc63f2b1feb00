// kernels_neo.cu -- compressible Neo-Hooke tangent + residual instantiations,
// hyperelasticity.jl:157-276, including the mixed hexahedron/tetrahedron/wedge kernel.
#include "instantiate.cuh"

namespace fe {
void register_neo(std::vector<KernelEntry>& out, std::vector<ElemEntry>& eout) {
    FE_ONE(KIND_HEX8, 8, PHYS_NEO)
    FE_ONE(KIND_TET4, 1, PHYS_NEO)
    FE_ONE(KIND_TET4, 4, PHYS_NEO)
    FE_ONE(KIND_WEDGE6, 5, PHYS_NEO)
    FE_ONE(KIND_WEDGE6, 1, PHYS_NEO)
    out.push_back(make_entry<KIND_HEX8, 8, KIND_TET4, 1, KIND_WEDGE6, 5, PHYS_NEO, float>());
    out.push_back(make_entry<KIND_HEX8, 8, KIND_TET4, 1, KIND_WEDGE6, 5, PHYS_NEO, double>());
    // the gather-only form of the same mix, for when every cell type is assembled two-phase
    out.push_back(make_entry<KIND_HEX8, 8, KIND_TET4, 1, KIND_WEDGE6, 5, PHYS_NEO, float, true>());
    out.push_back(make_entry<KIND_HEX8, 8, KIND_TET4, 1, KIND_WEDGE6, 5, PHYS_NEO, double, true>());
}
}  // namespace fe
