// kernels_heat.cu -- scalar heat (Poisson) instantiations, heat_equation.jl:143-164.
#include "instantiate.cuh"

namespace fe {
void register_heat(std::vector<KernelEntry>& out, std::vector<ElemEntry>& eout) {
    FE_ONE(KIND_QUAD4, 4, PHYS_HEAT)
    FE_ONE(KIND_QUAD4, 1, PHYS_HEAT)
    FE_ONE(KIND_TRI3, 1, PHYS_HEAT)
    FE_ONE(KIND_TRI3, 3, PHYS_HEAT)
    FE_ONE(KIND_QUAD9, 9, PHYS_HEAT)
    FE_ONE(KIND_HEX8, 8, PHYS_HEAT)
    FE_ONE(KIND_TET4, 1, PHYS_HEAT)
    FE_ONE(KIND_TET4, 4, PHYS_HEAT)
    FE_ONE(KIND_WEDGE6, 1, PHYS_HEAT)
    FE_ONE(KIND_WEDGE6, 5, PHYS_HEAT)
    FE_ONE(KIND_HEX27, 27, PHYS_HEAT)
    FE_EA(KIND_HEX27, 27, PHYS_HEAT)
    FE_EA(KIND_QUAD9, 9, PHYS_HEAT)
    // several cell types in one launch: hexahedra / tetrahedra / wedges, quadrilaterals / triangles
    out.push_back(make_entry<KIND_HEX8, 8, KIND_TET4, 1, KIND_WEDGE6, 5, PHYS_HEAT, float>());
    out.push_back(make_entry<KIND_HEX8, 8, KIND_TET4, 1, KIND_WEDGE6, 5, PHYS_HEAT, double>());
    out.push_back(make_entry<KIND_QUAD4, 4, KIND_TRI3, 1, -1, 0, PHYS_HEAT, float>());
    out.push_back(make_entry<KIND_QUAD4, 4, KIND_TRI3, 1, -1, 0, PHYS_HEAT, double>());
}
}  // namespace fe
