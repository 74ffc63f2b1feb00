// kernels_elastic.cu -- small-strain isotropic elasticity instantiations,
// threaded_assembly.jl:105-132 (per-cell modulus: topology_optimization.jl:347-383).
#include "instantiate.cuh"

namespace fe {
void register_elastic(std::vector<KernelEntry>& out, std::vector<ElemEntry>& eout) {
    FE_ONE(KIND_HEX8, 8, PHYS_ELASTIC)
    FE_ONE(KIND_HEX27, 27, PHYS_ELASTIC)
    FE_EA(KIND_HEX27, 27, PHYS_ELASTIC)
    FE_ONE(KIND_TET4, 1, PHYS_ELASTIC)
    FE_ONE(KIND_TET4, 4, PHYS_ELASTIC)
    FE_ONE(KIND_WEDGE6, 5, PHYS_ELASTIC)
    FE_ONE(KIND_QUAD4, 4, PHYS_ELASTIC)
    // P1 triangles, ip^2, 1 or 3 points (docs/src/literate-tutorials/linear_elasticity.jl)
    FE_ONE(KIND_TRI3, 1, PHYS_ELASTIC)
    FE_ONE(KIND_TRI3, 3, PHYS_ELASTIC)
    // Q2 quadrilaterals, ip^2, 3x3 Gauss (fused form: 9 base functions)
    FE_ONE(KIND_QUAD9, 9, PHYS_ELASTIC)
    // several cell types in one launch: hexahedra / tetrahedra / wedges, quadrilaterals / triangles
    out.push_back(make_entry<KIND_HEX8, 8, KIND_TET4, 1, KIND_WEDGE6, 5, PHYS_ELASTIC, float>());
    out.push_back(make_entry<KIND_HEX8, 8, KIND_TET4, 1, KIND_WEDGE6, 5, PHYS_ELASTIC, double>());
    out.push_back(make_entry<KIND_QUAD4, 4, KIND_TRI3, 1, -1, 0, PHYS_ELASTIC, float>());
    out.push_back(make_entry<KIND_QUAD4, 4, KIND_TRI3, 1, -1, 0, PHYS_ELASTIC, double>());
}
}  // namespace fe
