// kernels_adjoint.cu -- adjoint kernel instantiations (mixed precision and FP64).
#include "adjoint.cuh"
#include "registry.h"

namespace fe {

template <int K, int Q, int PH, typename R>
AdjEntry make_adj() {
    AdjEntry e;
    e.kind = K;
    e.nq = Q;
    e.phys = PH;
    e.fp64 = sizeof(R) == 8;
    e.fn = (const void*)&adjoint_kernel<K, Q, PH, R>;
    e.smem = AdjT<K, Q, PH, R>::SMEM_BYTES;
    return e;
}

#define FE_ADJ(K, Q, PH)                           \
    out.push_back(make_adj<K, Q, PH, float>());    \
    out.push_back(make_adj<K, Q, PH, double>());

void register_adjoint(std::vector<AdjEntry>& out) {
    FE_ADJ(KIND_HEX8, 8, PHYS_ELASTIC)
    FE_ADJ(KIND_TET4, 1, PHYS_ELASTIC)
    FE_ADJ(KIND_TET4, 4, PHYS_ELASTIC)
    FE_ADJ(KIND_WEDGE6, 5, PHYS_ELASTIC)
    FE_ADJ(KIND_QUAD4, 4, PHYS_ELASTIC)
    FE_ADJ(KIND_QUAD4, 4, PHYS_HEAT)
    FE_ADJ(KIND_QUAD4, 1, PHYS_HEAT)
    FE_ADJ(KIND_TRI3, 1, PHYS_HEAT)
    FE_ADJ(KIND_TRI3, 3, PHYS_HEAT)
    FE_ADJ(KIND_HEX8, 8, PHYS_HEAT)
    FE_ADJ(KIND_TET4, 1, PHYS_HEAT)
    FE_ADJ(KIND_TET4, 4, PHYS_HEAT)
}

const void* adjoint_node_sum_fn(bool fp64) {
    return fp64 ? (const void*)&adjoint_node_sum<double> : (const void*)&adjoint_node_sum<float>;
}

}  // namespace fe
