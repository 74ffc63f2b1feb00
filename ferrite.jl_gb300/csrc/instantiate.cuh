// instantiate.cuh -- helpers to list tile-kernel instantiations in the registry.
#pragma once
#include <type_traits>

#include "registry.h"
#include "tile_kernel.cuh"

namespace fe {

template <int K, int Q, int PH, typename R>
constexpr int table_bytes_or0() {
    if constexpr (K < 0) return 0;
    else return cell_table_bytes<K, Q, PH, R>();
}
template <int K>
constexpr int groups_or0() {
    if constexpr (K < 0) return 0;
    else return THREADS / ElemT<K>::GS;
}

template <int K0, int Q0, int K1, int Q1, int K2, int Q2, int PH, typename R, bool EAK = false>
KernelEntry make_entry() {
    KernelEntry e;
    e.ea_only = EAK ? 1 : 0;
    e.kind[0] = K0; e.kind[1] = K1; e.kind[2] = K2;
    e.nq[0] = Q0; e.nq[1] = Q1; e.nq[2] = Q2;
    e.phys = PH;
    e.fp64 = std::is_same<R, double>::value ? 1 : 0;
    e.fn = (const void*)&tile_kernel<K0, Q0, K1, Q1, K2, Q2, PH, R, EAK>;
    e.table_bytes[0] = table_bytes_or0<K0, Q0, PH, R>();
    e.table_bytes[1] = table_bytes_or0<K1, Q1, PH, R>();
    e.table_bytes[2] = table_bytes_or0<K2, Q2, PH, R>();
    e.groups[0] = groups_or0<K0>();
    e.groups[1] = groups_or0<K1>();
    e.groups[2] = groups_or0<K2>();
    return e;
}

template <int K, int Q, int PH, typename R>
ElemEntry make_elem_entry() {
    ElemEntry e;
    e.kind = K;
    e.nq = Q;
    e.phys = PH;
    e.fp64 = std::is_same<R, double>::value ? 1 : 0;
    e.fn = (const void*)&element_kernel<K, Q, PH, R, 1>;
    e.fn_out = (const void*)&element_kernel<K, Q, PH, R, 2>;
    e.fn_tc = nullptr;
    if constexpr (K == KIND_HEX27 && Q == 27 && PH == PHYS_ELASTIC && std::is_same<R, float>::value)
        e.fn_tc = (const void*)&element_kernel_tc<PHYS_ELASTIC>;
    e.group_bytes = EaGroup<K, Q, PH, R>::BYTES;
    e.groups = THREADS / ElemT<K>::GS;
    return e;
}

#define FE_ONE(K, Q, PH)                                                  \
    out.push_back(make_entry<K, Q, -1, 0, -1, 0, PH, float>());           \
    out.push_back(make_entry<K, Q, -1, 0, -1, 0, PH, double>());          \
    eout.push_back(make_elem_entry<K, Q, PH, float>());                   \
    eout.push_back(make_elem_entry<K, Q, PH, double>());

// the gather-only tile kernel of a kind whose default form is two-phase
#define FE_EA(K, Q, PH)                                                   \
    out.push_back(make_entry<K, Q, -1, 0, -1, 0, PH, float, true>());     \
    out.push_back(make_entry<K, Q, -1, 0, -1, 0, PH, double, true>());

}  // namespace fe
