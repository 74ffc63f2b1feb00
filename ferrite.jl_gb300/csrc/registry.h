// registry.h -- the compiled tile-kernel instantiations and how the host picks one.
#pragma once
#include <vector>

#include "common.h"

namespace fe {

struct KernelEntry {
    int kind[MAX_SUB];   // -1 = unused slot
    int nq[MAX_SUB];
    int phys;            // 1 heat, 2 elastic, 3 neo-hooke
    int fp64;            // 0 = mixed precision, 1 = FP64
    const void* fn;      // __global__ tile_kernel<...>
    int table_bytes[MAX_SUB];  // cell-table bytes per lane group of each slot
    int groups[MAX_SUB];       // lane groups per CTA of each slot
    int ea_only;               // gather-only form: every subdomain two-phase
};

// adjoint kernels: one instantiation per (kind, quadrature points, physics, precision)
struct AdjEntry {
    int kind, nq, phys, fp64;
    const void* fn;      // __global__ adjoint_kernel<...>
    int smem;            // dynamic shared memory per CTA
};

// per-cell element-matrix kernels (element_kernel): one per (kind, quadrature points, physics,
// precision)
struct ElemEntry {
    int kind, nq, phys, fp64;
    const void* fn;      // __global__ element_kernel<..., 1>: into the two-phase scratch
    const void* fn_out;  // __global__ element_kernel<..., 2>: into the caller's element arrays
    const void* fn_tc;   // tensor-core form into the two-phase scratch (nullptr: none)
    int group_bytes;     // shared memory per lane group (the shape tables come on top)
    int groups;          // lane groups per CTA
};

void register_heat(std::vector<KernelEntry>& out, std::vector<ElemEntry>& eout);
void register_elastic(std::vector<KernelEntry>& out, std::vector<ElemEntry>& eout);
void register_neo(std::vector<KernelEntry>& out, std::vector<ElemEntry>& eout);
void register_adjoint(std::vector<AdjEntry>& out);
const void* adjoint_node_sum_fn(bool fp64);

}  // namespace fe
