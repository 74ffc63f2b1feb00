// plan.h -- host-side set-up of a handle: validation of the Ferrite arrays, the compact
// element-to-nzval index map, and the owner-tile plan the kernels execute.
#pragma once
#include <stdint.h>

#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "common.h"
#include "ferrite_gb300.h"

namespace fe {

// Allocator whose value-less construct leaves the element uninitialised: large host buffers that
// are written in full right after they are sized (in parallel, so the first touch of their pages
// is spread over the threads) skip the serial zero fill of std::vector::resize.
template <typename T>
struct DefaultInitAllocator : std::allocator<T> {
    template <typename U>
    struct rebind {
        using other = DefaultInitAllocator<U>;
    };
    DefaultInitAllocator() = default;
    template <typename U>
    DefaultInitAllocator(const DefaultInitAllocator<U>&) noexcept {}
    template <typename U>
    void construct(U* p) noexcept(std::is_nothrow_default_constructible<U>::value) {
        ::new ((void*)p) U;
    }
    template <typename U, typename... A>
    void construct(U* p, A&&... a) {
        ::new ((void*)p) U(std::forward<A>(a)...);
    }
};
template <typename T>
using HostBuf = std::vector<T, DefaultInitAllocator<T>>;

struct HostSub {
    int32_t cell_type = 0, ip_order = 0, kind = 0;
    int32_t nb = 0, ng = 0, nq = 0, dim = 0, nc = 0;
    int64_t n_cells = 0;
    std::vector<int32_t> cellid;   // 0-based Ferrite cell ids
    std::vector<int32_t> conn;     // [n][ng] 0-based node ids
    std::vector<int32_t> ents;     // [n][nb] entity ids
    HostBuf<uint8_t> rank8;        // [n][nb][nb] (j-major), 255 = missing
    HostBuf<uint16_t> rank16;      // used when a rank exceeds 254; 65535 = missing
    bool wide_rank = false;
    std::vector<double> w, N, dN, dM;  // reference tables (row-major, as passed)
};

struct HostProblem {
    int32_t dim = 0;
    int64_t n_nodes = 0, n_cells = 0, ndofs = 0, nnz = 0;
    int32_t nc = 0;            // components per entity
    int64_t n_ent = 0;         // ndofs / nc
    std::vector<double> nodes; // [n_nodes][dim]
    std::vector<HostSub> subs;
    std::vector<int64_t> colptr;          // 1-based copy
    std::vector<int64_t> cell_dofs_off;   // per Ferrite cell: 1-based offset (for index-map queries)
    std::vector<int32_t> cell_sub;        // per Ferrite cell: subdomain or -1
    std::vector<int32_t> cell_local;      // per Ferrite cell: index within its subdomain
    HostBuf<int64_t> cell_dofs;           // copy of dh.cell_dofs (for index-map queries / errors)
};

struct PlanOptions {
    // staging values per tile (4 bytes each in mixed precision). 13056 is the largest capacity
    // whose 128^3 Q1 hexahedron tiles keep two CTAs per SM; a plan whose CTA lands just past
    // its occupancy line is re-planned smaller at its first assembly
    int32_t stage_cap = 13056;
    int32_t ent_cap = 1024;     // owned entities per tile
    int32_t red_cap = 2048;     // owned blocks (reduce lanes) per tile
    int32_t out_cap = 0;        // output-buffer doubles of one reduce pass; 0: 37.5 % of stage_cap
    int32_t resolved_out_cap() const {
        if (out_cap > 0) return out_cap;
        const int32_t v = (int32_t)(0.375 * stage_cap) / 256 * 256;
        return v < 1024 ? 1024 : (v > 16384 ? 16384 : v);
    }
};

struct Plan {
    HostBuf<uint8_t> rec;           // tile records, concatenated (each 16-byte aligned)
    std::vector<int64_t> rec_off;   // [n_tiles + 1] byte offsets
    int64_t n_tiles = 0;
    int32_t max_rec = 0, max_nodes = 0, max_stage = 0, max_out = 0;
    int64_t visits = 0, items = 0;
};

struct Error {
    int code = 0;
    std::string msg;
    int64_t cell = 0, row = 0, col = 0;
};

int kind_of(int32_t cell_type, int32_t ip_order, int32_t& nb, int32_t& ng, int32_t& rdim);

// Fill HostProblem from the C-ABI descriptors; validates sizes, bounds and the dof layout,
// builds the entity ranks (the index map). Returns an FE_* code.
struct CreateInput {
    const fe_grid_desc* grid;
    int32_t n_sub;
    const fe_subdomain_desc* subs;
    const fe_dof_desc* dofs;
    const fe_csc_desc* pattern;
    // the pattern's rowval stays in device memory (pattern->rowval may be null): build_problem
    // skips the pattern check and the rank tables, which device_index_map then builds
    bool device_pattern = false;
};
int build_problem(const CreateInput& in, HostProblem& hp, Error& err);
// The entity-blocked pattern check and the rank tables (the element -> nzval index map) of a
// device-resident pattern, on the device (pattern.cu): hp holds the host set-up of
// build_problem (entities, colptr); cp_dev / rv_dev are the pattern's device arrays.
int device_index_map(HostProblem& hp, const int64_t* cp_dev, const int64_t* rv_dev, Error& err);
int build_plan(const HostProblem& hp, const PlanOptions& opt, Plan& plan, Error& err);
int check_plan(const HostProblem& hp, const Plan& plan, Error& err);
// rank of entity(i) among the row entities of entity(j)'s columns for cell k of sub s, or -1
inline int rank_of(const HostSub& hs, int64_t k, int j, int i) {
    const size_t q = ((size_t)k * hs.nb + j) * hs.nb + i;
    if (hs.wide_rank) return hs.rank16[q] == 0xFFFF ? -1 : hs.rank16[q];
    return hs.rank8[q] == 255 ? -1 : hs.rank8[q];
}

}  // namespace fe
