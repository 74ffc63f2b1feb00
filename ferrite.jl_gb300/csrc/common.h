// common.h -- internal data layout shared by the planner (host) and the tile kernels.
//
// Design in one paragraph: the nzval array of a CSC matrix is a concatenation of columns,
// and the columns of one dof entity (a vertex, edge, face or cell interior carrying
// n_components interleaved dofs) are adjacent. The planner partitions the entities into
// spatially compact "owner tiles"; a tile's nzval is a handful of contiguous ranges. One CTA
// assembles one tile completely: it evaluates every cell that touches the tile (geometry in
// registers, shape-gradient tables in shared memory), accumulates the contributions to the
// tile's own columns in a shared-memory accumulator, and writes each nzval entry exactly
// once, coalesced. No atomics and no coloring passes over global memory; the order of the
// additions into every entry is fixed by the plan, so results are bitwise reproducible.
#pragma once
#include <stdint.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace fe {

// element kinds (cell type x interpolation)
enum Kind : int32_t {
    KIND_TRI3 = 0,
    KIND_QUAD4 = 1,
    KIND_TET4 = 2,
    KIND_HEX8 = 3,
    KIND_WEDGE6 = 4,
    KIND_HEX27 = 5,
    KIND_QUAD9 = 6,
    NKIND = 7
};

constexpr int MAX_NB = 27;   // base functions per cell
constexpr int MAX_NG = 8;    // geometric nodes per cell
constexpr int MAX_NQ = 27;   // quadrature points per cell
constexpr int MAX_SUB = 3;   // subdomains one kernel handles

// item word: local base function j (5 bits) | tile-local entity (10 bits) | k (6 bits), where
// k is the position of the item's cell among the cells of that entity (cell order)
constexpr int ITEM_J_BITS = 5, ITEM_ENT_BITS = 10, ITEM_K_BITS = 6;
constexpr int MAX_TILE_ENTS = 1 << ITEM_ENT_BITS;
constexpr int MAX_ENT_CELLS = (1 << ITEM_K_BITS) - 1;
__host__ __device__ inline uint32_t pack_item(uint32_t j, uint32_t ent, uint32_t k) {
    return j | (ent << ITEM_J_BITS) | (k << (ITEM_J_BITS + ITEM_ENT_BITS));
}

struct TileDesc {
    int32_t seg_begin, seg_end;      // into segs[]: the tile's cells, one segment per subdomain
    int32_t range_begin, range_end;  // into ranges[]: the owned entities as runs of ids
    int32_t ent_begin;               // into emeta[] / eids[]
    int32_t n_ent;                   // owned entities
    int32_t n_red;                   // owned (entity, row entity) blocks = reduce lanes
    int32_t stage_vals;              // staging values (block contributions + f contributions)
    int32_t map_bytes;               // contribution map bytes
    int32_t red_begin;               // into red_list[]: the n_red blocks, most contributions first
    int32_t cell_begin, n_cells;     // into tile_cells[] / cell_items[]: all cells of the tile
    int32_t item_begin, n_items;     // into items[]: all items of the tile
};

struct RangeDesc {
    int64_t nz0;      // 0-based nzval index of the first owned entry
    int32_t ent0;     // first entity id (0-based)
    int32_t n_ent;    // entities in the run
    int32_t nz_len;   // nzval entries in the run
    int32_t pad;
};

struct SegDesc {
    int32_t sub;         // subdomain index
    int32_t cell_begin;  // into tile_cells[] / cell_items[]
    int32_t n_cells;
    int32_t item_end;    // one past the last item of the segment's last cell
};

// Per owned entity of a tile (in range order):
//   x: staging offset (values): [kcount][NBmax][BS] block contributions (BS = nc*nc rounded up
//      to even), then [kcount][nc] f
//   y: map offset (bytes): [nnb][kcount], the row function i of each contribution or 0xFF
//   z: first reduce lane of the entity
//   w: kcount | nnb << 8  (cells of the entity, row entities of its columns)
struct alignas(16) EntMeta {
    int32_t x, y, z, w;
};

// per-subdomain device data
struct SubDev {
    int32_t kind, nb, ng, nq, dim, nc;
    int64_t n_cells;
    const int32_t* cellid;   // [n] 0-based Ferrite cell id
    const int32_t* conn;     // [n][ng] 0-based node ids
    const int32_t* ents;     // [n][nb] entity ids
    const uint8_t* rank8;    // [n][nb i][RS8] rank of entity i in the columns of entity j (byte j), or NULL;
                             // rows padded to RS8 = 8 * ceil(nb / 8) bytes
    const uint16_t* rank16;  // same with 16-bit ranks (some rank exceeds 254); rows of RS16 = 4 * ceil(nb / 4)
    // reference tables (float and double copies), row-major as in the C ABI
    const float* w_f;        // [nq]
    const float* N_f;        // [nq][nb]
    const float* dN_f;       // [nq][nb][dim]
    const float* dM_f;       // [nq][ng][dim]
    const double* w_d;
    const double* N_d;
    const double* dN_d;
    const double* dM_d;
};

// device status word of one assembly
struct DevStatus {
    unsigned long long detj_key;  // (cell id << 32) | bits(float detJ); min over failing cells
    unsigned long long miss_key;  // (cell id << 32) | (I << 16) | J; min over pattern misses
    unsigned int flagged;         // cells recomputed with FP64 Jacobians
    unsigned int timeout;         // tiles that gave up waiting for their table copy
};

struct Physics {
    int32_t kind;            // FE_HEAT / FE_LINEAR_ELASTIC / FE_NEO_HOOKE
    double p0, p1;           // as in fe_assemble_params
    double body[3];
    double lam, mu;          // elastic: Lame parameters from E, nu
    const float* scale_f;    // per Ferrite cell material factor (NULL = 1)
    const double* scale_d;
    const float* u_f;        // neo-hooke solution (float copy)
    const double* u_d;
    float cond_threshold;
};

struct KernelArgs {
    int32_t n_tiles;
    int32_t nc;              // components per entity (dofs per entity)
    int32_t n_sub;
    int32_t nb_max;          // staging stride: max base functions over subdomains
    int32_t bs;              // staging values per block: nc*nc rounded up to even
    SubDev sub[MAX_SUB];
    const TileDesc* tiles;
    const RangeDesc* ranges;
    const SegDesc* segs;
    const EntMeta* emeta;
    const int32_t* eids;             // global entity id of each owned entity
    const int32_t* tile_cells;       // subdomain-local cell index
    const int32_t* cell_items;       // first item of each tile cell
    const uint32_t* items;
    const uint32_t* red_list;        // per tile: owned blocks (entity << 22 | row entity), sorted
    const int64_t* colptr;   // device copy, 1-based
    const float* xh[3];      // node coordinates split into float hi + lo
    const float* xl[3];
    const double* xd;        // node coordinates [n_nodes][dim], FP64
    int32_t dim;
    double* nzval;
    double* f;
    int32_t do_k, do_f, fillzero;
    Physics phys;
    DevStatus* status;
    int32_t stage_cap;       // staging values the plan guarantees per tile
    int32_t map_cap;         // map bytes per tile
    int32_t ent_cap;         // owned entities per tile, max
    int32_t red_cap;         // reduce lanes (owned blocks) per tile, max
    int32_t cells_cap;       // cells per tile, max
    int32_t items_cap;       // items per tile, max
    int32_t ng_max;          // geometric nodes per cell, max over subdomains
    int32_t chunk_bytes;     // bytes of the per-group cell table buffers of the launched kernel
    int32_t groups[MAX_SUB]; // lane groups (cells in flight) per CTA, per subdomain
};

}  // namespace fe
