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

constexpr int CTA_THREADS = 256;  // threads of a tile CTA
// lanes per cell ("lane group") of each kind; CTA_THREADS / GROUP_LANES[kind] groups per CTA
constexpr int GROUP_LANES[NKIND] = {4, 4, 4, 8, 8, 32, 16};
constexpr int MAX_NB = 27;   // base functions per cell
constexpr int MAX_NG = 8;    // geometric nodes per cell
constexpr int MAX_NQ = 27;   // quadrature points per cell
constexpr int MAX_SUB = 3;   // subdomains one kernel handles

// ---------------------------------------------------------------------------------------
// Tile record: everything the kernel needs to assemble one tile, in one contiguous block
// of global memory that a CTA copies to shared memory with a single TMA bulk copy. All
// section offsets are bytes from the record start, multiples of 16; the record size is a
// multiple of 16. Sections:
//   RecHead                                   96 bytes
//   RecSeg[n_seg]                             the tile's cells, one segment per subdomain
//   RecEnt[n_ent]       (off_ent)             owned entities: column base and length, offset of
//                                             the entity's columns in its pass's output buffer
//   int32 eid[n_ent]    (off_eid)             entity ids (f rows id*nc .. id*nc+nc-1)
//   uint32 fk[n_ent]    (off_fk)              f staging: first f slot | cell count << 16
//   uint32 red[n_red]   (off_red)             owned (entity, row entity) blocks: ent << 22 | rank;
//                                             pass after pass, within a pass most contributions first
//   RecRun runs[n_runs] (off_runs)            the blocks as runs of equal contribution count:
//                                             contribution k of block first + j of a run is in
//                                             slot base + k * nblk + j (cell order in k)
//   RecPass pass[n_pass] (off_pass)           reduce passes: blocks, runs and output ranges whose
//                                             values fit the shared output buffer at once
//   RecRng rng[n_rng]   (off_rng)             contiguous nzval ranges of a pass's output buffer
//   uint32 items[n_items] (off_items)         per (cell, owned base function j): j | f slot << 16
//   int32 cells[n_cells] (off_cells)          sub-local cell index of each tile cell
//   RecTask[n_tasks]    (off_tasks)           (cell, item range) pieces of work for a lane group:
//                                             geometry of the cell, then the blocks of the items
//   uint16 gt[..]       (RecSeg::gt_off)      per segment: tasks gt[g] .. gt[g+1]-1 belong to
//                                             planned lane group g (n_grp groups); a CTA with
//                                             fewer groups runs planned groups g, g + groups, ...
//   uint16 conn[..]     (RecSeg::conn_off)    per segment: [cells][NG] tile-local node index
//   uint16 slots[..]    (RecSeg::slot_off)    per segment: [items][NB] staging slot of row i,
//                                             SLOT_MISS where the pattern has no entry
//   int32 nodes[n_nodes] (off_nodes)          global node ids (coordinates are gathered)
// Staging (shared memory, Real values): slot s holds one nc x nc block at s * BS
// (BS = nc*nc rounded up to even, column-major); f slot q holds nc values at
// n_slots * BS + q * nc.
// ---------------------------------------------------------------------------------------
constexpr uint16_t SLOT_MISS = 0xFFFF;
constexpr int RED_RANK_BITS = 22;
constexpr int MAX_TILE_ENTS = 1 << (32 - RED_RANK_BITS);
constexpr int MAX_ENT_CELLS = 255;   // cells of one dof entity
constexpr int MAX_TILE_SLOTS = 0xFFFF;

struct RecHead {
    int32_t bytes;
    int32_t n_seg, n_ent, n_cells;
    int32_t n_items, n_red, n_nodes, n_slots;
    int32_t n_fslots, n_runs, n_pass, n_rng;
    int32_t off_ent, off_eid, off_fk, off_red;
    int32_t off_runs, off_pass, off_rng, off_items;
    int32_t off_cells, off_nodes, n_tasks, off_tasks;
};
static_assert(sizeof(RecHead) == 96, "record head is 96 bytes");

struct RecSeg {
    int32_t sub;
    int32_t cell_begin, cell_end;  // tile cells of the segment
    int32_t item_begin, item_end;  // tile items of the segment
    int32_t conn_off, slot_off;    // byte offsets of the segment's conn and slot rows
    int32_t gt_off;                // byte offset of the segment's group task table
    int32_t n_grp;                 // planned lane groups
    int32_t pad[3];
};
static_assert(sizeof(RecSeg) == 48, "segment entry is 48 bytes");

struct RecTask {
    uint16_t cell;                  // tile cell index
    uint16_t item_begin, item_end;  // tile items
    uint16_t pad;
};
static_assert(sizeof(RecTask) == 8, "task entry is 8 bytes");

struct RecEnt {
    int64_t colbase;  // 0-based nzval index of the entity's first column
    int32_t L;        // column length (entries)
    int32_t out_off;  // offset of the entity's nc columns in its pass's output buffer (doubles)
};
static_assert(sizeof(RecEnt) == 16, "entity entry is 16 bytes");

struct RecRun {
    int32_t first;  // first block (position in red[]) of the run
    int32_t count;  // contributions (slots) of each block of the run
    int32_t base;   // first slot of the run
    int32_t nblk;   // blocks in the run
};
static_assert(sizeof(RecRun) == 16, "run entry is 16 bytes");

struct RecPass {
    int32_t red_begin, red_end;  // blocks of the pass (positions in red[])
    int32_t run_begin, run_end;  // their runs
    int32_t rng_begin, rng_end;  // output ranges
    int32_t out_len;             // output buffer doubles used
    int32_t pad;
};
static_assert(sizeof(RecPass) == 32, "pass entry is 32 bytes");

struct RecRng {
    int64_t nz0;      // first nzval index (0-based)
    int32_t buf_off;  // its position in the output buffer; buf_off - nz0 is even
    int32_t len;      // doubles
};
static_assert(sizeof(RecRng) == 16, "range entry is 16 bytes");

// per-subdomain device data
struct SubDev {
    int32_t kind, nb, ng, nq, dim, nc;
    int64_t n_cells;
    const int32_t* cellid;   // [n] 0-based Ferrite cell id
    const int32_t* ents;     // [n][nb] entity ids
    const int32_t* conn;     // [n][ng] 0-based node ids (adjoint kernel)
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
    // the same constants in FP32 (set by the host: the kernels convert nothing per cell)
    float p0_f, p1_f, lam_f, mu_f, body_f[3];
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
    int32_t bs;              // staging values per block: nc*nc rounded up to even
    SubDev sub[MAX_SUB];
    const char* rec;         // tile records (16-byte aligned)
    const int64_t* rec_off;  // [n_tiles + 1] byte offset of each record
    const float* xf6;        // [n_nodes][6]: x, y, z as float hi, then the float lo parts
    const double* xd3;       // [n_nodes][3]: x, y, z in FP64 (z = 0 in 2D)
    const double* xd;        // [n_nodes][dim] FP64 (Jacobians recomputed in FP64)
    int32_t dim;
    double* nzval;
    double* f;
    int32_t do_k, do_f, fillzero;
    int32_t compensated;     // mixed precision: compensated FP32 pair sums
    int32_t host_out;        // nzval is page-locked host memory (its mapping): plain stores only
    int32_t tensor;          // element matrices on the tensor cores where a kernel exists
    Physics phys;
    DevStatus* status;
    int32_t rec_cap;         // record bytes per ring buffer (max over tiles)
    int32_t out_cap;         // output-buffer doubles of one reduce pass (max over tiles)
    int32_t node_cap;        // nodes per tile, max
    int32_t stage_cap;       // staging values per tile, max
    int32_t chunk_bytes;     // bytes of the per-group cell table buffers of the launched kernel
    int32_t groups[MAX_SUB]; // lane groups (cells in flight) per CTA, per subdomain
    // two-phase form: per-cell element matrices of each subdomain (nullptr: computed in the
    // tiles), [cell][j][t][i] (column stride ea_col_values) then fe [x][i], ea_stride values
    // per cell (ea_cell_values)
    const void* ea[MAX_SUB];
    int64_t ea_stride[MAX_SUB];
};

// where element_kernel writes: the two-phase scratch (ke = base, ks[0] = values per cell) or
// the caller's arrays, Ke(cell, I, J) at ke[cell ks[0] + I ks[1] + J ks[2]] and fe(cell, I) at
// fe[cell fs[0] + I fs[1]] (cell = Ferrite cell id - 1, I = nc * base function + component)
struct EaOut {
    void* ke;
    void* fe;
    int64_t ks[3];
    int64_t fs[2];
};

// values of one column j (nb rows of nc*nc entries) of a cell's element matrix in the
// two-phase scratch, rounded up to 16 bytes of FP32 so that every column is one aligned copy
__host__ __device__ constexpr int ea_col_values(int nb, int nc) { return (nb * nc * nc + 3) / 4 * 4; }
// values per cell: nb columns, then nb*nc load entries, rounded up to 16 bytes of FP32
__host__ __device__ constexpr int64_t ea_cell_values(int nb, int nc) {
    return ((int64_t)nb * ea_col_values(nb, nc) + (int64_t)nb * nc + 3) / 4 * 4;
}

}  // namespace fe
