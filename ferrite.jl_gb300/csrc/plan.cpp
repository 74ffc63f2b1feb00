// plan.cpp -- host-side set-up: validation of Ferrite's arrays, the compact element-to-nzval
// index map ("ranks"), and the owner-tile plan.
//
// Index map. For a single field with n_components (nc) interleaved dofs per entity
// (Ferrite's VectorizedInterpolation layout, src/interpolations.jl:1769-1825, dofs created in
// groups of n_copies, src/Dofs/DofHandler.jl:715-794), every entity n owns the nc adjacent
// columns nc*n .. nc*n+nc-1 of K, all with the same row list, and that row list is made of
// whole entities (allocate_matrix couples all components, sparsity_pattern.jl:223-253).
// So the nzval position of Ke[(i,a),(j,b)] is
//     colptr[nc*n] - 1 + b*L_n + nc*rank_n(m) + a,   n = ent(j), m = ent(i),
// with L_n the column length and rank_n(m) the position of entity m among the row entities
// of n. The plan stores one small rank per (cell, j, i): 64 bytes per Q1 hexahedron instead
// of a 576-entry int32 map.
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>
#include <type_traits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace fe {

int kind_of(int32_t ct, int32_t order, int32_t& nb, int32_t& ng, int32_t& rdim) {
    rdim = (ct == FE_TRIANGLE || ct == FE_QUADRILATERAL) ? 2 : 3;
    if (order == 1) {
        switch (ct) {
            case FE_TRIANGLE: nb = ng = 3; return KIND_TRI3;
            case FE_QUADRILATERAL: nb = ng = 4; return KIND_QUAD4;
            case FE_TETRAHEDRON: nb = ng = 4; return KIND_TET4;
            case FE_HEXAHEDRON: nb = ng = 8; return KIND_HEX8;
            case FE_WEDGE: nb = ng = 6; return KIND_WEDGE6;
            default: return -1;
        }
    }
    if (order == 2 && ct == FE_HEXAHEDRON) { nb = 27; ng = 8; return KIND_HEX27; }
    if (order == 2 && ct == FE_QUADRILATERAL) { nb = 9; ng = 4; return KIND_QUAD9; }
    return -1;
}

static int fail(Error& err, int code, const std::string& msg) {
    err.code = code;
    err.msg = msg;
    return code;
}

int build_problem(const CreateInput& in, HostProblem& hp, Error& err) {
    const fe_grid_desc* g = in.grid;
    if (!g || !in.subs || !in.dofs || !in.pattern) return fail(err, FE_ERR_ARG, "null descriptor");
    if (g->dim != 2 && g->dim != 3) return fail(err, FE_ERR_ARG, "grid dim must be 2 or 3");
    if (g->n_nodes <= 0 || !g->nodes) return fail(err, FE_ERR_ARG, "grid has no nodes");
    if (g->n_nodes >= (int64_t)INT32_MAX) return fail(err, FE_ERR_UNSUPPORTED, "more than 2^31 nodes");
    if (in.n_sub < 1 || in.n_sub > MAX_SUB) return fail(err, FE_ERR_UNSUPPORTED, "1 to 3 subdomains supported");
    hp.dim = g->dim;
    hp.n_nodes = g->n_nodes;
    hp.n_cells = g->n_cells;
    hp.nodes.assign(g->nodes, g->nodes + g->n_nodes * g->dim);
    const fe_dof_desc* d = in.dofs;
    const fe_csc_desc* P = in.pattern;
    if (!d->cell_dofs || !d->cell_dofs_offset || d->ndofs <= 0) return fail(err, FE_ERR_ARG, "empty DofHandler");
    if (P->n != d->ndofs) return fail(err, FE_ERR_ARG, "K is not ndofs x ndofs");
    if (!P->colptr || (!P->rowval && !in.device_pattern)) return fail(err, FE_ERR_ARG, "null colptr/rowval");
    hp.ndofs = d->ndofs;
    hp.nnz = P->nnz;
    if (P->colptr[0] != 1 || P->colptr[P->n] - 1 != P->nnz) return fail(err, FE_ERR_ARG, "colptr inconsistent with nnz");
    hp.colptr.assign(P->colptr, P->colptr + P->n + 1);
    for (int64_t c = 0; c < P->n; ++c)
        if (hp.colptr[c + 1] < hp.colptr[c]) return fail(err, FE_ERR_ARG, "colptr not monotone");

    hp.cell_sub.assign(hp.n_cells, -1);
    hp.cell_local.assign(hp.n_cells, -1);
    hp.cell_dofs_off.assign(d->cell_dofs_offset, d->cell_dofs_offset + hp.n_cells);
    int64_t maxdof_end = 0;
    hp.subs.resize(in.n_sub);
    hp.nc = 0;
    for (int s = 0; s < in.n_sub; ++s) {
        const fe_subdomain_desc& sd = in.subs[s];
        HostSub& hs = hp.subs[s];
        int32_t nb, ng, rdim;
        const int kind = kind_of(sd.cell_type, sd.ip_order, nb, ng, rdim);
        if (kind < 0) return fail(err, FE_ERR_UNSUPPORTED, "unsupported cell type / interpolation order");
        if (rdim != hp.dim) return fail(err, FE_ERR_UNSUPPORTED, "embedded elements (rdim != sdim) not supported");
        if (sd.n_components != 1 && sd.n_components != hp.dim)
            return fail(err, FE_ERR_UNSUPPORTED, "n_components must be 1 or dim");
        if (hp.nc && hp.nc != sd.n_components) return fail(err, FE_ERR_UNSUPPORTED, "one field: n_components must agree");
        hp.nc = sd.n_components;
        if (sd.n_qp < 1 || sd.n_qp > MAX_NQ) return fail(err, FE_ERR_UNSUPPORTED, "1..27 quadrature points supported");
        if (!sd.qr_weights || !sd.N || !sd.dNdxi || !sd.dMdxi) return fail(err, FE_ERR_ARG, "null reference table");
        if (sd.n_cells < 1 || !sd.cellset || !sd.cell_nodes) return fail(err, FE_ERR_ARG, "empty cellset");
        hs.cell_type = sd.cell_type;
        hs.ip_order = sd.ip_order;
        hs.kind = kind;
        hs.nb = nb; hs.ng = ng; hs.nq = sd.n_qp; hs.dim = rdim; hs.nc = sd.n_components;
        hs.n_cells = sd.n_cells;
        for (int q = 0; q < sd.n_qp; ++q)
            if (!(sd.qr_weights[q] > 0.0))
                return fail(err, FE_ERR_UNSUPPORTED, "quadrature rules with non-positive weights are not supported");
        hs.w.assign(sd.qr_weights, sd.qr_weights + sd.n_qp);
        hs.N.assign(sd.N, sd.N + sd.n_qp * nb);
        hs.dN.assign(sd.dNdxi, sd.dNdxi + sd.n_qp * nb * rdim);
        hs.dM.assign(sd.dMdxi, sd.dMdxi + sd.n_qp * ng * rdim);
        hs.cellid.resize(sd.n_cells);
        hs.conn.resize(sd.n_cells * ng);
        hs.ents.resize(sd.n_cells * nb);
        const int nc = hs.nc;
        for (int64_t k = 0; k < sd.n_cells; ++k) {
            const int64_t c = sd.cellset[k] - 1;
            if (c < 0 || c >= hp.n_cells) { err.cell = c + 1; return fail(err, FE_ERR_BOUNDS, "cellset entry out of range"); }
            if (hp.cell_sub[c] >= 0) { err.cell = c + 1; return fail(err, FE_ERR_ARG, "cell in two subdomains"); }
            hp.cell_sub[c] = s;
            hp.cell_local[c] = (int32_t)k;
            hs.cellid[k] = (int32_t)c;
            for (int a = 0; a < ng; ++a) {
                const int64_t v = sd.cell_nodes[k * ng + a];
                if (v < 1 || v > hp.n_nodes) { err.cell = c + 1; return fail(err, FE_ERR_BOUNDS, "node id out of range"); }
                hs.conn[k * ng + a] = (int32_t)(v - 1);
            }
            const int64_t off = d->cell_dofs_offset[c];
            if (off < 1) { err.cell = c + 1; return fail(err, FE_ERR_BOUNDS, "cell_dofs_offset out of range"); }
            maxdof_end = std::max(maxdof_end, off - 1 + (int64_t)nb * nc);
        }
    }
    // The cell_dofs array length is not passed; its extent is implied by the offsets.
    hp.cell_dofs.resize(maxdof_end);
    {
        const int64_t chunk = 1 << 20;
#pragma omp parallel for schedule(static)
        for (int64_t b = 0; b < (maxdof_end + chunk - 1) / chunk; ++b)
            std::memcpy(hp.cell_dofs.data() + b * chunk, d->cell_dofs + b * chunk,
                        (size_t)(std::min(chunk, maxdof_end - b * chunk)) * sizeof(int64_t));
    }
    const int nc = hp.nc;
    if (hp.ndofs % nc) return fail(err, FE_ERR_UNSUPPORTED, "ndofs not a multiple of n_components");
    hp.n_ent = hp.ndofs / nc;
    if (hp.n_ent >= (int64_t)INT32_MAX) return fail(err, FE_ERR_UNSUPPORTED, "too many dof entities");
    // dof layout: per base function nc consecutive dofs starting at a multiple of nc
    for (int s = 0; s < in.n_sub; ++s) {
        HostSub& hs = hp.subs[s];
        for (int64_t k = 0; k < hs.n_cells; ++k) {
            const int64_t c = hs.cellid[k];
            const int64_t* cd = hp.cell_dofs.data() + hp.cell_dofs_off[c] - 1;
            for (int i = 0; i < hs.nb; ++i) {
                const int64_t d0 = cd[i * nc];
                if (d0 < 1 || d0 > hp.ndofs) { err.cell = c + 1; return fail(err, FE_ERR_BOUNDS, "dof out of range"); }
                if ((d0 - 1) % nc) { err.cell = c + 1; return fail(err, FE_ERR_UNSUPPORTED, "dofs of an entity are not nc-aligned"); }
                for (int a = 1; a < nc; ++a)
                    if (cd[i * nc + a] != d0 + a) { err.cell = c + 1; return fail(err, FE_ERR_UNSUPPORTED, "components of an entity are not consecutive dofs"); }
                hs.ents[k * hs.nb + i] = (int32_t)((d0 - 1) / nc);
            }
        }
    }
    // a device-resident pattern is checked and ranked on the device (device_index_map)
    if (in.device_pattern) return FE_OK;
    // pattern: entity-blocked columns (checked once, O(nnz))
    const int64_t* rv = P->rowval;
    const int64_t* cp = hp.colptr.data();
    int bad = 0;
    int64_t bad_col = 0;
#pragma omp parallel for schedule(dynamic, 2048) reduction(| : bad)
    for (int64_t n = 0; n < hp.n_ent; ++n) {
        const int64_t c0 = cp[nc * n] - 1, L = cp[nc * n + 1] - cp[nc * n];
        int b_ = 0;
        if (L % nc) b_ = 1;
        for (int b = 1; b < nc && !b_; ++b) {
            const int64_t cb = cp[nc * n + b] - 1;
            if (cp[nc * n + b + 1] - cp[nc * n + b] != L) { b_ = 1; break; }
            for (int64_t k = 0; k < L; ++k)
                if (rv[cb + k] != rv[c0 + k]) { b_ = 1; break; }
        }
        for (int64_t k = 0; k < L && !b_; k += nc) {
            const int64_t r0 = rv[c0 + k];
            if (r0 < 1 || r0 > hp.ndofs || (r0 - 1) % nc) { b_ = 1; break; }
            if (k && rv[c0 + k - nc] >= r0) { b_ = 1; break; }
            for (int a = 1; a < nc; ++a)
                if (rv[c0 + k + a] != r0 + a) { b_ = 1; break; }
        }
        if (b_) {
            bad |= 1;
#pragma omp critical
            bad_col = n * nc + 1;
        }
    }
    if (bad) {
        err.col = bad_col;
        return fail(err, FE_ERR_UNSUPPORTED, "sparsity pattern is not blocked by dof entity (all components coupled)");
    }
    // ranks (the index map): rank of row entity e[i] in column entity e[j]'s row list, by one
    // merge walk per (cell, j) over the column's ascending row entities against the cell's
    // entities in ascending order; 8-bit ranks unless some rank exceeds 254
    for (int s = 0; s < in.n_sub; ++s) {
        HostSub& hs = hp.subs[s];
        const int nb = hs.nb;
        auto fill_ranks = [&](auto* out, const int64_t miss, const int64_t limit) -> bool {
            int over = 0;
#pragma omp parallel for schedule(static) reduction(| : over)
            for (int64_t k = 0; k < hs.n_cells; ++k) {
                const int32_t* e = &hs.ents[k * nb];
                int32_t srt[MAX_NB];  // local indices by entity (ties by index)
                for (int i = 0; i < nb; ++i) srt[i] = i;
                std::sort(srt, srt + nb, [&](int32_t a, int32_t b) { return e[a] < e[b] || (e[a] == e[b] && a < b); });
                for (int j = 0; j < nb; ++j) {
                    const int64_t n = e[j];
                    const int64_t c0 = cp[nc * n] - 1;
                    const int64_t Le = (cp[nc * n + 1] - cp[nc * n]) / nc;
                    int64_t m = 0;
                    for (int q = 0; q < nb; ++q) {
                        const int i = srt[q];
                        const int64_t want = (int64_t)e[i] * nc + 1;
                        while (m < Le && rv[c0 + nc * m] < want) ++m;
                        int64_t r = miss;
                        if (m < Le && rv[c0 + nc * m] == want && m < 0xFFFF) r = m;
                        if (r != miss && r >= limit) over = 1;
                        out[((size_t)k * nb + j) * nb + i] = (typename std::remove_pointer<decltype(out)>::type)(r >= limit ? miss : r);
                    }
                }
            }
            return over == 0;
        };
        hs.rank8.resize((size_t)hs.n_cells * nb * nb);
        if (fill_ranks(hs.rank8.data(), 255, 255)) {
            hs.wide_rank = false;
        } else {
            decltype(hs.rank8)().swap(hs.rank8);
            hs.rank16.resize((size_t)hs.n_cells * nb * nb);
            fill_ranks(hs.rank16.data(), 0xFFFF, 0xFFFF);
            hs.wide_rank = true;
        }
    }
    return FE_OK;
}

// ---------------------------------------------------------------------------------------
// Owner tiles
//
// Entities are bucketed by position into compact tiles. A tile lists every cell touching one
// of its entities; for every (cell, owned base function j) an item, and for every row i of
// an item the staging slot its nc x nc block goes to. The slots of one owned block
// (entity n, row entity r) are consecutive and ordered by cell (k = position of the cell
// among the cells of n), so the reduce step sums each entry in the reference's cell order.
// The tile's data is emitted as one record (layout in common.h).
// ---------------------------------------------------------------------------------------
namespace {

inline int32_t pad16(int64_t b) { return (int32_t)((b + 15) & ~15ll); }

// relative cost of a lane group's work: the geometry of a cell against the blocks of one item
// (measured on Q1 hexahedra: about 2.6 items per cell geometry)
constexpr int64_t TASK_GEO_COST = 26, TASK_ITEM_COST = 10;

struct TileItem {
    int32_t cell;  // tile cell index (before the per-segment reorder)
    int32_t j, te, k;
};
struct TileSeg { int32_t sub, cell_begin, cell_end, item_begin, item_end; };
struct TileTask { int32_t cell, i0, i1, cost; };

// Working arrays of build_record, one set per thread and reused from tile to tile: the planner
// builds ~10^5 records in parallel, and allocating them per tile costs more than filling them.
struct RecScratch {
    std::vector<TileSeg> segs;
    std::vector<int32_t> cells, cell_item0, kc, z, cnt, item_nb, row_block, row_ord, ord, base, stride, fbase, nodes, pieces,
        bucket;
    std::vector<int64_t> item_row0, load;
    std::vector<TileItem> items;
    std::vector<RecEnt> rent;
    std::vector<RecPass> passes;
    std::vector<RecRng> rngs;
    std::vector<RecRun> runs;
    std::vector<uint32_t> red, red_sorted;
    std::vector<RecSeg> rsegs;
    std::vector<TileTask> tasks;
    std::vector<std::vector<std::vector<TileTask>>> seg_tasks;
};

// Build the record of one tile. ents: owned global entity ids; trip: the tile's (sub, cell,
// j) triples in (sub, cell, j) order. Returns 0 or an error code (internal inconsistency).
int build_record(const HostProblem& hp, const std::vector<int32_t>& kcount, const std::vector<int32_t>& tile_local,
                 const int32_t* ents, int32_t n_ent, const uint64_t* trip, int64_t n_trip, std::vector<uint8_t>& out,
                 int32_t& n_nodes_out, int32_t& stage_out, int32_t& n_cells_out, int32_t& n_items_out, int32_t& out_len_out,
                 int32_t out_cap) {
    const int nc = hp.nc;
    const int bs = (nc * nc + 1) & ~1;
    const int64_t* cp = hp.colptr.data();
    thread_local RecScratch S;
    // segments, cells, items (cell order)
    auto& segs = S.segs;
    auto& cells = S.cells;            // sub-local cell index
    auto& cell_item0 = S.cell_item0;  // first item of each cell
    auto& items = S.items;
    auto& kc = S.kc;
    segs.clear();
    cells.clear();
    cell_item0.clear();
    items.clear();
    kc.assign(n_ent, 0);
    for (int64_t q = 0; q < n_trip; ++q) {
        const int s = (int)(trip[q] >> 40);
        const int32_t cell = (int32_t)((trip[q] >> 8) & 0xFFFFFFFFull);
        const int j = (int)(trip[q] & 0xFF);
        const bool new_cell = q == 0 || (trip[q] >> 8) != (trip[q - 1] >> 8);
        if (new_cell) {
            if (segs.empty() || segs.back().sub != s) {
                if (!segs.empty()) { segs.back().cell_end = (int32_t)cells.size(); segs.back().item_end = (int32_t)items.size(); }
                segs.push_back(TileSeg{s, (int32_t)cells.size(), 0, (int32_t)items.size(), 0});
            }
            cells.push_back(cell);
            cell_item0.push_back((int32_t)items.size());
        }
        const HostSub& hs = hp.subs[s];
        const int32_t te = tile_local[hs.ents[(int64_t)cell * hs.nb + j]];
        items.push_back(TileItem{(int32_t)cells.size() - 1, j, te, kc[te]++});
    }
    if (!segs.empty()) { segs.back().cell_end = (int32_t)cells.size(); segs.back().item_end = (int32_t)items.size(); }
    for (int32_t te = 0; te < n_ent; ++te)
        if (kc[te] != kcount[ents[te]]) return 1;
    // owned blocks: z[te] + r
    auto& z = S.z;
    z.assign(n_ent + 1, 0);
    for (int32_t te = 0; te < n_ent; ++te) {
        const int64_t n = ents[te];
        z[te + 1] = z[te] + (int32_t)((cp[nc * n + 1] - cp[nc * n]) / nc);
    }
    const int32_t n_red = z[n_ent];
    auto& cnt = S.cnt;
    cnt.assign(n_red, 0);
    // per (item, i): block index or -1
    auto cell_sub = [&](int32_t c) {
        int s = 0;
        while (s + 1 < (int)segs.size() && c >= segs[s].cell_end) ++s;
        return s;
    };
    auto& item_nb = S.item_nb;
    auto& item_row0 = S.item_row0;
    item_nb.resize(items.size());
    item_row0.assign(items.size() + 1, 0);
    {
        int sg = 0;
        for (size_t it = 0; it < items.size(); ++it) {
            while (sg + 1 < (int)segs.size() && (int32_t)it >= segs[sg].item_end) ++sg;
            item_nb[it] = hp.subs[segs[sg].sub].nb;
            item_row0[it + 1] = item_row0[it] + item_nb[it];
        }
    }
    auto& row_block = S.row_block;
    auto& row_ord = S.row_ord;  // position among the block's contributions
    row_block.resize(item_row0.back());
    row_ord.resize(item_row0.back());
    for (size_t it = 0; it < items.size(); ++it) {
        const TileItem& I = items[it];
        const int sg = cell_sub(I.cell);
        const HostSub& hs = hp.subs[segs[sg].sub];
        const int32_t cell = cells[I.cell];
        for (int i = 0; i < hs.nb; ++i) {
            const int r = rank_of(hs, cell, I.j, i);
            int32_t b = -1;
            if (r >= 0) {
                b = z[I.te] + r;
                row_ord[item_row0[it] + i] = cnt[b]++;
            }
            row_block[item_row0[it] + i] = b;
        }
    }
    for (int32_t b = 0; b < n_red; ++b)
        if (cnt[b] > MAX_ENT_CELLS) return 2;
    // reduce passes: consecutive owned entities whose columns fit the output buffer; within a
    // pass, contiguous nzval ranges, each placed in the buffer with the parity of its start so
    // the 16-byte aligned middle can be stored with one bulk copy
    auto& rent = S.rent;
    auto& passes = S.passes;
    auto& rngs = S.rngs;
    rent.assign(n_ent, RecEnt{});
    passes.clear();
    rngs.clear();
    {
        int32_t e = 0;
        while (e < n_ent) {
            RecPass P{};
            P.rng_begin = (int32_t)rngs.size();
            int32_t used = 0, e1 = e;
            while (e1 < n_ent) {
                const int64_t n = ents[e1];
                const int64_t cb = cp[nc * n] - 1, len = cp[nc * n + nc] - cp[nc * n];
                const bool joins = (int32_t)rngs.size() > P.rng_begin && rngs.back().nz0 + rngs.back().len == cb;
                int32_t start = joins ? rngs.back().buf_off + rngs.back().len : used;
                if (!joins && ((start - cb) & 1)) ++start;
                if (start + len > out_cap) {
                    if (e1 == e) return 4;  // one entity's columns exceed the buffer
                    break;
                }
                if (joins) {
                    rngs.back().len += (int32_t)len;
                } else {
                    rngs.push_back(RecRng{cb, start, (int32_t)len});
                }
                rent[e1] = RecEnt{cb, (int32_t)(cp[nc * n + 1] - cp[nc * n]), start};
                used = (int32_t)(start + len);
                ++e1;
            }
            P.rng_end = (int32_t)rngs.size();
            P.out_len = used;
            P.red_begin = z[e];   // filled with positions below; z ranges of the pass's entities
            P.red_end = z[e1];
            passes.push_back(P);
            e = e1;
        }
    }
    // reduce order within each pass: most contributions first (stable in (entity, rank)); the
    // slots of a run are k-major so the lanes of a warp read consecutive slots
    auto& ord = S.ord;
    auto& bucket = S.bucket;
    ord.resize(n_red);
    for (const RecPass& P : passes) {
        // a stable counting sort by contribution count (at most MAX_ENT_CELLS), most first
        bucket.assign(MAX_ENT_CELLS + 2, 0);
        for (int32_t b = P.red_begin; b < P.red_end; ++b) ++bucket[MAX_ENT_CELLS - cnt[b] + 1];
        for (int v = 1; v <= MAX_ENT_CELLS + 1; ++v) bucket[v] += bucket[v - 1];
        for (int32_t b = P.red_begin; b < P.red_end; ++b) ord[P.red_begin + bucket[MAX_ENT_CELLS - cnt[b]]++] = b;
    }
    auto& base = S.base;
    auto& stride = S.stride;
    auto& runs = S.runs;
    base.resize(n_red);
    stride.resize(n_red);
    runs.clear();
    int32_t n_slots = 0;
    for (RecPass& P : passes) {
        P.run_begin = (int32_t)runs.size();
        int32_t q = P.red_begin;
        while (q < P.red_end) {
            int32_t q1 = q;
            while (q1 < P.red_end && cnt[ord[q1]] == cnt[ord[q]]) ++q1;
            RecRun U{q, cnt[ord[q]], n_slots, q1 - q};
            for (int32_t x = q; x < q1; ++x) {
                base[ord[x]] = n_slots + (x - q);
                stride[ord[x]] = U.nblk;
            }
            n_slots += U.count * U.nblk;
            if (n_slots > MAX_TILE_SLOTS - 1) return 3;
            runs.push_back(U);
            q = q1;
        }
        P.run_end = (int32_t)runs.size();
    }
    const int32_t n_runs = (int32_t)runs.size(), n_pass = (int32_t)passes.size(), n_rng = (int32_t)rngs.size();
    auto& red = S.red;
    auto& red_sorted = S.red_sorted;
    red.resize(n_red);
    red_sorted.resize(n_red);
    for (int32_t te = 0; te < n_ent; ++te)
        for (int32_t r = 0; r < z[te + 1] - z[te]; ++r) red[z[te] + r] = ((uint32_t)te << RED_RANK_BITS) | (uint32_t)r;
    for (int32_t q = 0; q < n_red; ++q) red_sorted[q] = red[ord[q]];
    // f slots: per owned entity, one per cell in k order
    auto& fbase = S.fbase;
    fbase.assign(n_ent + 1, 0);
    for (int32_t te = 0; te < n_ent; ++te) fbase[te + 1] = fbase[te] + kc[te];
    const int32_t n_fslots = fbase[n_ent];
    if (n_fslots > 0xFFFF) return 3;
    // work of the lane groups: per segment, (cell, item range) tasks scheduled longest first
    // onto the least loaded of the planned groups; a cell whose geometry plus blocks would
    // exceed the even share is split into pieces that each redo the geometry
    auto& seg_tasks = S.seg_tasks;  // entries past segs.size() are stale
    if (seg_tasks.size() < segs.size()) seg_tasks.resize(segs.size());
    for (size_t g = 0; g < segs.size(); ++g) {
        const HostSub& hs = hp.subs[segs[g].sub];
        const int G = CTA_THREADS / GROUP_LANES[hs.kind];
        const int32_t c0 = segs[g].cell_begin, c1 = segs[g].cell_end;
        auto n_items_of = [&](int32_t c) {
            return (c + 1 < (int32_t)cells.size() ? cell_item0[c + 1] : (int32_t)items.size()) - cell_item0[c];
        };
        auto& pieces = S.pieces;
        pieces.assign(c1 - c0, 1);
        for (int pass = 0; pass < 3; ++pass) {
            int64_t total = 0;
            for (int32_t c = c0; c < c1; ++c)
                total += (int64_t)pieces[c - c0] * TASK_GEO_COST + (int64_t)n_items_of(c) * TASK_ITEM_COST;
            const int64_t share = std::max<int64_t>((total + G - 1) / G, TASK_GEO_COST + TASK_ITEM_COST);
            for (int32_t c = c0; c < c1; ++c) {
                const int32_t n = n_items_of(c);
                int32_t m = 1;
                while (m < n && TASK_GEO_COST + (int64_t)((n + m - 1) / m) * TASK_ITEM_COST > share) ++m;
                pieces[c - c0] = m;
            }
        }
        auto& tasks = S.tasks;
        tasks.clear();
        for (int32_t c = c0; c < c1; ++c) {
            const int32_t n = n_items_of(c), m = pieces[c - c0];
            int32_t i = cell_item0[c];
            for (int32_t q = 0; q < m; ++q) {
                const int32_t len = n / m + (q < n % m ? 1 : 0);
                tasks.push_back(TileTask{c, i, i + len, (int32_t)(TASK_GEO_COST + len * TASK_ITEM_COST)});
                i += len;
            }
        }
        std::stable_sort(tasks.begin(), tasks.end(), [](const TileTask& x, const TileTask& y) { return x.cost > y.cost; });
        auto& load = S.load;
        load.assign(G, 0);
        seg_tasks[g].resize(G);
        for (auto& gl : seg_tasks[g]) gl.clear();
        for (const TileTask& T : tasks) {
            const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            load[w] += T.cost;
            seg_tasks[g][w].push_back(T);
        }
    }
    // nodes of the tile, ascending
    auto& nodes = S.nodes;
    nodes.clear();
    for (size_t c = 0; c < cells.size(); ++c) {
        const HostSub& hs = hp.subs[segs[cell_sub((int32_t)c)].sub];
        for (int a = 0; a < hs.ng; ++a) nodes.push_back(hs.conn[(int64_t)cells[c] * hs.ng + a]);
    }
    std::sort(nodes.begin(), nodes.end());
    nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
    if (nodes.size() > 0xFFFF) return 3;
    auto local_node = [&](int32_t g) { return (uint16_t)(std::lower_bound(nodes.begin(), nodes.end(), g) - nodes.begin()); };
    // layout
    const int32_t n_seg = (int32_t)segs.size(), n_cells = (int32_t)cells.size(), n_items = (int32_t)items.size();
    RecHead H{};
    H.n_seg = n_seg; H.n_ent = n_ent; H.n_cells = n_cells; H.n_items = n_items;
    H.n_red = n_red; H.n_nodes = (int32_t)nodes.size(); H.n_slots = n_slots; H.n_fslots = n_fslots;
    H.n_runs = n_runs; H.n_pass = n_pass; H.n_rng = n_rng;
    int64_t o = (int64_t)sizeof(RecHead) + (int64_t)n_seg * (int64_t)sizeof(RecSeg);
    H.off_ent = pad16(o); o = H.off_ent + (int64_t)n_ent * 16;
    H.off_eid = pad16(o); o = H.off_eid + (int64_t)n_ent * 4;
    H.off_fk = pad16(o); o = H.off_fk + (int64_t)n_ent * 4;
    H.off_red = pad16(o); o = H.off_red + (int64_t)n_red * 4;
    H.off_runs = pad16(o); o = H.off_runs + (int64_t)n_runs * 16;
    H.off_pass = pad16(o); o = H.off_pass + (int64_t)n_pass * 32;
    H.off_rng = pad16(o); o = H.off_rng + (int64_t)n_rng * 16;
    H.off_items = pad16(o); o = H.off_items + (int64_t)n_items * 4;
    H.off_cells = pad16(o); o = H.off_cells + (int64_t)n_cells * 4;
    auto& rsegs = S.rsegs;
    rsegs.assign(n_seg, RecSeg{});
    for (int32_t g = 0; g < n_seg; ++g) {
        const HostSub& hs = hp.subs[segs[g].sub];
        RecSeg& R = rsegs[g];
        R.sub = segs[g].sub;
        R.cell_begin = segs[g].cell_begin; R.cell_end = segs[g].cell_end;
        R.item_begin = segs[g].item_begin; R.item_end = segs[g].item_end;
        R.conn_off = pad16(o); o = R.conn_off + (int64_t)(R.cell_end - R.cell_begin) * hs.ng * 2;
        R.slot_off = pad16(o); o = R.slot_off + (int64_t)(R.item_end - R.item_begin) * hs.nb * 2;
        R.n_grp = (int32_t)seg_tasks[g].size();
        R.gt_off = pad16(o); o = R.gt_off + (int64_t)(R.n_grp + 1) * 2;
        R.pad[0] = R.pad[1] = R.pad[2] = 0;
    }
    int32_t n_tasks = 0;
    for (int32_t g = 0; g < n_seg; ++g)
        for (const auto& gl : seg_tasks[g]) n_tasks += (int32_t)gl.size();
    if (n_tasks > 0xFFFF) return 3;
    H.n_tasks = n_tasks;
    H.off_tasks = pad16(o); o = H.off_tasks + (int64_t)n_tasks * 8;
    H.off_nodes = pad16(o); o = H.off_nodes + (int64_t)nodes.size() * 4;
    H.bytes = pad16(o);
    if (H.bytes > (1 << 20)) return 3;
    out.assign(H.bytes, 0);
    uint8_t* B = out.data();
    std::memcpy(B, &H, sizeof(RecHead));
    std::memcpy(B + sizeof(RecHead), rsegs.data(), (size_t)n_seg * sizeof(RecSeg));
    for (int32_t te = 0; te < n_ent; ++te) {
        std::memcpy(B + H.off_ent + (int64_t)te * 16, &rent[te], 16);
        const int32_t id = ents[te];
        std::memcpy(B + H.off_eid + (int64_t)te * 4, &id, 4);
        const uint32_t fk = (uint32_t)fbase[te] | ((uint32_t)kc[te] << 16);
        std::memcpy(B + H.off_fk + (int64_t)te * 4, &fk, 4);
    }
    std::memcpy(B + H.off_red, red_sorted.data(), (size_t)n_red * 4);
    std::memcpy(B + H.off_runs, runs.data(), (size_t)n_runs * 16);
    std::memcpy(B + H.off_pass, passes.data(), (size_t)n_pass * 32);
    std::memcpy(B + H.off_rng, rngs.data(), (size_t)n_rng * 16);
    // cells, items and slot rows in cell order
    for (int32_t g = 0; g < n_seg; ++g) {
        const HostSub& hs = hp.subs[segs[g].sub];
        const RecSeg& R = rsegs[g];
        for (int32_t c = R.cell_begin; c < R.cell_end; ++c) {
            const int32_t i0 = cell_item0[c], i1 = c + 1 < n_cells ? cell_item0[c + 1] : n_items;
            std::memcpy(B + H.off_cells + (int64_t)c * 4, &cells[c], 4);
            uint16_t* cn = (uint16_t*)(B + R.conn_off) + (int64_t)(c - R.cell_begin) * hs.ng;
            for (int a = 0; a < hs.ng; ++a) cn[a] = local_node(hs.conn[(int64_t)cells[c] * hs.ng + a]);
            for (int32_t it = i0; it < i1; ++it) {
                const TileItem& I = items[it];
                const uint32_t w = (uint32_t)I.j | ((uint32_t)(fbase[I.te] + I.k) << 16);
                std::memcpy(B + H.off_items + (int64_t)it * 4, &w, 4);
                uint16_t* sl = (uint16_t*)(B + R.slot_off) + (int64_t)(it - R.item_begin) * hs.nb;
                for (int i = 0; i < hs.nb; ++i) {
                    const int32_t b = row_block[item_row0[it] + i];
                    sl[i] = b < 0 ? SLOT_MISS : (uint16_t)(base[b] + row_ord[item_row0[it] + i] * stride[b]);
                }
            }
        }
    }
    {
        int32_t tn = 0;
        for (int32_t g = 0; g < n_seg; ++g) {
            uint16_t* gt = (uint16_t*)(B + rsegs[g].gt_off);
            for (int32_t w = 0; w < rsegs[g].n_grp; ++w) {
                gt[w] = (uint16_t)tn;
                for (const TileTask& T : seg_tasks[g][w]) {
                    RecTask rt{(uint16_t)T.cell, (uint16_t)T.i0, (uint16_t)T.i1, 0};
                    std::memcpy(B + H.off_tasks + (int64_t)tn * 8, &rt, 8);
                    ++tn;
                }
            }
            gt[rsegs[g].n_grp] = (uint16_t)tn;
        }
    }
    std::memcpy(B + H.off_nodes, nodes.data(), nodes.size() * 4);
    n_nodes_out = (int32_t)nodes.size();
    stage_out = n_slots * bs + n_fslots * nc;
    n_cells_out = n_cells;
    n_items_out = n_items;
    out_len_out = 0;
    for (const RecPass& P : passes) out_len_out = std::max(out_len_out, P.out_len);
    return 0;
}

}  // namespace

int build_plan(const HostProblem& hp, const PlanOptions& opt, Plan& plan, Error& err) {
    const int nc = hp.nc;
    const int64_t n_ent = hp.n_ent;
    const int dim = hp.dim;
    const int64_t* cp = hp.colptr.data();
    int nb_max = 0;
    for (const HostSub& hs : hp.subs) nb_max = std::max(nb_max, hs.nb);
    // entity "positions" (mean of incident cell centroids) and incident cell counts
    std::vector<double> pos(n_ent * 3, 0.0);
    std::vector<int32_t> kcount(n_ent, 0);
    for (const HostSub& hs : hp.subs) {
        // cell centroids in parallel, then the sums per entity in cell order (the same bits)
        HostBuf<double> cens((size_t)hs.n_cells * 3);
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < hs.n_cells; ++k) {
            double cen[3] = {0, 0, 0};
            for (int a = 0; a < hs.ng; ++a)
                for (int x = 0; x < dim; ++x) cen[x] += hp.nodes[(int64_t)hs.conn[k * hs.ng + a] * dim + x];
            for (int x = 0; x < 3; ++x) cens[k * 3 + x] = x < dim ? cen[x] / hs.ng : 0.0;
        }
        for (int64_t k = 0; k < hs.n_cells; ++k)
            for (int i = 0; i < hs.nb; ++i) {
                const int64_t n = hs.ents[k * hs.nb + i];
                for (int x = 0; x < dim; ++x) pos[n * 3 + x] += cens[k * 3 + x];
                kcount[n]++;
            }
    }
    for (int64_t n = 0; n < n_ent; ++n) {
        if (kcount[n] > MAX_ENT_CELLS) return fail(err, FE_ERR_UNSUPPORTED, "a dof entity belongs to more than 255 cells");
        if (!kcount[n]) continue;
        for (int x = 0; x < dim; ++x) pos[n * 3 + x] /= kcount[n];
    }
    auto nnb_of = [&](int64_t n) { return (int64_t)((cp[nc * n + 1] - cp[nc * n]) / nc); };
    const int bs = (nc * nc + 1) & ~1;
    const int32_t out_cap = opt.resolved_out_cap();
    // per-entity loads of a tile: staging values (an upper bound: every row of every cell gets a
    // slot), reduce lanes, and output doubles (the reduce's one-pass buffer)
    auto stage_of = [&](int64_t n) { return (int64_t)kcount[n] * (nb_max * bs + nc); };
    auto out_of = [&](int64_t n) { return (int64_t)(cp[nc * n + nc] - cp[nc * n]); };
    for (int64_t n = 0; n < n_ent; ++n)
        if (stage_of(n) > opt.stage_cap || nnb_of(n) > opt.red_cap || out_of(n) > out_cap)
            return fail(err, FE_ERR_UNSUPPORTED, "a dof entity's contributions exceed the tile capacity");
    // sized for the heaviest entities (the interior ones), so interior tiles fit without splits
    double max_stage = 1, max_nnb = 1, max_out = 1, sum_stage = 0, sum_nnb = 0, sum_out = 0, n_act = 0;
    for (int64_t n = 0; n < n_ent; ++n) {
        max_stage = std::max(max_stage, (double)stage_of(n));
        max_nnb = std::max(max_nnb, (double)nnb_of(n));
        max_out = std::max(max_out, (double)out_of(n));
        if (!kcount[n]) continue;
        sum_stage += (double)stage_of(n);
        sum_nnb += (double)nnb_of(n);
        sum_out += (double)out_of(n);
        n_act += 1;
    }
    // Tiles by recursive coordinate bisection: the entities are split along the longest extent
    // into as many equal parts as an average tile size allows, so tiles are compact, of nearly
    // equal size and all fit the capacities (a part that does not is split again). Within a
    // tile entities are ordered by id, so its nzval is a few contiguous ranges.
    const double lim = std::min((double)opt.ent_cap, (double)MAX_TILE_ENTS);
    const double target = std::max(1.0, std::min({std::floor(opt.stage_cap / max_stage), std::floor(opt.red_cap / max_nnb),
                                                  std::floor(out_cap / max_out), lim}));
    // Entities of unequal loads (on Q2 meshes a vertex node sits in 8 cells, edge, face and
    // interior nodes in 4, 2 and 1; mixed cell types): tiles sized for the heaviest would hold
    // half as many entities as fit. Each part of the bisection is then cut into as many pieces
    // as its own summed load needs, so tiles are full where entities are light or heavy alike.
    const bool uneven = n_act > 0 && (max_stage > 1.25 * sum_stage / n_act || max_nnb > 1.25 * sum_nnb / n_act ||
                                      max_out > 1.25 * sum_out / n_act);
    // The entities with their positions, permuted together, so the selections and bounding
    // boxes below read memory in order.
    struct EntPos {
        double p[3];
        int32_t id;
    };
    std::vector<EntPos> ep(n_ent);
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < n_ent; ++n) {
        for (int x = 0; x < 3; ++x) ep[n].p[x] = pos[n * 3 + x];
        ep[n].id = (int32_t)n;
    }
    auto fits = [&](int64_t lo, int64_t hi) {
        if (hi - lo > opt.ent_cap || hi - lo > MAX_TILE_ENTS) return false;
        int64_t st = 0, rd = 0, ot = 0;
        for (int64_t q = lo; q < hi; ++q) {
            st += stage_of(ep[q].id);
            rd += nnb_of(ep[q].id);
            ot += out_of(ep[q].id);
        }
        return st <= opt.stage_cap && rd <= opt.red_cap && ot <= out_cap;
    };
    // Recursive bisection of ep[lo, hi) into k parts. The parts are disjoint ranges, so the
    // leaves in depth-first (left first) order are the leaves by ascending start; large parts
    // are split in parallel and the leaves sorted afterwards.
    std::vector<std::pair<int64_t, int64_t>> leaves;
    // pieces of ep[lo, hi) by its load relative to the capacities (leaves average 88 % of it)
    auto pieces = [&](int64_t lo, int64_t hi) {
        double st = 0, rd = 0, ot = 0;
        for (int64_t q = lo; q < hi; ++q) {
            const int64_t id = ep[q].id;
            st += (double)stage_of(id);
            rd += (double)nnb_of(id);
            ot += (double)out_of(id);
        }
        const double load = std::max({st / opt.stage_cap, rd / opt.red_cap, ot / out_cap, (double)(hi - lo) / lim});
        return std::max<int64_t>(1, (int64_t)std::ceil(load / 0.88));
    };
    std::function<void(int64_t, int64_t, int64_t)> split = [&](int64_t lo, int64_t hi, int64_t k) {
        const int64_t n = hi - lo;
        if (n == 0) return;
        if (uneven) k = pieces(lo, hi);
        k = std::min(k, n);
        if (k == 1) {
            if (fits(lo, hi) || n == 1) {
#pragma omp critical(fe_plan_leaves)
                leaves.emplace_back(lo, hi);
                return;
            }
            k = 2;
        }
        double lo_[3] = {1e300, 1e300, 1e300}, hi_[3] = {-1e300, -1e300, -1e300};
        for (int64_t q = lo; q < hi; ++q)
            for (int x = 0; x < dim; ++x) {
                lo_[x] = std::min(lo_[x], ep[q].p[x]);
                hi_[x] = std::max(hi_[x], ep[q].p[x]);
            }
        int ax = 0;
        for (int x = 1; x < dim; ++x)
            if (hi_[x] - lo_[x] > hi_[ax] - lo_[ax]) ax = x;
        const int64_t kl = k / 2;
        int64_t nl = (int64_t)std::llround((double)n * (double)kl / (double)k);
        // order along the axis (ties by the other coordinates, then id) and move the cut to the
        // nearest change of the axis coordinate within 15 %, so cuts follow element layers
        const int ax1 = (ax + 1) % dim, ax2 = (ax + 2) % dim;
        auto less = [&](const EntPos& x, const EntPos& y) {
            if (x.p[ax] != y.p[ax]) return x.p[ax] < y.p[ax];
            if (x.p[ax1] != y.p[ax1]) return x.p[ax1] < y.p[ax1];
            if (dim > 2 && x.p[ax2] != y.p[ax2]) return x.p[ax2] < y.p[ax2];
            return x.id < y.id;
        };
        const int64_t slack = std::max<int64_t>(1, (int64_t)(0.15 * (double)nl));
        // In axis order the axis coordinate changes only at layer boundaries, so the nearest
        // change to rank nl is the start c1 or the end c2 of the layer of the entity of rank nl:
        // one selection finds that entity, one counting pass the layer's ranks, and a second
        // selection (if the cut moves) puts the `best` smallest entities first. `less` is a
        // strict total order, so the parts hold the same entities as after a full sort, and each
        // part is ordered again before it is split or emitted.
        auto b = ep.begin() + lo;
        std::nth_element(b, b + nl, b + n, less);
        const double v = b[nl].p[ax];
        int64_t c1 = 0, c2 = 0;
        for (int64_t q = 0; q < n; ++q) {
            c1 += b[q].p[ax] < v;
            c2 += b[q].p[ax] <= v;
        }
        int64_t best = nl;  // the nearer of c1 and c2 within the slack, c1 on a tie
        const bool ok1 = c1 > 0 && nl - c1 <= slack, ok2 = c2 < n && c2 - nl <= slack;
        if (ok1 && (!ok2 || nl - c1 <= c2 - nl)) best = c1;
        else if (ok2) best = c2;
        if (best != nl) std::nth_element(b, b + best, b + n, less);
        nl = best;
        if (n >= (1 << 16)) {
#pragma omp task default(shared) firstprivate(lo, nl, kl)
            split(lo, lo + nl, kl);
            split(lo + nl, hi, k - kl);
#pragma omp taskwait
        } else {
            split(lo, lo + nl, kl);
            split(lo + nl, hi, k - kl);
        }
    };
    // leaves average 88 % of the target: the layer-snapped cuts vary part sizes by up to 15 %
    const int64_t k0 = std::max<int64_t>(1, (int64_t)std::ceil((double)n_ent / (0.88 * target)));
#pragma omp parallel
#pragma omp single
    split(0, n_ent, k0);
    std::sort(leaves.begin(), leaves.end());
    // tiles in leaf order; within a tile entities by id, so its nzval is a few contiguous ranges
    const int64_t n_leaves = (int64_t)leaves.size();
    std::vector<int32_t> tile_of(n_ent), tile_local(n_ent);
    std::vector<int32_t> eids(n_ent);  // owned entities, tile after tile
    std::vector<int64_t> tent(n_leaves + 1, 0);  // tile t owns eids[tent[t] .. tent[t+1])
    for (int64_t t = 0; t < n_leaves; ++t) tent[t + 1] = leaves[t].second;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t t = 0; t < n_leaves; ++t) {
        const int64_t lo = leaves[t].first, hi = leaves[t].second;
        for (int64_t q = lo; q < hi; ++q) eids[q] = ep[q].id;
        std::sort(eids.begin() + lo, eids.begin() + hi);
        for (int64_t q = lo; q < hi; ++q) {
            tile_of[eids[q]] = (int32_t)t;
            tile_local[eids[q]] = (int32_t)(q - lo);
        }
    }
    const int64_t n_tiles = (int64_t)tent.size() - 1;
    // (sub, cell, j) triples per tile, in (sub, cell, j) order
    std::vector<int64_t> tstart(n_tiles + 1, 0);
    for (const HostSub& hs : hp.subs)
        for (size_t t = 0; t < hs.ents.size(); ++t) tstart[tile_of[hs.ents[t]] + 1]++;
    for (int64_t t = 0; t < n_tiles; ++t) tstart[t + 1] += tstart[t];
    HostBuf<uint64_t> trip(tstart[n_tiles]);
    {
        std::vector<int64_t> cur(tstart.begin(), tstart.end() - 1);
        for (size_t s = 0; s < hp.subs.size(); ++s) {
            const HostSub& hs = hp.subs[s];
            for (int64_t k = 0; k < hs.n_cells; ++k)
                for (int j = 0; j < hs.nb; ++j) {
                    const int32_t t = tile_of[hs.ents[k * hs.nb + j]];
                    trip[cur[t]++] = ((uint64_t)s << 40) | ((uint64_t)k << 8) | (uint64_t)j;
                }
        }
    }
    std::vector<std::vector<uint8_t>> recs(n_tiles);
    std::vector<int32_t> rn(n_tiles), rs(n_tiles), rc(n_tiles), ri(n_tiles), ro(n_tiles);
    int status = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(max : status)
    for (int64_t t = 0; t < n_tiles; ++t) {
        const int st = build_record(hp, kcount, tile_local, eids.data() + tent[t], (int32_t)(tent[t + 1] - tent[t]),
                                    trip.data() + tstart[t], tstart[t + 1] - tstart[t], recs[t], rn[t], rs[t], rc[t], ri[t], ro[t], out_cap);
        status = std::max(status, st);
    }
    if (status == 1) return fail(err, FE_ERR_ARG, "internal: incident cell count mismatch");
    if (status == 2) return fail(err, FE_ERR_UNSUPPORTED, "an owned block has more than 255 contributions");
    if (status == 4) return fail(err, FE_ERR_UNSUPPORTED, "the columns of one dof entity exceed the output buffer");
    if (status) return fail(err, FE_ERR_UNSUPPORTED, "a tile record exceeds its limits");
    plan.n_tiles = n_tiles;
    plan.rec_off.assign(n_tiles + 1, 0);
    plan.max_rec = plan.max_nodes = plan.max_stage = plan.max_out = 0;
    plan.visits = plan.items = 0;
    for (int64_t t = 0; t < n_tiles; ++t) {
        plan.rec_off[t + 1] = plan.rec_off[t] + (int64_t)recs[t].size();
        plan.max_rec = std::max(plan.max_rec, (int32_t)recs[t].size());
        plan.max_nodes = std::max(plan.max_nodes, rn[t]);
        plan.max_stage = std::max(plan.max_stage, rs[t]);
        plan.max_out = std::max(plan.max_out, ro[t]);
        plan.visits += rc[t];
        plan.items += ri[t];
    }
    plan.rec.resize(plan.rec_off[n_tiles]);
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_tiles; ++t) {
        std::memcpy(plan.rec.data() + plan.rec_off[t], recs[t].data(), recs[t].size());
        std::vector<uint8_t>().swap(recs[t]);
    }
    return FE_OK;
}

// ---------------------------------------------------------------------------------------
// Record check: parses every record the way the kernel does and verifies that each index
// stays inside the buffer it addresses (record, staging, node list, nzval, f, subdomain
// arrays) and that the slots are a bijection onto the owned blocks' contributions with
// the right destinations. Run once per fe_create.
// ---------------------------------------------------------------------------------------
namespace {
// Working arrays of check_plan, one set per thread and reused from tile to tile
struct CheckScratch {
    std::vector<int32_t> slot_block, blk_pass, slot_writes, fslot_writes, item_cover;
    std::vector<int64_t> slot_cell;
    std::vector<std::vector<int32_t>> owner;  // per pass; entries past n_pass are stale
};
}  // namespace

int check_plan(const HostProblem& hp, const Plan& pl, Error& err) {
    const int nc = hp.nc;
    const int64_t* cp = hp.colptr.data();
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : bad)
    for (int64_t t = 0; t < pl.n_tiles; ++t) {
        thread_local CheckScratch CS;
        const int64_t off = pl.rec_off[t], len = pl.rec_off[t + 1] - off;
        if ((off & 15) || len < (int64_t)sizeof(RecHead) || len > pl.max_rec) { bad = 1; continue; }
        const uint8_t* B = pl.rec.data() + off;
        RecHead H;
        std::memcpy(&H, B, sizeof(RecHead));
        auto in = [&](int64_t o, int64_t n) { return o >= 0 && (o & 15) == 0 && o + n <= len; };
        if (H.bytes != len || H.n_seg < 0 || H.n_ent < 0 || H.n_cells < 0 || H.n_items < 0 || H.n_red < 0 ||
            H.n_nodes < 0 || H.n_nodes > pl.max_nodes || H.n_slots < 0 || H.n_fslots < 0 || H.n_runs < 0 ||
            H.n_pass < 0 || H.n_rng < 0 || H.n_tasks < 0 || !in(H.off_tasks, (int64_t)H.n_tasks * 8) ||
            (int64_t)sizeof(RecHead) + (int64_t)H.n_seg * (int64_t)sizeof(RecSeg) > len ||
            !in(H.off_ent, (int64_t)H.n_ent * 16) || !in(H.off_eid, (int64_t)H.n_ent * 4) ||
            !in(H.off_fk, (int64_t)H.n_ent * 4) || !in(H.off_red, (int64_t)H.n_red * 4) ||
            !in(H.off_runs, (int64_t)H.n_runs * 16) || !in(H.off_pass, (int64_t)H.n_pass * 32) ||
            !in(H.off_rng, (int64_t)H.n_rng * 16) || !in(H.off_items, (int64_t)H.n_items * 4) ||
            !in(H.off_cells, (int64_t)H.n_cells * 4) || !in(H.off_nodes, (int64_t)H.n_nodes * 4) ||
            H.n_ent > MAX_TILE_ENTS ||
            (int64_t)H.n_slots * ((nc * nc + 1) & ~1) + (int64_t)H.n_fslots * nc > pl.max_stage) {
            bad = 1;
            continue;
        }
        const RecSeg* S = (const RecSeg*)(B + sizeof(RecHead));
        const RecEnt* E = (const RecEnt*)(B + H.off_ent);
        const int32_t* EID = (const int32_t*)(B + H.off_eid);
        const uint32_t* FK = (const uint32_t*)(B + H.off_fk);
        const uint32_t* RED = (const uint32_t*)(B + H.off_red);
        const RecRun* RU = (const RecRun*)(B + H.off_runs);
        const RecPass* PS = (const RecPass*)(B + H.off_pass);
        const RecRng* RG = (const RecRng*)(B + H.off_rng);
        const uint32_t* IT = (const uint32_t*)(B + H.off_items);
        const int32_t* C = (const int32_t*)(B + H.off_cells);
        const int32_t* ND = (const int32_t*)(B + H.off_nodes);
        // entities: column base and length as in colptr; f slots inside the f area
        for (int32_t e = 0; e < H.n_ent && !bad; ++e) {
            const int64_t n = EID[e];
            if (n < 0 || n >= hp.n_ent || E[e].colbase != cp[nc * n] - 1 || E[e].L != cp[nc * n + 1] - cp[nc * n] ||
                E[e].colbase + (int64_t)nc * E[e].L > hp.nnz || (int64_t)(FK[e] & 0xFFFF) + (FK[e] >> 16) > H.n_fslots)
                bad = 1;
        }
        // passes partition the blocks, runs and ranges in order; within a pass the runs cover
        // its blocks and hand out k-major slot ranges, consecutive over the whole tile
        auto& slot_block = CS.slot_block;
        auto& blk_pass = CS.blk_pass;
        slot_block.assign(H.n_slots, -1);
        blk_pass.assign(H.n_red, -1);
        {
            int32_t red_next = 0, run_next = 0, rng_next = 0, slot_next = 0;
            for (int32_t p = 0; p < H.n_pass && !bad; ++p) {
                const RecPass& P = PS[p];
                if (P.red_begin != red_next || P.red_end < P.red_begin || P.red_end > H.n_red || P.run_begin != run_next ||
                    P.run_end < P.run_begin || P.run_end > H.n_runs || P.rng_begin != rng_next || P.rng_end < P.rng_begin ||
                    P.rng_end > H.n_rng || P.out_len < 0 || P.out_len > pl.max_out) {
                    bad = 1;
                    break;
                }
                int32_t q = P.red_begin;
                for (int32_t u = P.run_begin; u < P.run_end; ++u) {
                    const RecRun& U = RU[u];
                    if (U.first != q || U.nblk < 1 || q + U.nblk > P.red_end || U.count < 0 || U.count > MAX_ENT_CELLS ||
                        U.base != slot_next || (int64_t)U.base + (int64_t)U.count * U.nblk > H.n_slots) { bad = 1; break; }
                    // the kernel's lookup: block first + j, contribution k -> base + k * nblk + j
                    for (int32_t j = 0; j < U.nblk; ++j) {
                        blk_pass[q + j] = p;
                        for (int32_t k = 0; k < U.count; ++k) slot_block[U.base + k * U.nblk + j] = q + j;
                    }
                    q += U.nblk;
                    slot_next += U.count * U.nblk;
                }
                if (bad || q != P.red_end) { bad = 1; break; }
                for (int32_t g = P.rng_begin; g < P.rng_end; ++g)
                    if (RG[g].len < 1 || RG[g].buf_off < 0 || RG[g].buf_off + RG[g].len > P.out_len || ((RG[g].buf_off - RG[g].nz0) & 1) ||
                        RG[g].nz0 < 0 || RG[g].nz0 + RG[g].len > hp.nnz) { bad = 1; break; }
                red_next = P.red_end;
                run_next = P.run_end;
                rng_next = P.rng_end;
            }
            if (bad || red_next != H.n_red || run_next != H.n_runs || rng_next != H.n_rng || slot_next != H.n_slots) {
                bad = 1;
                continue;
            }
        }
        // blocks: ranks inside the column; every output entry lands in a buffer position of its
        // pass that one range maps to that entry's nzval index, and every range position is written once
        {
            // per pass and buffer position: -1 no range, g the one range covering it (a second
            // range is an error), -2 - g once a block entry has been written there
            auto& own = CS.owner;
            if ((int32_t)own.size() < H.n_pass) own.resize(H.n_pass);
            for (int32_t p = 0; p < H.n_pass && !bad; ++p) {
                own[p].assign(PS[p].out_len, -1);
                for (int32_t g = PS[p].rng_begin; g < PS[p].rng_end && !bad; ++g)
                    for (int32_t i = RG[g].buf_off; i < RG[g].buf_off + RG[g].len; ++i) {
                        if (own[p][i] != -1) { bad = 1; break; }
                        own[p][i] = g;
                    }
            }
            for (int32_t q = 0; q < H.n_red && !bad; ++q) {
                const int32_t e = (int32_t)(RED[q] >> RED_RANK_BITS), r = (int32_t)(RED[q] & ((1u << RED_RANK_BITS) - 1));
                const int32_t p = blk_pass[q];
                if (e >= H.n_ent || (int64_t)nc * r >= E[e].L || p < 0) { bad = 1; break; }
                const RecPass& P = PS[p];
                for (int b = 0; b < nc && !bad; ++b)
                    for (int x = 0; x < nc; ++x) {
                        const int64_t i = (int64_t)E[e].out_off + (int64_t)b * E[e].L + (int64_t)nc * r + x;
                        if (E[e].out_off < 0 || i >= P.out_len) { bad = 1; break; }
                        const int64_t want = E[e].colbase + (int64_t)b * E[e].L + (int64_t)nc * r + x;
                        // one range covers i, it maps i to this entry's nzval index, and no other
                        // entry was written there
                        const int32_t g = own[p][i];
                        if (g < 0 || RG[g].nz0 + (i - RG[g].buf_off) != want) { bad = 1; break; }
                        own[p][i] = -2 - g;
                    }
            }
            // every range position written
            for (int32_t p = 0; p < H.n_pass && !bad; ++p)
                for (int32_t g = PS[p].rng_begin; g < PS[p].rng_end && !bad; ++g)
                    for (int32_t i = RG[g].buf_off; i < RG[g].buf_off + RG[g].len; ++i)
                        if (own[p][i] >= -1) { bad = 1; break; }
        }
        if (bad) continue;
        for (int32_t e = 0; e < H.n_nodes && !bad; ++e)
            if (ND[e] < 0 || ND[e] >= hp.n_nodes) bad = 1;
        // segments, cells, items, slots
        auto& slot_writes = CS.slot_writes;
        auto& fslot_writes = CS.fslot_writes;
        auto& slot_cell = CS.slot_cell;  // (sub, cell) of each slot's contribution
        slot_writes.assign(H.n_slots, 0);
        fslot_writes.assign(H.n_fslots, 0);
        slot_cell.assign(H.n_slots, -1);
        int32_t cell_next = 0, item_next = 0, task_next = 0;
        for (int32_t g = 0; g < H.n_seg && !bad; ++g) {
            const RecSeg& G = S[g];
            if (G.sub < 0 || G.sub >= (int)hp.subs.size() || G.cell_begin != cell_next || G.cell_end < G.cell_begin ||
                G.cell_end > H.n_cells || G.item_begin != item_next || G.item_end < G.item_begin || G.item_end > H.n_items) {
                bad = 1;
                break;
            }
            const HostSub& hs = hp.subs[G.sub];
            if (!in(G.conn_off, (int64_t)(G.cell_end - G.cell_begin) * hs.ng * 2) ||
                !in(G.slot_off, (int64_t)(G.item_end - G.item_begin) * hs.nb * 2)) { bad = 1; break; }
            const uint16_t* CN = (const uint16_t*)(B + G.conn_off);
            const uint16_t* SL = (const uint16_t*)(B + G.slot_off);
            // cells: node list entries of the cell's nodes
            for (int32_t c = G.cell_begin; c < G.cell_end && !bad; ++c) {
                const int64_t cell = C[c];
                if (cell < 0 || cell >= hs.n_cells) { bad = 1; break; }
                for (int a = 0; a < hs.ng; ++a) {
                    const int ln = CN[(int64_t)(c - G.cell_begin) * hs.ng + a];
                    if (ln >= H.n_nodes || ND[ln] != hs.conn[cell * hs.ng + a]) { bad = 1; break; }
                }
            }
            // group task table: consecutive task ranges; tasks inside the segment, together
            // covering each item of the segment exactly once; each item's j, f slot and slots
            // are those of the task's cell
            if (bad || G.n_grp < 1 || !in(G.gt_off, (int64_t)(G.n_grp + 1) * 2)) { bad = 1; break; }
            const uint16_t* GT = (const uint16_t*)(B + G.gt_off);
            const RecTask* TK = (const RecTask*)(B + H.off_tasks);
            if (GT[0] != task_next || GT[G.n_grp] > H.n_tasks) { bad = 1; break; }
            auto& cover = CS.item_cover;
            cover.assign(G.item_end - G.item_begin, 0);
            for (int32_t w = 0; w < G.n_grp && !bad; ++w) {
                if (GT[w + 1] < GT[w]) { bad = 1; break; }
                for (int32_t q = GT[w]; q < GT[w + 1] && !bad; ++q) {
                    const RecTask& T = TK[q];
                    if (T.cell < G.cell_begin || T.cell >= G.cell_end || T.item_begin < G.item_begin || T.item_end > G.item_end ||
                        T.item_end < T.item_begin) { bad = 1; break; }
                    const int64_t cell = C[T.cell];
                    for (int32_t it = T.item_begin; it < T.item_end && !bad; ++it) {
                        cover[it - G.item_begin]++;
                        const int j = (int)(IT[it] & 0xFF);
                        const int32_t fs = (int32_t)(IT[it] >> 16);
                        if (j >= hs.nb || fs >= H.n_fslots) { bad = 1; break; }
                        fslot_writes[fs]++;
                        const int64_t n = hs.ents[cell * hs.nb + j];
                        for (int i = 0; i < hs.nb; ++i) {
                            const uint16_t sl = SL[(int64_t)(it - G.item_begin) * hs.nb + i];
                            const int r = rank_of(hs, cell, j, i);
                            if (sl == SLOT_MISS) {
                                if (r >= 0) { bad = 1; break; }
                                continue;
                            }
                            if (sl >= H.n_slots || r < 0) { bad = 1; break; }
                            const int32_t qb = slot_block[sl];
                            const int32_t e = (int32_t)(RED[qb] >> RED_RANK_BITS);
                            if (EID[e] != n || (int32_t)(RED[qb] & ((1u << RED_RANK_BITS) - 1)) != r) { bad = 1; break; }
                            slot_writes[sl]++;
                            slot_cell[sl] = ((int64_t)G.sub << 32) | cell;
                        }
                    }
                }
            }
            for (int32_t it = 0; it < G.item_end - G.item_begin && !bad; ++it)
                if (cover[it] != 1) bad = 1;
            task_next = GT[G.n_grp];
            cell_next = G.cell_end;
            item_next = G.item_end;
        }
        if (bad || cell_next != H.n_cells || item_next != H.n_items || task_next != H.n_tasks) { bad = 1; continue; }
        for (int32_t sl = 0; sl < H.n_slots; ++sl)
            if (slot_writes[sl] != 1) { bad = 1; break; }
        // each block sums its contributions in cell order: (sub, cell) increasing along its slots
        for (int32_t u = 0; u < H.n_runs && !bad; ++u)
            for (int32_t j = 0; j < RU[u].nblk && !bad; ++j)
                for (int32_t k = 1; k < RU[u].count; ++k)
                    if (slot_cell[RU[u].base + k * RU[u].nblk + j] <= slot_cell[RU[u].base + (k - 1) * RU[u].nblk + j]) { bad = 1; break; }
        for (int32_t fs = 0; fs < H.n_fslots; ++fs)
            if (fslot_writes[fs] != 1) { bad = 1; break; }
    }
    if (bad) return fail(err, FE_ERR_ARG, "internal: tile plan failed its bounds check");
    return FE_OK;
}

}  // namespace fe
