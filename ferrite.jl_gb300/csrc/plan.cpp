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
#include <numeric>
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
    if (!P->colptr || !P->rowval) return fail(err, FE_ERR_ARG, "null colptr/rowval");
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
    hp.cell_dofs.assign(d->cell_dofs, d->cell_dofs + maxdof_end);
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
    // ranks (the index map)
    for (int s = 0; s < in.n_sub; ++s) {
        HostSub& hs = hp.subs[s];
        const int nb = hs.nb;
        std::vector<uint16_t> r16((size_t)hs.n_cells * nb * nb);
        int maxr = 0;
#pragma omp parallel for schedule(static) reduction(max : maxr)
        for (int64_t k = 0; k < hs.n_cells; ++k) {
            const int32_t* e = &hs.ents[k * nb];
            for (int j = 0; j < nb; ++j) {
                const int64_t n = e[j];
                const int64_t c0 = cp[nc * n] - 1;
                const int64_t Le = (cp[nc * n + 1] - cp[nc * n]) / nc;
                for (int i = 0; i < nb; ++i) {
                    const int64_t want = (int64_t)e[i] * nc + 1;
                    int64_t lo = 0, hi = Le;
                    while (lo < hi) {
                        const int64_t mid = (lo + hi) >> 1;
                        if (rv[c0 + nc * mid] < want) lo = mid + 1; else hi = mid;
                    }
                    uint16_t r = 0xFFFF;
                    if (lo < Le && rv[c0 + nc * lo] == want && lo < 0xFFFF) r = (uint16_t)lo;
                    r16[((size_t)k * nb + j) * nb + i] = r;
                    if (r != 0xFFFF) maxr = std::max(maxr, (int)r);
                }
            }
        }
        if (maxr < 255) {
            hs.rank8.resize(r16.size());
            for (size_t t = 0; t < r16.size(); ++t) hs.rank8[t] = r16[t] == 0xFFFF ? 255 : (uint8_t)r16[t];
            hs.wide_rank = false;
        } else {
            hs.rank16.swap(r16);
            hs.wide_rank = true;
        }
    }
    return FE_OK;
}

// ---------------------------------------------------------------------------------------
// Owner tiles
//
// Entities are bucketed by position into compact tiles (a handful of contiguous id runs
// each). A tile lists every cell touching one of its entities; for every (cell, owned base
// function j) an item carries k, the position of the cell among the cells of entity(j) in
// cell order. The kernel writes each contribution to its own staging slot (entity, k, i) and
// the reduce step sums the slots of an entry in k order: the reference's cell order.
// ---------------------------------------------------------------------------------------
int build_plan(const HostProblem& hp, const PlanOptions& opt, Plan& plan, Error& err) {
    const int nc = hp.nc;
    const int64_t n_ent = hp.n_ent;
    const int dim = hp.dim;
    const int64_t* cp = hp.colptr.data();
    int nb_max = 0;
    for (const HostSub& hs : hp.subs) nb_max = std::max(nb_max, hs.nb);
    plan.nb_max = nb_max;
    // entity "positions" (mean of incident cell centroids) and incident cell counts
    std::vector<double> pos(n_ent * 3, 0.0);
    std::vector<int32_t> kcount(n_ent, 0);
    for (const HostSub& hs : hp.subs) {
        for (int64_t k = 0; k < hs.n_cells; ++k) {
            double cen[3] = {0, 0, 0};
            for (int a = 0; a < hs.ng; ++a)
                for (int x = 0; x < dim; ++x) cen[x] += hp.nodes[(int64_t)hs.conn[k * hs.ng + a] * dim + x];
            for (int x = 0; x < dim; ++x) cen[x] /= hs.ng;
            for (int i = 0; i < hs.nb; ++i) {
                const int64_t n = hs.ents[k * hs.nb + i];
                for (int x = 0; x < dim; ++x) pos[n * 3 + x] += cen[x];
                kcount[n]++;
            }
        }
    }
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t n = 0; n < n_ent; ++n) {
        if (kcount[n] > MAX_ENT_CELLS) return fail(err, FE_ERR_UNSUPPORTED, "a dof entity belongs to more than 63 cells");
        if (!kcount[n]) continue;
        for (int x = 0; x < dim; ++x) {
            pos[n * 3 + x] /= kcount[n];
            lo[x] = std::min(lo[x], pos[n * 3 + x]);
            hi[x] = std::max(hi[x], pos[n * 3 + x]);
        }
    }
    auto nnb_of = [&](int64_t n) { return (int64_t)((cp[nc * n + 1] - cp[nc * n]) / nc); };
    const int bs = (nc * nc + 1) & ~1;
    auto stage_of = [&](int64_t n) { return ((int64_t)kcount[n] * (nb_max * bs + nc) + 1) & ~1ll; };
    auto map_of = [&](int64_t n) { return nnb_of(n) * kcount[n]; };
    // target entities per tile from the staging capacity
    double avg_stage = 0;
    for (int64_t n = 0; n < n_ent; ++n) avg_stage += (double)stage_of(n);
    avg_stage = std::max(1.0, avg_stage / (double)n_ent);
    double avg_nnb = 0;
    for (int64_t n = 0; n < n_ent; ++n) avg_nnb += (double)nnb_of(n);
    avg_nnb = std::max(1.0, avg_nnb / (double)n_ent);
    const double target_ent = std::max(1.0, std::min({0.85 * opt.stage_cap / avg_stage, 0.85 * opt.ent_cap,
                                                       0.85 * opt.red_cap / avg_nnb}));
    const double n_tiles_target = std::max(1.0, (double)n_ent / target_ent);
    double ext[3] = {1, 1, 1}, vol = 1;
    for (int x = 0; x < dim; ++x) {
        ext[x] = std::max(hi[x] - lo[x], 1e-300);
        vol *= ext[x];
    }
    const double side = std::pow(vol / n_tiles_target, 1.0 / dim);
    int64_t nt[3] = {1, 1, 1};
    for (int x = 0; x < dim; ++x) nt[x] = std::max<int64_t>(1, (int64_t)std::llround(ext[x] / side));
    const int64_t nbk = nt[0] * nt[1] * nt[2];
    std::vector<int64_t> bstart(nbk + 1, 0);
    std::vector<int64_t> bucket(n_ent);
    for (int64_t n = 0; n < n_ent; ++n) {
        int64_t id[3] = {0, 0, 0};
        if (kcount[n])
            for (int x = 0; x < dim; ++x) {
                int64_t t = (int64_t)((pos[n * 3 + x] - lo[x]) / ext[x] * nt[x]);
                id[x] = std::min(std::max<int64_t>(t, 0), nt[x] - 1);
            }
        bucket[n] = id[0] + nt[0] * (id[1] + nt[1] * id[2]);
        bstart[bucket[n] + 1]++;
    }
    for (int64_t b = 0; b < nbk; ++b) bstart[b + 1] += bstart[b];
    std::vector<int32_t> order(n_ent);
    {
        std::vector<int64_t> cur(bstart.begin(), bstart.end() - 1);
        for (int64_t n = 0; n < n_ent; ++n) order[cur[bucket[n]]++] = (int32_t)n;
    }
    // tiles: split buckets by capacity; runs of consecutive ids become ranges
    std::vector<int32_t> tile_of(n_ent), tile_local(n_ent);
    plan.tiles.clear();
    plan.ranges.clear();
    plan.emeta.clear();
    plan.eids.clear();
    for (int64_t b = 0; b < nbk; ++b) {
        int64_t k = bstart[b];
        while (k < bstart[b + 1]) {
            TileDesc t{};
            t.range_begin = (int32_t)plan.ranges.size();
            t.ent_begin = (int32_t)plan.emeta.size();
            int64_t stage = 0, map = 0, red = 0;
            int32_t ne = 0;
            const int32_t tid = (int32_t)plan.tiles.size();
            while (k < bstart[b + 1]) {
                const int64_t n = order[k];
                const int64_t st = stage_of(n), mp = (map_of(n) + 3) & ~3ll;
                if (st > opt.stage_cap || mp > opt.map_cap)
                    return fail(err, FE_ERR_UNSUPPORTED, "a dof entity's contributions exceed the tile staging capacity");
                if (ne && (stage + st > opt.stage_cap || map + mp > opt.map_cap || ne + 1 > opt.ent_cap ||
                           ne + 1 > MAX_TILE_ENTS || red + nnb_of(n) > opt.red_cap))
                    break;
                const int64_t z = (int64_t)(cp[nc * n + nc] - cp[nc * n]);
                if ((int32_t)plan.ranges.size() > t.range_begin && plan.ranges.back().ent0 + plan.ranges.back().n_ent == n) {
                    plan.ranges.back().n_ent++;
                    plan.ranges.back().nz_len += (int32_t)z;
                } else {
                    RangeDesc r{};
                    r.nz0 = cp[nc * n] - 1;
                    r.ent0 = (int32_t)n;
                    r.n_ent = 1;
                    r.nz_len = (int32_t)z;
                    plan.ranges.push_back(r);
                }
                EntMeta m;
                m.x = (int32_t)stage;
                m.y = (int32_t)map;
                m.z = (int32_t)red;
                m.w = kcount[n] | (int32_t)(nnb_of(n) << 8);
                plan.emeta.push_back(m);
                plan.eids.push_back((int32_t)n);
                tile_of[n] = tid;
                tile_local[n] = ne;
                stage += st;
                map += mp;
                red += nnb_of(n);
                ++ne;
                ++k;
            }
            t.range_end = (int32_t)plan.ranges.size();
            t.n_ent = ne;
            t.n_red = (int32_t)red;
            t.stage_vals = (int32_t)stage;
            t.map_bytes = (int32_t)map;
            plan.tiles.push_back(t);
            plan.max_stage = std::max(plan.max_stage, t.stage_vals);
            plan.max_map = std::max(plan.max_map, t.map_bytes);
            plan.max_ent = std::max(plan.max_ent, ne);
            plan.max_red = std::max(plan.max_red, t.n_red);
        }
    }
    const int64_t n_tiles = (int64_t)plan.tiles.size();
    // (sub, cell, j) triples per tile, in (sub, cell, j) order
    std::vector<int64_t> tstart(n_tiles + 1, 0);
    for (const HostSub& hs : hp.subs)
        for (size_t t = 0; t < hs.ents.size(); ++t) tstart[tile_of[hs.ents[t]] + 1]++;
    for (int64_t t = 0; t < n_tiles; ++t) tstart[t + 1] += tstart[t];
    std::vector<uint64_t> trip(tstart[n_tiles]);
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
    struct TileOut {
        std::vector<SegDesc> segs;
        std::vector<int32_t> cells, cell_items;
        std::vector<uint32_t> items, red;
        int status = 0;
    };
    std::vector<TileOut> outs(n_tiles);
#pragma omp parallel
    {
        std::vector<int32_t> kc;
#pragma omp for schedule(dynamic, 16)
        for (int64_t t = 0; t < n_tiles; ++t) {
            TileOut& o = outs[t];
            kc.assign(plan.tiles[t].n_ent, 0);
            for (int64_t q = tstart[t]; q < tstart[t + 1]; ++q) {
                const int s = (int)(trip[q] >> 40);
                const int64_t cell = (int64_t)((trip[q] >> 8) & 0xFFFFFFFFull);
                const int j = (int)(trip[q] & 0xFF);
                const bool new_cell = q == tstart[t] || (trip[q] >> 8) != (trip[q - 1] >> 8);
                if (new_cell) {
                    if (o.segs.empty() || o.segs.back().sub != s) {
                        if (!o.segs.empty()) o.segs.back().item_end = (int32_t)o.items.size();
                        SegDesc g{};
                        g.sub = s;
                        g.cell_begin = (int32_t)o.cells.size();
                        o.segs.push_back(g);
                    }
                    o.cells.push_back((int32_t)cell);
                    o.cell_items.push_back((int32_t)o.items.size());
                    o.segs.back().n_cells++;
                }
                const HostSub& hs = hp.subs[s];
                const int32_t te = tile_local[hs.ents[cell * hs.nb + j]];
                o.items.push_back(pack_item((uint32_t)j, (uint32_t)te, (uint32_t)kc[te]));
                kc[te]++;
            }
            if (!o.segs.empty()) o.segs.back().item_end = (int32_t)o.items.size();
            // reduce order: owned blocks by contribution count, most first (stable in (entity, r))
            {
                const TileDesc& T = plan.tiles[t];
                std::vector<int32_t> cnt(T.n_red, 0);
                for (int64_t q = tstart[t]; q < tstart[t + 1]; ++q) {
                    const int s = (int)(trip[q] >> 40);
                    const int64_t cell = (int64_t)((trip[q] >> 8) & 0xFFFFFFFFull);
                    const int j = (int)(trip[q] & 0xFF);
                    const HostSub& hs = hp.subs[s];
                    const int32_t te = tile_local[hs.ents[cell * hs.nb + j]];
                    const int32_t z = plan.emeta[T.ent_begin + te].z;
                    for (int i = 0; i < hs.nb; ++i) {
                        const size_t rq = ((size_t)cell * hs.nb + j) * hs.nb + i;
                        const int r = hs.wide_rank ? (hs.rank16[rq] == 0xFFFF ? -1 : hs.rank16[rq]) : (hs.rank8[rq] == 255 ? -1 : hs.rank8[rq]);
                        if (r >= 0) cnt[z + r]++;
                    }
                }
                std::vector<uint32_t> keys(T.n_red);
                for (int32_t te = 0; te < T.n_ent; ++te) {
                    const EntMeta m = plan.emeta[T.ent_begin + te];
                    for (int32_t r = 0; r < (m.w >> 8); ++r) keys[m.z + r] = ((uint32_t)te << 22) | (uint32_t)r;
                }
                std::vector<int32_t> ord(T.n_red);
                for (int32_t q = 0; q < T.n_red; ++q) ord[q] = q;
                std::stable_sort(ord.begin(), ord.end(), [&](int32_t x, int32_t y) { return cnt[x] > cnt[y]; });
                o.red.resize(T.n_red);
                for (int32_t q = 0; q < T.n_red; ++q) o.red[q] = keys[ord[q]];
            }
            // within a segment, cells with more owned base functions first: the lane groups of
            // one warp then run loops of similar length
            for (SegDesc& g : o.segs) {
                const int32_t c0 = g.cell_begin, c1 = g.cell_begin + g.n_cells;
                std::vector<int32_t> idx(g.n_cells);
                for (int32_t c = 0; c < g.n_cells; ++c) idx[c] = c0 + c;
                auto cnt = [&](int32_t c) { return (c + 1 < c1 ? o.cell_items[c + 1] : g.item_end) - o.cell_items[c]; };
                std::stable_sort(idx.begin(), idx.end(), [&](int32_t x, int32_t y) { return cnt(x) > cnt(y); });
                std::vector<int32_t> cells2, ci2;
                std::vector<uint32_t> items2;
                const int32_t ib = o.cell_items[c0];
                for (int32_t c : idx) {
                    cells2.push_back(o.cells[c]);
                    ci2.push_back(ib + (int32_t)items2.size());
                    const int32_t e0 = o.cell_items[c], e1 = c + 1 < c1 ? o.cell_items[c + 1] : g.item_end;
                    items2.insert(items2.end(), o.items.begin() + e0, o.items.begin() + e1);
                }
                std::copy(cells2.begin(), cells2.end(), o.cells.begin() + c0);
                std::copy(ci2.begin(), ci2.end(), o.cell_items.begin() + c0);
                std::copy(items2.begin(), items2.end(), o.items.begin() + ib);
            }
            for (int32_t te = 0; te < plan.tiles[t].n_ent; ++te)
                if (kc[te] != (plan.emeta[plan.tiles[t].ent_begin + te].w & 0xFF)) o.status = 1;
        }
    }
    plan.segs.clear();
    plan.tile_cells.clear();
    plan.cell_items.clear();
    plan.items.clear();
    plan.red_list.clear();
    plan.visits = 0;
    size_t ncl = 0, nit = 0;
    for (auto& o : outs) {
        if (o.status) return fail(err, FE_ERR_ARG, "internal: incident cell count mismatch");
        ncl += o.cells.size();
        nit += o.items.size();
    }
    if (nit >= (size_t)INT32_MAX || ncl >= (size_t)INT32_MAX) return fail(err, FE_ERR_UNSUPPORTED, "plan too large");
    plan.tile_cells.reserve(ncl);
    plan.cell_items.reserve(ncl);
    plan.items.reserve(nit);
    for (int64_t t = 0; t < n_tiles; ++t) {
        TileOut& o = outs[t];
        const int32_t cb = (int32_t)plan.tile_cells.size(), ib = (int32_t)plan.items.size();
        plan.tiles[t].seg_begin = (int32_t)plan.segs.size();
        for (SegDesc g : o.segs) {
            g.cell_begin += cb;
            g.item_end += ib;
            plan.segs.push_back(g);
        }
        plan.tiles[t].seg_end = (int32_t)plan.segs.size();
        for (size_t c = 0; c < o.cells.size(); ++c) {
            plan.tile_cells.push_back(o.cells[c]);
            plan.cell_items.push_back(o.cell_items[c] + ib);
        }
        plan.items.insert(plan.items.end(), o.items.begin(), o.items.end());
        plan.tiles[t].cell_begin = cb;
        plan.tiles[t].n_cells = (int32_t)o.cells.size();
        plan.tiles[t].item_begin = ib;
        plan.tiles[t].n_items = (int32_t)o.items.size();
        plan.max_items = std::max(plan.max_items, (int32_t)o.items.size());
        plan.tiles[t].red_begin = (int32_t)plan.red_list.size();
        plan.red_list.insert(plan.red_list.end(), o.red.begin(), o.red.end());
        plan.visits += (int64_t)o.cells.size();
        plan.max_cells = std::max(plan.max_cells, (int32_t)o.cells.size());
        std::vector<uint32_t>().swap(o.items);
    }
    return FE_OK;
}

// Every index the kernel derives from the plan stays inside the buffers it addresses: the
// tile staging (stage_vals), the contribution map (map_bytes), the entity table, the cell
// tables and the per-cell rank rows. Run once per fe_create; O(items * n_base).
int check_plan(const HostProblem& hp, const Plan& pl, Error& err) {
    const int nc = hp.nc;
    const int64_t* cp = hp.colptr.data();
    const int nbm = pl.nb_max;
    const int bs = (nc * nc + 1) & ~1;
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : bad)
    for (int64_t t = 0; t < (int64_t)pl.tiles.size(); ++t) {
        const TileDesc& T = pl.tiles[t];
        int64_t stage = 0, map = 0, red = 0;
        int32_t e = 0;
        for (int r = T.range_begin; r < T.range_end && !bad; ++r) {
            const RangeDesc& R = pl.ranges[r];
            if (R.nz0 != cp[(int64_t)nc * R.ent0] - 1 || R.nz_len != cp[(int64_t)nc * (R.ent0 + R.n_ent)] - cp[(int64_t)nc * R.ent0])
                bad = 1;
            for (int q = 0; q < R.n_ent && !bad; ++q, ++e) {
                const EntMeta m = pl.emeta[T.ent_begin + e];
                const int64_t n = R.ent0 + q;
                const int kcnt = m.w & 0xFF, nnb = m.w >> 8;
                if (pl.eids[T.ent_begin + e] != n || m.x != stage || m.y != map || m.z != red ||
                    nnb != (cp[nc * n + 1] - cp[nc * n]) / nc)
                    bad = 1;
                stage += ((int64_t)kcnt * (nbm * bs + nc) + 1) & ~1ll;
                map += ((int64_t)nnb * kcnt + 3) & ~3ll;
                red += nnb;
            }
        }
        if (bad || e != T.n_ent || stage != T.stage_vals || map != T.map_bytes || red != T.n_red) { bad = 1; continue; }
        {
            std::vector<char> seen(T.n_red, 0);
            for (int32_t q = 0; q < T.n_red && !bad; ++q) {
                const uint32_t key = pl.red_list[T.red_begin + q];
                const int te = (int)(key >> 22), r = (int)(key & ((1u << 22) - 1));
                if (te >= T.n_ent) { bad = 1; break; }
                const EntMeta m = pl.emeta[T.ent_begin + te];
                if (r >= (m.w >> 8) || seen[m.z + r]) { bad = 1; break; }
                seen[m.z + r] = 1;
            }
        }
        if (T.seg_end > T.seg_begin) {
            const SegDesc& G0 = pl.segs[T.seg_begin];
            const SegDesc& G1 = pl.segs[T.seg_end - 1];
            if (G0.cell_begin != T.cell_begin || G1.cell_begin + G1.n_cells != T.cell_begin + T.n_cells ||
                pl.cell_items[T.cell_begin] != T.item_begin || G1.item_end != T.item_begin + T.n_items)
                bad = 1;
        }
        for (int g = T.seg_begin; g < T.seg_end && !bad; ++g) {
            const SegDesc& G = pl.segs[g];
            if (G.sub < 0 || G.sub >= (int)hp.subs.size() || G.n_cells < 1) { bad = 1; break; }
            const HostSub& hs = hp.subs[G.sub];
            for (int c = 0; c < G.n_cells && !bad; ++c) {
                const int32_t cell = pl.tile_cells[G.cell_begin + c];
                if (cell < 0 || cell >= hs.n_cells) { bad = 1; break; }
                const int32_t i0 = pl.cell_items[G.cell_begin + c];
                const int32_t i1 = c + 1 < G.n_cells ? pl.cell_items[G.cell_begin + c + 1] : G.item_end;
                if (i1 < i0) { bad = 1; break; }
                for (int32_t it = i0; it < i1; ++it) {
                    const uint32_t w = pl.items[it];
                    const int j = (int)(w & ((1u << ITEM_J_BITS) - 1));
                    const int te = (int)((w >> ITEM_J_BITS) & ((1u << ITEM_ENT_BITS) - 1));
                    const int k = (int)(w >> (ITEM_J_BITS + ITEM_ENT_BITS));
                    if (j >= hs.nb || te >= T.n_ent || pl.eids[T.ent_begin + te] != hs.ents[(int64_t)cell * hs.nb + j]) { bad = 1; break; }
                    const EntMeta m = pl.emeta[T.ent_begin + te];
                    const int kcnt = m.w & 0xFF, nnb = m.w >> 8;
                    if (k >= kcnt) { bad = 1; break; }
                    for (int i = 0; i < hs.nb; ++i) {
                        const size_t q = ((size_t)cell * hs.nb + j) * hs.nb + i;
                        const int r = hs.wide_rank ? (hs.rank16[q] == 0xFFFF ? -1 : hs.rank16[q]) : (hs.rank8[q] == 255 ? -1 : hs.rank8[q]);
                        if (r >= nnb || m.y + (int64_t)r * kcnt + k >= T.map_bytes) { bad = 1; break; }
                    }
                    if ((int64_t)m.x + ((int64_t)k * nbm + hs.nb) * bs > T.stage_vals ||
                        (int64_t)m.x + (int64_t)kcnt * nbm * bs + (int64_t)(k + 1) * nc > T.stage_vals) { bad = 1; break; }
                }
            }
        }
    }
    if (bad) return fail(err, FE_ERR_ARG, "internal: tile plan failed its bounds check");
    return FE_OK;
}

}  // namespace fe
