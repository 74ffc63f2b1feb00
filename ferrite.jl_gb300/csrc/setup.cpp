// setup.cpp -- host-side set-up in Ferrite's numbering, for callers that do not have
// Ferrite objects at hand (Python users, the benchmark): dof distribution and the CSC
// sparsity pattern. A Julia caller passes Ferrite's own arrays instead and skips these.
//
//   fe_distribute_dofs   close!(dh) for one field (src/Dofs/DofHandler.jl:493-794): cells are
//                        visited per SubDofHandler in cellset order; a cell's vertices, then
//                        edges, then faces, then interior get n_components consecutive dofs
//                        each, reusing the dofs of entities met before. Edges are keyed by
//                        their sorted vertex pair, faces by their three smallest vertices.
//   fe_sparsity_pattern  allocate_matrix(dh) (src/Dofs/sparsity_pattern.jl:223-253): every
//                        dof pair sharing a cell, plus the diagonal, rows ascending. Built
//                        per dof entity (all components of two entities are coupled), then
//                        expanded to dofs.
#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ferrite_gb300.h"
#include "plan.h"

namespace {

// Reference-element topology: local vertex lists of edges and faces, in Ferrite's order
// (src/Grid/grid.jl:195-250). Only the cell types with edge/face dofs in this engine
// (second-order quadrilateral and hexahedron) need them.
const int HEX_EDGES[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int HEX_FACES[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};
const int QUAD_EDGES[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};

struct Key3 {
    int64_t a, b, c;
    bool operator==(const Key3& o) const { return a == o.a && b == o.b && c == o.c; }
};
struct Key3Hash {
    size_t operator()(const Key3& k) const {
        uint64_t h = (uint64_t)k.a * 0x9E3779B97F4A7C15ull;
        h ^= (uint64_t)k.b + 0x7F4A7C159E3779B9ull + (h << 6) + (h >> 2);
        h ^= (uint64_t)k.c + 0x94D049BB133111EBull + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};

}  // namespace

extern "C" {

int fe_distribute_dofs(const fe_grid_desc* grid, int32_t n_sub, const fe_subdomain_desc* subs, int64_t* cell_dofs,
                       int64_t* cell_dofs_offset, int64_t* ndofs) {
    if (!grid || !subs || n_sub < 1 || !cell_dofs || !cell_dofs_offset || !ndofs) return FE_ERR_ARG;
    std::vector<int64_t> vfirst(grid->n_nodes, 0);
    std::unordered_map<Key3, int64_t, Key3Hash> edge_first, face_first;
    for (int64_t c = 0; c < grid->n_cells; ++c) cell_dofs_offset[c] = 0;
    int64_t next = 1, len = 0;
    for (int s = 0; s < n_sub; ++s) {
        const fe_subdomain_desc& sd = subs[s];
        int32_t nb, ng, rdim;
        const int kind = fe::kind_of(sd.cell_type, sd.ip_order, nb, ng, rdim);
        if (kind < 0) return FE_ERR_UNSUPPORTED;
        const int nc = sd.n_components;
        if (nc < 1) return FE_ERR_ARG;
        edge_first.reserve(edge_first.size() + (kind == fe::KIND_HEX27 || kind == fe::KIND_QUAD9 ? 3 * sd.n_cells : 0));
        face_first.reserve(face_first.size() + (kind == fe::KIND_HEX27 ? 3 * sd.n_cells : 0));
        auto take = [&](int64_t& first) {  // dofs of one entity: reuse or create
            if (!first) {
                first = next;
                next += nc;
            }
            for (int a = 0; a < nc; ++a) cell_dofs[len++] = first + a;
        };
        for (int64_t k = 0; k < sd.n_cells; ++k) {
            const int64_t c = sd.cellset[k] - 1;
            if (c < 0 || c >= grid->n_cells) return FE_ERR_BOUNDS;
            const int64_t* v = sd.cell_nodes + k * ng;
            for (int a = 0; a < ng; ++a)
                if (v[a] < 1 || v[a] > grid->n_nodes) return FE_ERR_BOUNDS;
            cell_dofs_offset[c] = len + 1;
            for (int a = 0; a < ng; ++a) take(vfirst[v[a] - 1]);
            if (kind == fe::KIND_HEX27 || kind == fe::KIND_QUAD9) {
                const int ne = kind == fe::KIND_HEX27 ? 12 : 4;
                for (int e = 0; e < ne; ++e) {
                    const int* ed = kind == fe::KIND_HEX27 ? HEX_EDGES[e] : QUAD_EDGES[e];
                    int64_t a = v[ed[0]], b = v[ed[1]];
                    if (a > b) std::swap(a, b);
                    take(edge_first[Key3{a, b, 0}]);
                }
                if (kind == fe::KIND_HEX27) {
                    for (int f = 0; f < 6; ++f) {
                        int64_t q[4] = {v[HEX_FACES[f][0]], v[HEX_FACES[f][1]], v[HEX_FACES[f][2]], v[HEX_FACES[f][3]]};
                        std::sort(q, q + 4);
                        take(face_first[Key3{q[0], q[1], q[2]}]);
                    }
                } else {  // the quadrilateral's face is its interior: key by its 3 smallest vertices
                    int64_t q[4] = {v[0], v[1], v[2], v[3]};
                    std::sort(q, q + 4);
                    take(face_first[Key3{q[0], q[1], q[2]}]);
                }
                if (kind == fe::KIND_HEX27) {
                    int64_t fresh = 0;
                    take(fresh);
                }
            }
        }
    }
    *ndofs = next - 1;
    return FE_OK;
}

int fe_sparsity_pattern(const fe_grid_desc* grid, int32_t n_sub, const fe_subdomain_desc* subs, const fe_dof_desc* dofs,
                        int64_t* colptr, int64_t* rowval, int64_t* nnz) {
    if (!grid || !subs || !dofs || !colptr || !nnz || n_sub < 1) return FE_ERR_ARG;
    const int nc = subs[0].n_components;
    const int64_t nd = dofs->ndofs;
    if (nc < 1 || nd % nc) return FE_ERR_UNSUPPORTED;
    const int64_t ne = nd / nc;
    // cell entity lists and entity -> cells
    struct CellRef { int32_t sub; int64_t k; int nb; };
    std::vector<int64_t> eptr(ne + 1, 0);
    std::vector<std::vector<int32_t>> cell_ents(n_sub);
    for (int s = 0; s < n_sub; ++s) {
        const fe_subdomain_desc& sd = subs[s];
        if (sd.n_components != nc) return FE_ERR_UNSUPPORTED;
        int32_t nb, ng, rdim;
        if (fe::kind_of(sd.cell_type, sd.ip_order, nb, ng, rdim) < 0) return FE_ERR_UNSUPPORTED;
        cell_ents[s].resize(sd.n_cells * nb);
        for (int64_t k = 0; k < sd.n_cells; ++k) {
            const int64_t c = sd.cellset[k] - 1;
            const int64_t* cd = dofs->cell_dofs + dofs->cell_dofs_offset[c] - 1;
            for (int i = 0; i < nb; ++i) {
                const int64_t d = cd[i * nc];
                if (d < 1 || d > nd || (d - 1) % nc) return FE_ERR_UNSUPPORTED;
                const int32_t e = (int32_t)((d - 1) / nc);
                cell_ents[s][k * nb + i] = e;
                eptr[e + 1]++;
            }
        }
    }
    for (int64_t e = 0; e < ne; ++e) eptr[e + 1] += eptr[e];
    std::vector<std::pair<int32_t, int64_t>> ecells(eptr[ne]);
    {
        std::vector<int64_t> cur(eptr.begin(), eptr.end() - 1);
        for (int s = 0; s < n_sub; ++s) {
            const int64_t n = subs[s].n_cells;
            const int nb = (int)(cell_ents[s].size() / std::max<int64_t>(n, 1));
            for (int64_t k = 0; k < n; ++k)
                for (int i = 0; i < nb; ++i) ecells[cur[cell_ents[s][k * nb + i]]++] = {s, k};
        }
    }
    std::vector<int32_t> nnb(ne);  // neighbour entities per entity
    auto neighbours = [&](int64_t e, std::vector<int32_t>& buf) {
        buf.clear();
        buf.push_back((int32_t)e);
        for (int64_t t = eptr[e]; t < eptr[e + 1]; ++t) {
            const int s = ecells[t].first;
            const int64_t k = ecells[t].second;
            const int nb = (int)(cell_ents[s].size() / subs[s].n_cells);
            buf.insert(buf.end(), cell_ents[s].begin() + k * nb, cell_ents[s].begin() + (k + 1) * nb);
        }
        std::sort(buf.begin(), buf.end());
        buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
    };
#pragma omp parallel
    {
        std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 4096)
        for (int64_t e = 0; e < ne; ++e) {
            neighbours(e, buf);
            nnb[e] = (int32_t)buf.size();
        }
    }
    colptr[0] = 1;
    for (int64_t e = 0; e < ne; ++e)
        for (int b = 0; b < nc; ++b) colptr[e * nc + b + 1] = colptr[e * nc + b] + (int64_t)nnb[e] * nc;
    *nnz = colptr[nd] - 1;
    if (!rowval) return FE_OK;
#pragma omp parallel
    {
        std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 4096)
        for (int64_t e = 0; e < ne; ++e) {
            neighbours(e, buf);
            int64_t* out = rowval + colptr[e * nc] - 1;
            const size_t L = buf.size() * nc;
            for (size_t t = 0; t < buf.size(); ++t)
                for (int a = 0; a < nc; ++a) out[t * nc + a] = (int64_t)buf[t] * nc + a + 1;
            for (int b = 1; b < nc; ++b) std::memcpy(out + b * L, out, L * sizeof(int64_t));
        }
    }
    return FE_OK;
}

}  // extern "C"
