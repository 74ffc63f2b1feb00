// Host planner under AddressSanitizer / UndefinedBehaviorSanitizer (built and run by
// tests/test_planner_sanitize.py): a perturbed hexahedron grid, dofs and pattern from the
// library's own host set-up (fe_distribute_dofs, fe_sparsity_pattern), then validation, the
// owner-tile plan and the record check (build_problem, build_plan, check_plan).
#include <cstdio>
#include <cstring>
#include <vector>
#include <cmath>
#include "plan.h"
using namespace fe;
extern "C" int fe_distribute_dofs(const fe_grid_desc*, int32_t, const fe_subdomain_desc*, int64_t*, int64_t*, int64_t*);
extern "C" int fe_sparsity_pattern(const fe_grid_desc*, int32_t, const fe_subdomain_desc*, const fe_dof_desc*, int64_t*, int64_t*, int64_t*);
int main(int argc, char** argv) {
    int n = argc > 1 ? atoi(argv[1]) : 12, nc = argc > 2 ? atoi(argv[2]) : 3;
    int nx = n, ny = n - 1, nz = n - 2;
    std::vector<double> nodes;
    for (int k = 0; k <= nz; ++k) for (int j = 0; j <= ny; ++j) for (int i = 0; i <= nx; ++i) {
        double x = i / (double)nx, y = j / (double)ny, z = k / (double)nz;
        if (i > 0 && i < nx && j > 0 && j < ny && k > 0 && k < nz) { x += 0.1 / nx * std::sin(7.0 * (i + 3 * j + 5 * k)); }
        nodes.push_back(x); nodes.push_back(y); nodes.push_back(z);
    }
    auto nid = [&](int i, int j, int k) { return (int64_t)(k * (ny + 1) + j) * (nx + 1) + i + 1; };
    std::vector<int64_t> cells, cellset;
    int64_t c = 0;
    for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) {
        int64_t v[8] = {nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                        nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)};
        for (int a = 0; a < 8; ++a) cells.push_back(v[a]);
        cellset.push_back(++c);
    }
    // 2x2x2 Gauss tables for the trilinear hexahedron
    const double g = 1.0 / std::sqrt(3.0);
    double xi[8][3]; int q = 0;
    for (int kk = 0; kk < 2; ++kk) for (int jj = 0; jj < 2; ++jj) for (int ii = 0; ii < 2; ++ii) { xi[q][0] = ii ? g : -g; xi[q][1] = jj ? g : -g; xi[q][2] = kk ? g : -g; ++q; }
    const int s[8][3] = {{-1,-1,-1},{1,-1,-1},{1,1,-1},{-1,1,-1},{-1,-1,1},{1,-1,1},{1,1,1},{-1,1,1}};
    std::vector<double> w(8, 1.0), N(64), dN(192);
    for (int p = 0; p < 8; ++p) for (int a = 0; a < 8; ++a) {
        double f[3]; for (int d = 0; d < 3; ++d) f[d] = 0.5 * (1 + s[a][d] * xi[p][d]);
        N[p * 8 + a] = f[0] * f[1] * f[2];
        dN[(p * 8 + a) * 3 + 0] = 0.5 * s[a][0] * f[1] * f[2];
        dN[(p * 8 + a) * 3 + 1] = 0.5 * s[a][1] * f[0] * f[2];
        dN[(p * 8 + a) * 3 + 2] = 0.5 * s[a][2] * f[0] * f[1];
    }
    fe_grid_desc gd{3, (int64_t)nodes.size() / 3, nodes.data(), c};
    fe_subdomain_desc sd{};
    sd.cell_type = FE_HEXAHEDRON; sd.ip_order = 1; sd.n_components = nc; sd.n_qp = 8;
    sd.qr_weights = w.data(); sd.N = N.data(); sd.dNdxi = dN.data(); sd.M = N.data(); sd.dMdxi = dN.data();
    sd.n_cells = c; sd.cellset = cellset.data(); sd.cell_nodes = cells.data();
    std::vector<int64_t> cd(c * 8 * nc), off(c);
    int64_t ndofs = 0;
    int rc = fe_distribute_dofs(&gd, 1, &sd, cd.data(), off.data(), &ndofs);
    if (rc) { printf("dofs rc %d\n", rc); return 1; }
    fe_dof_desc dd{ndofs, cd.data(), off.data()};
    std::vector<int64_t> cp(ndofs + 1);
    int64_t nnz = 0;
    rc = fe_sparsity_pattern(&gd, 1, &sd, &dd, cp.data(), nullptr, &nnz);
    std::vector<int64_t> rv(nnz);
    rc |= fe_sparsity_pattern(&gd, 1, &sd, &dd, cp.data(), rv.data(), &nnz);
    if (rc) { printf("pattern rc %d\n", rc); return 1; }
    fe_csc_desc pd{ndofs, nnz, cp.data(), rv.data()};
    CreateInput in{&gd, 1, &sd, &dd, &pd};
    HostProblem hp; Plan pl; Error err; PlanOptions opt;
    if (argc > 3) opt.stage_cap = atoi(argv[3]);
    rc = build_problem(in, hp, err);
    if (!rc) rc = build_plan(hp, opt, pl, err);
    if (!rc) rc = check_plan(hp, pl, err);
    printf("n=%d nc=%d cells=%lld ndofs=%lld nnz=%lld rc=%d tiles=%lld msg=%s\n", n, nc, (long long)c, (long long)ndofs,
           (long long)nnz, rc, (long long)pl.n_tiles, err.msg.c_str());
    if (rc) return rc;
    // the record check rejects a corrupted record: a range's nzval start, a node id, the size
    int rejected = 0;
    for (int kind = 0; kind < 3; ++kind) {
        Plan bad = pl;
        uint8_t* B = bad.rec.data() + bad.rec_off[pl.n_tiles / 2];
        RecHead H;
        std::memcpy(&H, B, sizeof H);
        if (kind == 0 && H.n_rng > 0) {
            RecRng R;
            std::memcpy(&R, B + H.off_rng, sizeof R);
            R.nz0 += 2;  // keeps the parity of buf_off - nz0, so only the mapping check can see it
            std::memcpy(B + H.off_rng, &R, sizeof R);
        } else if (kind == 1 && H.n_nodes > 0) {
            const int32_t v = (int32_t)hp.n_nodes;
            std::memcpy(B + H.off_nodes, &v, sizeof v);
        } else if (kind == 2) {
            H.bytes += 16;
            std::memcpy(B, &H, sizeof H);
        }
        Error e2;
        if (check_plan(hp, bad, e2) != 0) ++rejected;
    }
    printf("corrupted records rejected: %d of 3\n", rejected);
    return rejected == 3 ? 0 : 3;
}
