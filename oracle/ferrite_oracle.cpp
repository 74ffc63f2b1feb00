// ferrite_oracle.cpp -- CPU FP64 restatement of Ferrite.jl's assembly path.
//
// TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA engine and the timed CPU
// baseline. The product library never links or calls it. Each function cites the Ferrite.jl
// (v1.6.0) source it follows; see ferrite_oracle.h for the overall map.
//
// Build (no cmake): g++ -O2 -fopenmp -ffp-contract=off -fPIC -shared ferrite_oracle.cpp
// -ffp-contract=off keeps a*b+c as two roundings, as Julia evaluates it without @fastmath.
#include "ferrite_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------------------
// Reference shapes: vertices, edges, faces (src/Grid/grid.jl:195-250)
// ---------------------------------------------------------------------------------------
struct RefTopo {
    int nvert;
    int rdim;
    std::vector<std::vector<int>> edges;  // 1-based local vertex ids
    std::vector<std::vector<int>> faces;
};

const RefTopo& ref_topo(int ct) {
    static const RefTopo tri{3, 2, {{1, 2}, {2, 3}, {3, 1}}, {{1, 2, 3}}};
    static const RefTopo quad{4, 2, {{1, 2}, {2, 3}, {3, 4}, {4, 1}}, {{1, 2, 3, 4}}};
    static const RefTopo tet{4, 3, {{1, 2}, {2, 3}, {3, 1}, {1, 4}, {2, 4}, {3, 4}},
                             {{1, 3, 2}, {1, 2, 4}, {2, 3, 4}, {1, 4, 3}}};
    static const RefTopo hex{8, 3,
                             {{1, 2}, {2, 3}, {3, 4}, {4, 1}, {5, 6}, {6, 7},
                              {7, 8}, {8, 5}, {1, 5}, {2, 6}, {3, 7}, {4, 8}},
                             {{1, 4, 3, 2}, {1, 2, 6, 5}, {2, 3, 7, 6},
                              {3, 4, 8, 7}, {1, 5, 8, 4}, {5, 6, 7, 8}}};
    static const RefTopo wedge{6, 3,
                               {{2, 1}, {1, 3}, {1, 4}, {3, 2}, {2, 5}, {3, 6}, {4, 5}, {4, 6}, {6, 5}},
                               {{1, 3, 2}, {1, 2, 5, 4}, {3, 1, 4, 6}, {2, 3, 6, 5}, {4, 5, 6}}};
    switch (ct) {
        case OR_TRIANGLE: return tri;
        case OR_QUADRILATERAL: return quad;
        case OR_TETRAHEDRON: return tet;
        case OR_HEXAHEDRON: return hex;
        default: return wedge;
    }
}

int ref_dim(int ct) { return (ct == OR_TRIANGLE || ct == OR_QUADRILATERAL) ? 2 : 3; }

// Number of Lagrange base functions; the supported (shape, order) pairs.
int nbase(int ct, int order) {
    if (order == 1) return ref_topo(ct).nvert;
    if (order == 2 && ct == OR_HEXAHEDRON) return 27;
    if (order == 2 && ct == OR_QUADRILATERAL) return 9;
    return -1;
}

// ---------------------------------------------------------------------------------------
// Shape functions (src/interpolations.jl). Gradients are the analytic derivatives of the
// listed polynomials; Ferrite takes them by forward-mode AD (interpolations.jl:280-292),
// which gives the same values up to rounding.
// ---------------------------------------------------------------------------------------
// Q2 hexahedron: node i -> (ix, iy, iz) in {1: phi1, 2: phi2, 3: phi3}, interpolations.jl:1118-1164
const int Q2HEX_IDX[27][3] = {
    {1, 1, 1}, {3, 1, 1}, {3, 3, 1}, {1, 3, 1}, {1, 1, 3}, {3, 1, 3}, {3, 3, 3}, {1, 3, 3},
    {2, 1, 1}, {3, 2, 1}, {2, 3, 1}, {1, 2, 1}, {2, 1, 3}, {3, 2, 3}, {2, 3, 3}, {1, 2, 3},
    {1, 1, 2}, {3, 1, 2}, {3, 3, 2}, {1, 3, 2},
    {2, 2, 1}, {2, 1, 2}, {3, 2, 2}, {2, 3, 2}, {1, 2, 2}, {2, 2, 3},
    {2, 2, 2}};
// Q2 quadrilateral: interpolations.jl (RefQuadrilateral order 2), same phi convention
const int Q2QUAD_IDX[9][2] = {{1, 1}, {3, 1}, {3, 3}, {1, 3}, {2, 1}, {3, 2}, {2, 3}, {1, 2}, {2, 2}};

inline double phi(int k, double x) {
    if (k == 1) return -x * (1 - x) / 2;
    if (k == 2) return (1 + x) * (1 - x);
    return x * (1 + x) / 2;
}
inline double dphi(int k, double x) {
    if (k == 1) return x - 0.5;
    if (k == 2) return -2 * x;
    return x + 0.5;
}

// Value and reference gradient of base function i (0-based) at xi.
void shape_value_grad(int ct, int order, int i, const double* xi, double& N, double* dN) {
    const double x = xi[0], y = xi[1], z = ref_dim(ct) == 3 ? xi[2] : 0.0;
    dN[0] = dN[1] = 0;
    if (ref_dim(ct) == 3) dN[2] = 0;
    if (ct == OR_QUADRILATERAL && order == 1) {  // interpolations.jl:640-661
        const double sx[4] = {-1, 1, 1, -1}, sy[4] = {-1, -1, 1, 1};
        N = (1 + sx[i] * x) * (1 + sy[i] * y) / 4;
        dN[0] = sx[i] * (1 + sy[i] * y) / 4;
        dN[1] = (1 + sx[i] * x) * sy[i] / 4;
    } else if (ct == OR_QUADRILATERAL && order == 2) {
        const int a = Q2QUAD_IDX[i][0], b = Q2QUAD_IDX[i][1];
        N = phi(a, x) * phi(b, y);
        dN[0] = dphi(a, x) * phi(b, y);
        dN[1] = phi(a, x) * dphi(b, y);
    } else if (ct == OR_HEXAHEDRON && order == 1) {  // interpolations.jl:1054-1064
        const double sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
                     sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
        N = (1 + sx[i] * x) * (1 + sy[i] * y) * (1 + sz[i] * z) / 8;
        dN[0] = sx[i] * (1 + sy[i] * y) * (1 + sz[i] * z) / 8;
        dN[1] = (1 + sx[i] * x) * sy[i] * (1 + sz[i] * z) / 8;
        dN[2] = (1 + sx[i] * x) * (1 + sy[i] * y) * sz[i] / 8;
    } else if (ct == OR_HEXAHEDRON && order == 2) {  // interpolations.jl:1126-1164
        const int a = Q2HEX_IDX[i][0], b = Q2HEX_IDX[i][1], c = Q2HEX_IDX[i][2];
        N = phi(a, x) * phi(b, y) * phi(c, z);
        dN[0] = dphi(a, x) * phi(b, y) * phi(c, z);
        dN[1] = phi(a, x) * dphi(b, y) * phi(c, z);
        dN[2] = phi(a, x) * phi(b, y) * dphi(c, z);
    } else if (ct == OR_TETRAHEDRON) {  // interpolations.jl:904-913
        const double v[4] = {1 - x - y - z, x, y, z};
        const double g[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        N = v[i];
        dN[0] = g[i][0]; dN[1] = g[i][1]; dN[2] = g[i][2];
    } else if (ct == OR_TRIANGLE) {  // Lagrange{RefTriangle,1}: N1 = x, N2 = y, N3 = 1 - x - y
        const double v[3] = {x, y, 1 - x - y};
        const double g[3][2] = {{1, 0}, {0, 1}, {-1, -1}};
        N = v[i];
        dN[0] = g[i][0]; dN[1] = g[i][1];
    } else {  // OR_WEDGE, interpolations.jl:1271-1280
        switch (i) {
            case 0: N = 1 - x - y - z * (1 - x - y); dN[0] = -1 + z; dN[1] = -1 + z; dN[2] = -(1 - x - y); break;
            case 1: N = x * (1 - z); dN[0] = 1 - z; dN[2] = -x; break;
            case 2: N = y * (1 - z); dN[1] = 1 - z; dN[2] = -y; break;
            case 3: N = z * (1 - x - y); dN[0] = -z; dN[1] = -z; dN[2] = 1 - x - y; break;
            case 4: N = x * z; dN[0] = z; dN[2] = x; break;
            default: N = y * z; dN[1] = z; dN[2] = y; break;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Quadrature (src/Quadrature/quadrature.jl:83-154)
// ---------------------------------------------------------------------------------------
// Gauss-Legendre points ascending, by Newton iteration on P_n in long double. Ferrite uses
// Golub-Welsch (generate_quadrature.jl:93-112); both give the rule to within an ulp.
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (int k = 0; k < n; ++k) {
        long double t = -cosl(3.14159265358979323846264338327950288L * (k + 0.75L) / (n + 0.5L));
        long double dp = 0;
        for (int it = 0; it < 100; ++it) {
            long double p0 = 1, p1 = t;
            for (int m = 2; m <= n; ++m) {
                long double p2 = ((2 * m - 1) * t * p1 - (m - 1) * p0) / m;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p1 = t; p0 = 1; }
            dp = n * (t * p1 - p0) / (t * t - 1);
            long double dt = p1 / dp;
            t -= dt;
            if (fabsl(dt) < 1e-19L) break;
        }
        long double p0 = 1, p1 = t;
        for (int m = 2; m <= n; ++m) {
            long double p2 = ((2 * m - 1) * t * p1 - (m - 1) * p0) / m;
            p0 = p1;
            p1 = p2;
        }
        if (n == 1) p0 = 1;
        dp = n * (t * p1 - p0) / (t * t - 1);
        if (n == 1) { t = 0; dp = 1; }
        x[k] = (double)t;
        w[k] = (double)(2.0L / ((1 - t * t) * dp * dp));
    }
}

int quadrature(int ct, int order, std::vector<double>& wts, std::vector<double>& pts) {
    wts.clear();
    pts.clear();
    const int rd = ref_dim(ct);
    if (ct == OR_QUADRILATERAL || ct == OR_HEXAHEDRON) {
        // tensor rule; xi_1 varies fastest, weight = product (quadrature.jl:93-107)
        std::vector<double> p, w;
        gauss_legendre(order, p, w);
        const int n = order;
        const int total = rd == 2 ? n * n : n * n * n;
        for (int c = 0; c < total; ++c) {
            int i1 = c % n, i2 = (c / n) % n, i3 = c / (n * n);
            double weight = 1.0;
            weight *= w[i1];
            weight *= w[i2];
            if (rd == 3) weight *= w[i3];
            wts.push_back(weight);
            pts.push_back(p[i1]);
            pts.push_back(p[i2]);
            if (rd == 3) pts.push_back(p[i3]);
        }
        return OR_OK;
    }
    if (ct == OR_TETRAHEDRON) {  // Keast minimal == Jinyun for orders 1-3 (gaussquad_tet_table.jl)
        if (order == 1) {
            wts = {1.0 / 6.0};
            pts = {0.25, 0.25, 0.25};
        } else if (order == 2) {
            const double a = (5.0 + 3.0 * std::sqrt(5.0)) / 20.0, b = (5.0 - std::sqrt(5.0)) / 20.0;
            wts = {1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0};
            pts = {a, b, b, b, a, b, b, b, a, b, b, b};
        } else if (order == 3) {
            const double a1 = 0.25, a2 = 0.5, b2 = 1.0 / 6.0;
            wts = {-2.0 / 15.0, 3.0 / 40.0, 3.0 / 40.0, 3.0 / 40.0, 3.0 / 40.0};
            pts = {a1, a1, a1, a2, b2, b2, b2, a2, b2, b2, b2, a2, b2, b2, b2};
        } else {
            return OR_ERR_UNSUPPORTED;
        }
        return OR_OK;
    }
    if (ct == OR_TRIANGLE) {  // Dunavant order 1 and 2
        if (order == 1) {
            wts = {0.5};
            pts = {1.0 / 3.0, 1.0 / 3.0};
        } else if (order == 2) {
            wts = {1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0};
            pts = {2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0};
        } else {
            return OR_ERR_UNSUPPORTED;
        }
        return OR_OK;
    }
    // OR_WEDGE: Witherden-Vincent polyquad rules on [-1,1]^3 mapped to [0,1]^3
    // (gaussquad_prism_table.jl:6-16, transform 352-364)
    std::vector<double> xw;
    if (order == 1) {
        wts = {0.5};
        pts = {1.0 / 3.0, 1.0 / 3.0, 0.5};
        return OR_OK;
    } else if (order == 2) {
        const double t = -0.33333333333333333333333333333333333333;
        const double zz = 0.99999999999999985119303811076522004183;
        const double w1 = 0.66666666666666686507594918564641756458;
        const double a = -0.74158162379719638007464124598498266439;
        const double b = 0.48316324759439276014928249196996532878;
        const double w2 = 0.88888888888888875661603387623572162361;
        xw = {t, t, -zz, w1, t, t, zz, w1, a, b, 0.0, w2, b, a, 0.0, w2, a, a, 0.0, w2};
    } else {
        return OR_ERR_UNSUPPORTED;
    }
    for (size_t r = 0; r < xw.size() / 4; ++r) {
        double px = xw[4 * r + 0], py = xw[4 * r + 1], pz = xw[4 * r + 2], pw = xw[4 * r + 3];
        px += 1.0; px /= 2.0;
        py += 1.0; py /= 2.0;
        pz += 1.0; pz /= 2.0;
        pw /= 8.0;
        pts.push_back(px);
        pts.push_back(py);
        pts.push_back(pz);
        wts.push_back(pw);
    }
    return OR_OK;
}

// ---------------------------------------------------------------------------------------
// Small tensor helpers (Tensors.jl semantics for det/inv of 2x2 and 3x3)
// ---------------------------------------------------------------------------------------
double det_n(int d, const double* J) {
    if (d == 2) return J[0] * J[3] - J[1] * J[2];
    return J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
           J[2] * (J[3] * J[7] - J[4] * J[6]);
}
void inv_n(int d, const double* J, double dt, double* Ji) {
    if (d == 2) {
        Ji[0] = J[3] / dt; Ji[1] = -J[1] / dt;
        Ji[2] = -J[2] / dt; Ji[3] = J[0] / dt;
        return;
    }
    Ji[0] = (J[4] * J[8] - J[5] * J[7]) / dt;
    Ji[1] = -(J[1] * J[8] - J[2] * J[7]) / dt;
    Ji[2] = (J[1] * J[5] - J[2] * J[4]) / dt;
    Ji[3] = -(J[3] * J[8] - J[5] * J[6]) / dt;
    Ji[4] = (J[0] * J[8] - J[2] * J[6]) / dt;
    Ji[5] = -(J[0] * J[5] - J[2] * J[3]) / dt;
    Ji[6] = (J[3] * J[7] - J[4] * J[6]) / dt;
    Ji[7] = -(J[0] * J[7] - J[1] * J[6]) / dt;
    Ji[8] = (J[0] * J[4] - J[1] * J[3]) / dt;
}

// ---------------------------------------------------------------------------------------
// CellValues for one (cell type, interpolation order, quadrature order) combination
// (src/FEValues/CellValues.jl:57-140)
// ---------------------------------------------------------------------------------------
struct CellValues {
    int ct = 0, order = 0, dim = 0, nq = 0, nb = 0, ng = 0;
    std::vector<double> w;          // [nq]
    std::vector<double> N, dNdxi;   // [nq][nb], [nq][nb][dim]
    std::vector<double> M, dMdxi;   // geometry [nq][ng], [nq][ng][dim]
    // per-reinit values
    std::vector<double> dNdx, detJdV;

    int init(int ct_, int order_, int qorder) {
        ct = ct_; order = order_; dim = ref_dim(ct);
        std::vector<double> pts;
        int rc = quadrature(ct, qorder, w, pts);
        if (rc) return rc;
        nq = (int)w.size();
        nb = nbase(ct, order);
        ng = nbase(ct, 1);
        if (nb < 0) return OR_ERR_UNSUPPORTED;
        N.assign(nq * nb, 0); dNdxi.assign(nq * nb * dim, 0);
        M.assign(nq * ng, 0); dMdxi.assign(nq * ng * dim, 0);
        for (int q = 0; q < nq; ++q) {
            for (int i = 0; i < nb; ++i)
                shape_value_grad(ct, order, i, &pts[q * dim], N[q * nb + i], &dNdxi[(q * nb + i) * dim]);
            for (int i = 0; i < ng; ++i)
                shape_value_grad(ct, 1, i, &pts[q * dim], M[q * ng + i], &dMdxi[(q * ng + i) * dim]);
        }
        dNdx.assign(nq * nb * dim, 0);
        detJdV.assign(nq, 0);
        return OR_OK;
    }

    // reinit!(cv, x): CellValues.jl:122-140; returns OR_ERR_DETJ with the offending detJ.
    int reinit(const double* x, double* bad_detJ) {
        double J[9], Ji[9];
        for (int q = 0; q < nq; ++q) {
            // calculate_mapping: J = sum_j x_j (x) dMdxi[j,q] (GeometryMapping.jl:124-130)
            for (int a = 0; a < dim * dim; ++a) J[a] = 0.0;
            for (int k = 0; k < ng; ++k)
                for (int a = 0; a < dim; ++a)
                    for (int b = 0; b < dim; ++b) J[a * dim + b] += x[k * dim + a] * dMdxi[(q * ng + k) * dim + b];
            const double dt = det_n(dim, J);
            if (!(dt > 0.0)) {  // _update_detJdV!, CellValues.jl:110-115
                *bad_detJ = dt;
                return OR_ERR_DETJ;
            }
            detJdV[q] = dt * w[q];
            inv_n(dim, J, dt, Ji);
            // apply_mapping!: dNdx = dNdxi . Jinv (FunctionValues.jl:186-192)
            for (int i = 0; i < nb; ++i)
                for (int b = 0; b < dim; ++b) {
                    double s = 0.0;
                    for (int a = 0; a < dim; ++a) s += dNdxi[(q * nb + i) * dim + a] * Ji[a * dim + b];
                    dNdx[(q * nb + i) * dim + b] = s;
                }
        }
        return OR_OK;
    }
};

// ---------------------------------------------------------------------------------------
// Neo-Hooke constitutive driver (hyperelasticity.jl:157-176) in closed form.
// S = mu (I - C^-1) + lambda (J-1) J C^-1, dS/dC from the same potential.
// Returns P = F S and A = dP/dF (A[i][J][k][L], row-major 3x3x3x3).
// ---------------------------------------------------------------------------------------
void neo_hooke(double mu, double lam, const double* F, double* P, double* A) {
    double C[9];
    for (int I = 0; I < 3; ++I)
        for (int J = 0; J < 3; ++J) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += F[k * 3 + I] * F[k * 3 + J];
            C[I * 3 + J] = s;
        }
    const double detC = det_n(3, C);
    double Ci[9];
    inv_n(3, C, detC, Ci);
    const double Jd = std::sqrt(detC);
    double S[9];
    for (int I = 0; I < 3; ++I)
        for (int J = 0; J < 3; ++J)
            S[I * 3 + J] = mu * ((I == J ? 1.0 : 0.0) - Ci[I * 3 + J]) + lam * (Jd - 1) * Jd * Ci[I * 3 + J];
    // dS/dC_IJKL = c1 * 1/2 (Ci_IK Ci_JL + Ci_IL Ci_JK) + c2 * Ci_IJ Ci_KL
    const double c1 = mu - lam * (Jd - 1) * Jd;
    const double c2 = lam * (2 * Jd - 1) * Jd / 2;
    double dS[81];
    for (int I = 0; I < 3; ++I)
        for (int J = 0; J < 3; ++J)
            for (int K = 0; K < 3; ++K)
                for (int L = 0; L < 3; ++L)
                    dS[((I * 3 + J) * 3 + K) * 3 + L] =
                        c1 * 0.5 * (Ci[I * 3 + K] * Ci[J * 3 + L] + Ci[I * 3 + L] * Ci[J * 3 + K]) +
                        c2 * Ci[I * 3 + J] * Ci[K * 3 + L];
    for (int i = 0; i < 3; ++i)
        for (int J = 0; J < 3; ++J) {
            double s = 0;
            for (int I = 0; I < 3; ++I) s += F[i * 3 + I] * S[I * 3 + J];
            P[i * 3 + J] = s;
        }
    // dP/dF_iJkL = delta_ik S_JL + 2 sum_IK F_iI dS_IJKL F_kK  (hyperelasticity.jl:254)
    for (int i = 0; i < 3; ++i)
        for (int J = 0; J < 3; ++J)
            for (int k = 0; k < 3; ++k)
                for (int L = 0; L < 3; ++L) {
                    double s = 0;
                    for (int I = 0; I < 3; ++I)
                        for (int K = 0; K < 3; ++K) s += F[i * 3 + I] * dS[((I * 3 + J) * 3 + K) * 3 + L] * F[k * 3 + K];
                    A[((i * 3 + J) * 3 + k) * 3 + L] = (i == k ? S[J * 3 + L] : 0.0) + 2 * s;
                }
}

// ---------------------------------------------------------------------------------------
// Problem view helpers
// ---------------------------------------------------------------------------------------
struct Setup {
    const or_problem* p;
    std::vector<int> cell_sdh;              // [n_cells], -1 if none
    std::vector<CellValues> cvs;            // per sdh
    std::vector<int> ndpc;                  // dofs per cell, per sdh

    int init(const or_problem* p_) {
        p = p_;
        cell_sdh.assign(p->n_cells, -1);
        cvs.resize(p->n_sdh);
        ndpc.resize(p->n_sdh);
        for (int s = 0; s < p->n_sdh; ++s) {
            const int64_t b = p->sdh_cellset_offset[s], e = p->sdh_cellset_offset[s + 1];
            if (e <= b) return OR_ERR_ARG;
            for (int64_t k = b; k < e; ++k) {
                const int64_t c = p->sdh_cellset[k] - 1;
                if (c < 0 || c >= p->n_cells) return OR_ERR_BOUNDS;
                cell_sdh[c] = s;
            }
            const int ct = p->cell_types[p->sdh_cellset[b] - 1];
            const int qo = p->sdh_qr_order ? p->sdh_qr_order[s] : 2;
            int rc = cvs[s].init(ct, p->sdh_ip_order[s], qo);
            if (rc) return rc;
            ndpc[s] = cvs[s].nb * p->sdh_ncomp[s];
        }
        return OR_OK;
    }
};

// ---------------------------------------------------------------------------------------
// CSC assembler (src/assembler.jl:347-457): sorted dofs, then per column a merge walk,
// binary search when the column is long, or the dense fast path. Exact zeros are skipped;
// a non-zero value without a pattern entry is an error.
// ---------------------------------------------------------------------------------------
const int SPARSE_COLUMN_SEARCH_RATIO = 8;  // assembler.jl:374

struct CSCView {
    int64_t n;
    const int64_t* colptr;
    const int64_t* rowval;
};

// Calls visit(R0, kerow, kecol) for every (row, col) of the element, with R0 the 0-based
// nzval index (or -1 if missing). Returns OR_ERR_PATTERN_MISSING via miss() callback.
template <class Visit, class Miss>
void merge_walk(const CSCView& K, const int64_t* dofs, int ld, std::vector<int64_t>& sorted,
                std::vector<int>& perm, Visit visit, Miss miss) {
    sorted.assign(dofs, dofs + ld);
    perm.resize(ld);
    for (int i = 0; i < ld; ++i) perm[i] = i;
    std::sort(perm.begin(), perm.end(), [&](int a, int b) {
        return dofs[a] < dofs[b] || (dofs[a] == dofs[b] && a < b);
    });
    for (int i = 0; i < ld; ++i) sorted[i] = dofs[perm[i]];
    for (int cc = 0; cc < ld; ++cc) {
        const int64_t Kcol = sorted[cc];
        const int kecol = perm[cc];
        const int64_t lo0 = K.colptr[Kcol - 1] - 1, hi0 = K.colptr[Kcol] - 2;  // 0-based inclusive
        const int64_t len = hi0 - lo0 + 1;
        if (len == K.n) {  // dense column
            for (int ri = 0; ri < ld; ++ri) visit(lo0 + sorted[ri] - 1, perm[ri], kecol);
            continue;
        }
        if (len > (int64_t)SPARSE_COLUMN_SEARCH_RATIO * ld) {  // binary search path
            int64_t lo = lo0;
            for (int ri = 0; ri < ld; ++ri) {
                const int64_t d = sorted[ri];
                const int64_t* first = std::lower_bound(K.rowval + lo, K.rowval + hi0 + 1, d);
                const int64_t R = first - K.rowval;
                if (R <= hi0 && K.rowval[R] == d) {
                    visit(R, perm[ri], kecol);
                    lo = R + 1;
                } else {
                    miss(d, Kcol, perm[ri], kecol);
                    lo = R;
                }
            }
            continue;
        }
        int ri = 0;
        int64_t Ri = 0;
        while (Ri < len && ri < ld) {
            const int64_t R = lo0 + Ri;
            const int64_t Krow = K.rowval[R];
            const int64_t d = sorted[ri];
            if (Krow == d) {
                visit(R, perm[ri], kecol);
                ++ri;
                ++Ri;
            } else if (Krow < d) {
                ++Ri;
            } else {
                miss(d, Kcol, perm[ri], kecol);
                ++ri;
            }
        }
        for (int i = ri; i < ld; ++i) miss(sorted[i], Kcol, perm[i], kecol);
    }
}

// Element routine for one cell: fills Ke (ld x ld, column-major like Julia) and fe.
int element(const Setup& S, CellValues& cv, int sdh, int64_t c, const or_physics* ph, double* Ke,
            double* fe, std::vector<double>& x, std::vector<double>& ue, or_error* err) {
    const or_problem* p = S.p;
    const int dim = cv.dim;
    const int nc = p->sdh_ncomp[sdh];
    const int nb = cv.nb, ng = cv.ng, ld = nb * nc;
    // CellCache reinit: coordinates of the geometric nodes (iterators.jl:72-87, grid.jl:612-624)
    const int64_t off = p->cell_nodes_offset[c];
    x.resize(ng * dim);
    for (int k = 0; k < ng; ++k) {
        const int64_t nid = p->cell_nodes[off + k] - 1;
        if (nid < 0 || nid >= p->n_nodes) { err->code = OR_ERR_BOUNDS; err->cell = c + 1; return OR_ERR_BOUNDS; }
        for (int a = 0; a < dim; ++a) x[k * dim + a] = p->nodes[nid * p->dim + a];
    }
    double bad = 0;
    if (cv.reinit(x.data(), &bad)) {
        err->code = OR_ERR_DETJ;
        err->cell = c + 1;
        err->detJ = bad;
        return OR_ERR_DETJ;
    }
    for (int i = 0; i < ld * ld; ++i) Ke[i] = 0.0;
    for (int i = 0; i < ld; ++i) fe[i] = 0.0;
    const double scale = ph->cell_scale ? ph->cell_scale[c] : 1.0;
    const int64_t* cdofs = p->cell_dofs + (p->cell_dofs_offset[c] - 1);
    if (ph->physics == OR_HEAT) {  // heat_equation.jl:143-164
        const double k = ph->p0 * scale, src = ph->p1;
        for (int q = 0; q < cv.nq; ++q) {
            const double dO = cv.detJdV[q];
            for (int i = 0; i < nb; ++i) {
                const double* gi = &cv.dNdx[(q * nb + i) * dim];
                fe[i] += src * cv.N[q * nb + i] * dO;
                for (int j = 0; j < nb; ++j) {
                    const double* gj = &cv.dNdx[(q * nb + j) * dim];
                    double dot = 0;
                    for (int a = 0; a < dim; ++a) dot += gi[a] * gj[a];
                    Ke[j * ld + i] += k * dot * dO;
                }
            }
        }
    } else if (ph->physics == OR_LINEAR_ELASTIC) {
        // threaded_assembly.jl:105-132: (eps_i : C : eps_j) dOmega with isotropic C,
        // written out as lambda d_a N_i d_b N_j + mu (d_b N_i d_a N_j + delta_ab gradN_i.gradN_j)
        const double E = ph->p0 * scale, nu = ph->p1;
        const double lam = E * nu / ((1 + nu) * (1 - 2 * nu)), mu = E / (2 * (1 + nu));
        for (int q = 0; q < cv.nq; ++q) {
            const double dO = cv.detJdV[q];
            for (int i = 0; i < nb; ++i) {
                const double* gi = &cv.dNdx[(q * nb + i) * dim];
                for (int a = 0; a < nc; ++a) fe[i * nc + a] += cv.N[q * nb + i] * ph->body[a] * dO;
                for (int j = 0; j < nb; ++j) {
                    const double* gj = &cv.dNdx[(q * nb + j) * dim];
                    double dot = 0;
                    for (int d = 0; d < dim; ++d) dot += gi[d] * gj[d];
                    for (int a = 0; a < nc; ++a)
                        for (int b = 0; b < nc; ++b) {
                            double v = lam * gi[a] * gj[b] + mu * gi[b] * gj[a];
                            if (a == b) v += mu * dot;
                            Ke[(j * nc + b) * ld + (i * nc + a)] += v * dO;
                        }
                }
            }
        }
    } else if (ph->physics == OR_NEO_HOOKE) {  // hyperelasticity.jl:241-276 (cell part)
        if (nc != 3 || dim != 3) return OR_ERR_UNSUPPORTED;
        ue.resize(ld);
        for (int i = 0; i < ld; ++i) ue[i] = ph->u ? ph->u[cdofs[i] - 1] : 0.0;
        const double mu = ph->p0, lam = ph->p1;
        double F[9], P[9], A[81];
        for (int q = 0; q < cv.nq; ++q) {
            const double dO = cv.detJdV[q];
            for (int a = 0; a < 9; ++a) F[a] = 0.0;
            for (int i = 0; i < nb; ++i)  // function_gradient (common_values.jl:217-227)
                for (int a = 0; a < 3; ++a)
                    for (int J = 0; J < 3; ++J) F[a * 3 + J] += ue[i * 3 + a] * cv.dNdx[(q * nb + i) * 3 + J];
            F[0] += 1; F[4] += 1; F[8] += 1;
            neo_hooke(mu, lam, F, P, A);
            for (int i = 0; i < nb; ++i) {
                const double* gi = &cv.dNdx[(q * nb + i) * 3];
                const double Ni = cv.N[q * nb + i];
                for (int a = 0; a < 3; ++a) {
                    double s = 0;
                    for (int J = 0; J < 3; ++J) s += gi[J] * P[a * 3 + J];
                    fe[i * 3 + a] += (s - Ni * ph->body[a]) * dO;
                }
                for (int j = 0; j < nb; ++j) {
                    const double* gj = &cv.dNdx[(q * nb + j) * 3];
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) {
                            double s = 0;
                            for (int J = 0; J < 3; ++J)
                                for (int L = 0; L < 3; ++L) s += gi[J] * A[((a * 3 + J) * 3 + b) * 3 + L] * gj[L];
                            Ke[(j * 3 + b) * ld + (i * 3 + a)] += s * dO;
                        }
                }
            }
        }
    } else {
        return OR_ERR_ARG;
    }
    return OR_OK;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------------------
// Grid generation (src/Grid/grid_generators.jl)
// ---------------------------------------------------------------------------------------
int or_grid_counts(int32_t ct, const int64_t* nel, int64_t* n_nodes, int64_t* n_cells, int32_t* npc,
                   int32_t* dim) {
    if (ct == OR_QUADRILATERAL || ct == OR_TRIANGLE) {
        *dim = 2;
        *n_nodes = (nel[0] + 1) * (nel[1] + 1);
        *n_cells = nel[0] * nel[1] * (ct == OR_TRIANGLE ? 2 : 1);
        *npc = ct == OR_TRIANGLE ? 3 : 4;
        return OR_OK;
    }
    *dim = 3;
    *n_nodes = (nel[0] + 1) * (nel[1] + 1) * (nel[2] + 1);
    const int64_t cubes = nel[0] * nel[1] * nel[2];
    if (ct == OR_HEXAHEDRON) { *n_cells = cubes; *npc = 8; return OR_OK; }
    if (ct == OR_TETRAHEDRON) { *n_cells = 6 * cubes; *npc = 4; return OR_OK; }
    if (ct == OR_WEDGE) { *n_cells = 2 * cubes; *npc = 6; return OR_OK; }
    return OR_ERR_UNSUPPORTED;
}

int or_generate_grid(int32_t ct, const int64_t* nel, const double* left, const double* right,
                     double* nodes, int64_t* cells) {
    if (ct == OR_QUADRILATERAL || ct == OR_TRIANGLE) {
        const int64_t nx = nel[0] + 1, ny = nel[1] + 1;
        // corners from _extrema_to_corners (grid_generators.jl:562-578): reference corner
        // xi in {-1,1}^2, x = left + diag(dx/2) . (xi + 1)
        double corners[4][2];
        const double refc[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
        for (int k = 0; k < 4; ++k)
            for (int a = 0; a < 2; ++a) {
                const double dxi = refc[k][a] - (-1.0);
                const double A = (right[a] - left[a]) / 2.0;
                double s = 0.0;
                for (int b = 0; b < 2; ++b) s += (a == b ? A : 0.0) * (refc[k][b] - (-1.0));
                (void)dxi;
                corners[k][a] = left[a] + s;
            }
        // _generate_nodes (grid_generators.jl:550-559), first index fastest
        int64_t id = 0;
        for (int64_t j = 0; j < ny; ++j)
            for (int64_t i = 0; i < nx; ++i, ++id) {
                const double xi[2] = {2.0 * (double)i / (double)(nx - 1) - 1.0, 2.0 * (double)j / (double)(ny - 1) - 1.0};
                double x[2] = {0.0, 0.0};
                for (int k = 0; k < 4; ++k) {
                    double Mk, dM[3];
                    shape_value_grad(OR_QUADRILATERAL, 1, k, xi, Mk, dM);
                    for (int a = 0; a < 2; ++a) x[a] += Mk * corners[k][a];
                }
                nodes[2 * id] = x[0];
                nodes[2 * id + 1] = x[1];
            }
        // cells, j outer, i inner (grid_generators.jl:89-92)
        int64_t c = 0;
        for (int64_t j = 0; j < nel[1]; ++j)
            for (int64_t i = 0; i < nel[0]; ++i) {
                const int64_t n1 = i + j * nx + 1, n2 = i + 1 + j * nx + 1, n3 = i + 1 + (j + 1) * nx + 1,
                              n4 = i + (j + 1) * nx + 1;
                if (ct == OR_QUADRILATERAL) {
                    cells[4 * c + 0] = n1; cells[4 * c + 1] = n2; cells[4 * c + 2] = n3; cells[4 * c + 3] = n4;
                    ++c;
                } else {  // Triangle split (grid_generators.jl:396-397)
                    cells[3 * c + 0] = n1; cells[3 * c + 1] = n2; cells[3 * c + 2] = n4; ++c;
                    cells[3 * c + 0] = n2; cells[3 * c + 1] = n3; cells[3 * c + 2] = n4; ++c;
                }
            }
        return OR_OK;
    }
    const int64_t nx = nel[0] + 1, ny = nel[1] + 1, nz = nel[2] + 1;
    double corners[8][3];
    const double refc[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                               {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (int k = 0; k < 8; ++k)
        for (int a = 0; a < 3; ++a) {
            const double A = (right[a] - left[a]) / 2.0;
            double s = 0.0;
            for (int b = 0; b < 3; ++b) s += (a == b ? A : 0.0) * (refc[k][b] - (-1.0));
            corners[k][a] = left[a] + s;
        }
    int64_t id = 0;
    for (int64_t kk = 0; kk < nz; ++kk)
        for (int64_t j = 0; j < ny; ++j)
            for (int64_t i = 0; i < nx; ++i, ++id) {
                const double xi[3] = {2.0 * (double)i / (double)(nx - 1) - 1.0, 2.0 * (double)j / (double)(ny - 1) - 1.0,
                                      2.0 * (double)kk / (double)(nz - 1) - 1.0};
                double x[3] = {0.0, 0.0, 0.0};
                for (int k = 0; k < 8; ++k) {
                    double Mk, dM[3];
                    shape_value_grad(OR_HEXAHEDRON, 1, k, xi, Mk, dM);
                    for (int a = 0; a < 3; ++a) x[a] += Mk * corners[k][a];
                }
                for (int a = 0; a < 3; ++a) nodes[3 * id + a] = x[a];
            }
    auto nd = [&](int64_t i, int64_t j, int64_t k) { return i + j * nx + k * nx * ny + 1; };
    int64_t c = 0;
    for (int64_t k = 0; k < nel[2]; ++k)
        for (int64_t j = 0; j < nel[1]; ++j)
            for (int64_t i = 0; i < nel[0]; ++i) {
                const int64_t v[8] = {nd(i, j, k),     nd(i + 1, j, k),     nd(i + 1, j + 1, k),     nd(i, j + 1, k),
                                      nd(i, j, k + 1), nd(i + 1, j, k + 1), nd(i + 1, j + 1, k + 1), nd(i, j + 1, k + 1)};
                if (ct == OR_HEXAHEDRON) {  // grid_generators.jl:170-180
                    for (int a = 0; a < 8; ++a) cells[8 * c + a] = v[a];
                    ++c;
                } else if (ct == OR_TETRAHEDRON) {  // grid_generators.jl:506-511
                    const int T[6][4] = {{1, 2, 4, 8}, {1, 5, 2, 8}, {2, 3, 4, 8}, {2, 7, 3, 8}, {2, 5, 6, 8}, {2, 6, 7, 8}};
                    for (int t = 0; t < 6; ++t, ++c)
                        for (int a = 0; a < 4; ++a) cells[4 * c + a] = v[T[t][a] - 1];
                } else if (ct == OR_WEDGE) {  // grid_generators.jl:218-233
                    const int64_t w1[6] = {nd(i, j, k), nd(i + 1, j, k), nd(i, j + 1, k), nd(i, j, k + 1), nd(i + 1, j, k + 1), nd(i, j + 1, k + 1)};
                    const int64_t w2[6] = {nd(i + 1, j, k), nd(i + 1, j + 1, k), nd(i, j + 1, k), nd(i + 1, j, k + 1), nd(i + 1, j + 1, k + 1), nd(i, j + 1, k + 1)};
                    for (int a = 0; a < 6; ++a) cells[6 * c + a] = w1[a];
                    ++c;
                    for (int a = 0; a < 6; ++a) cells[6 * c + a] = w2[a];
                    ++c;
                } else {
                    return OR_ERR_UNSUPPORTED;
                }
            }
    return OR_OK;
}

int or_nbase(int32_t ct, int32_t order) { return nbase(ct, order); }

// ---------------------------------------------------------------------------------------
// Dof distribution (src/Dofs/DofHandler.jl:493-794). One field shared by all SubDofHandlers
// (its vertex/edge/face dicts are shared, so dofs on shared vertices coincide).
// ---------------------------------------------------------------------------------------
int or_close_dofhandler(const or_problem* p, int64_t* cell_dofs, int64_t* cell_dofs_offset, int64_t* ndofs) {
    std::vector<int64_t> vertexdict(p->n_nodes, 0);
    std::map<std::pair<int64_t, int64_t>, int64_t> edgedict;
    std::map<std::tuple<int64_t, int64_t, int64_t>, int64_t> facedict;
    for (int64_t c = 0; c < p->n_cells; ++c) cell_dofs_offset[c] = 0;
    int64_t nextdof = 1, len = 0;
    for (int s = 0; s < p->n_sdh; ++s) {
        const int order = p->sdh_ip_order[s];
        const int ncp = p->sdh_ncomp[s];
        for (int64_t k = p->sdh_cellset_offset[s]; k < p->sdh_cellset_offset[s + 1]; ++k) {
            const int64_t c = p->sdh_cellset[k] - 1;
            const int ct = p->cell_types[c];
            const RefTopo& T = ref_topo(ct);
            const int64_t* nodes = p->cell_nodes + p->cell_nodes_offset[c];
            if (nbase(ct, order) < 0) return OR_ERR_UNSUPPORTED;
            cell_dofs_offset[c] = len + 1;
            // add_vertex_dofs (DofHandler.jl:715-738)
            for (int v = 0; v < T.nvert; ++v) {
                const int64_t vid = nodes[v] - 1;
                if (vertexdict[vid] > 0) {
                    for (int d = 0; d < ncp; ++d) cell_dofs[len++] = vertexdict[vid] + d;
                } else {
                    vertexdict[vid] = nextdof;
                    for (int d = 0; d < ncp; ++d) cell_dofs[len++] = nextdof++;
                }
            }
            if (order == 2) {
                // add_edge_dofs (DofHandler.jl:774-785) with sortedge (854-857); one dof per
                // edge, so no permutation (Lagrange order 2: adjust_dofs_during_distribution = false)
                const bool has_edges = T.rdim == 3 || ct == OR_QUADRILATERAL;
                if (has_edges) {
                    for (const auto& e : T.edges) {
                        int64_t a = nodes[e[0] - 1], b = nodes[e[1] - 1];
                        if (a > b) std::swap(a, b);
                        auto it = edgedict.find({a, b});
                        int64_t first;
                        if (it != edgedict.end()) {
                            first = it->second;
                        } else {
                            first = nextdof;
                            edgedict[{a, b}] = nextdof;
                            nextdof += ncp;
                        }
                        for (int d = 0; d < ncp; ++d) cell_dofs[len++] = first + d;
                    }
                }
                // add_face_dofs (761-772) with sortface (1029-1057): key = 3 smallest vertices
                if (ct == OR_HEXAHEDRON || ct == OR_QUADRILATERAL) {
                    for (const auto& f : T.faces) {
                        std::vector<int64_t> v;
                        for (int q : f) v.push_back(nodes[q - 1]);
                        std::sort(v.begin(), v.end());
                        auto key = std::make_tuple(v[0], v[1], v[2]);
                        auto it = facedict.find(key);
                        int64_t first;
                        if (it != facedict.end()) {
                            first = it->second;
                        } else {
                            first = nextdof;
                            facedict[key] = nextdof;
                            nextdof += ncp;
                        }
                        for (int d = 0; d < ncp; ++d) cell_dofs[len++] = first + d;
                    }
                }
                // add_volume_dofs (787-794)
                if (ct == OR_HEXAHEDRON)
                    for (int d = 0; d < ncp; ++d) cell_dofs[len++] = nextdof++;
            }
        }
    }
    *ndofs = nextdof - 1;
    return OR_OK;
}

// ---------------------------------------------------------------------------------------
// Sparsity pattern (sparsity_pattern.jl:223-253, 549, 1136-1249): every (row, col) pair of
// dofs sharing a cell, plus the diagonal; rows ascending within each column. The pattern is
// symmetric, so the column lists equal the row lists Ferrite builds.
// ---------------------------------------------------------------------------------------
int or_sparsity_pattern(const or_problem* p, int64_t* colptr, int64_t* rowval, int64_t* nnz) {
    Setup S;
    // only cellsets and dofs are needed here
    std::vector<int> cell_sdh(p->n_cells, -1);
    std::vector<int> ndpc(p->n_sdh);
    for (int s = 0; s < p->n_sdh; ++s) {
        const int64_t b = p->sdh_cellset_offset[s];
        const int ct = p->cell_types[p->sdh_cellset[b] - 1];
        ndpc[s] = nbase(ct, p->sdh_ip_order[s]) * p->sdh_ncomp[s];
        for (int64_t k = b; k < p->sdh_cellset_offset[s + 1]; ++k) cell_sdh[p->sdh_cellset[k] - 1] = s;
    }
    const int64_t n = p->ndofs;
    // dof -> cells (CSR)
    std::vector<int64_t> dptr(n + 1, 0);
    for (int64_t c = 0; c < p->n_cells; ++c) {
        if (cell_sdh[c] < 0) continue;
        const int64_t* cd = p->cell_dofs + p->cell_dofs_offset[c] - 1;
        for (int i = 0; i < ndpc[cell_sdh[c]]; ++i) {
            if (cd[i] < 1 || cd[i] > n) return OR_ERR_BOUNDS;
            dptr[cd[i]]++;
        }
    }
    for (int64_t d = 0; d < n; ++d) dptr[d + 1] += dptr[d];
    std::vector<int64_t> dcells(dptr[n]);
    {
        std::vector<int64_t> cur(dptr.begin(), dptr.end() - 1);
        for (int64_t c = 0; c < p->n_cells; ++c) {
            if (cell_sdh[c] < 0) continue;
            const int64_t* cd = p->cell_dofs + p->cell_dofs_offset[c] - 1;
            for (int i = 0; i < ndpc[cell_sdh[c]]; ++i) dcells[cur[cd[i] - 1]++] = c;
        }
    }
    auto column = [&](int64_t col, std::vector<int64_t>& buf) {
        buf.clear();
        buf.push_back(col + 1);
        for (int64_t k = dptr[col]; k < dptr[col + 1]; ++k) {
            const int64_t c = dcells[k];
            const int64_t* cd = p->cell_dofs + p->cell_dofs_offset[c] - 1;
            buf.insert(buf.end(), cd, cd + ndpc[cell_sdh[c]]);
        }
        std::sort(buf.begin(), buf.end());
        buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
    };
    if (!rowval) {
        std::vector<int64_t> cnt(n);
#pragma omp parallel
        {
            std::vector<int64_t> buf;
#pragma omp for schedule(dynamic, 4096)
            for (int64_t col = 0; col < n; ++col) {
                column(col, buf);
                cnt[col] = (int64_t)buf.size();
            }
        }
        colptr[0] = 1;
        for (int64_t col = 0; col < n; ++col) colptr[col + 1] = colptr[col] + cnt[col];
        *nnz = colptr[n] - 1;
        return OR_OK;
    }
#pragma omp parallel
    {
        std::vector<int64_t> buf;
#pragma omp for schedule(dynamic, 4096)
        for (int64_t col = 0; col < n; ++col) {
            column(col, buf);
            std::memcpy(rowval + colptr[col] - 1, buf.data(), buf.size() * sizeof(int64_t));
        }
    }
    *nnz = colptr[n] - 1;
    (void)S;
    return OR_OK;
}

int or_quadrature(int32_t ct, int32_t order, int32_t* n_qp, double* weights, double* points) {
    std::vector<double> w, pts;
    int rc = quadrature(ct, order, w, pts);
    if (rc) return rc;
    *n_qp = (int32_t)w.size();
    if (weights) std::memcpy(weights, w.data(), w.size() * sizeof(double));
    if (points) std::memcpy(points, pts.data(), pts.size() * sizeof(double));
    return OR_OK;
}

int or_shape_tables(int32_t ct, int32_t order, int32_t nq, const double* points, double* N, double* dN) {
    const int nb = nbase(ct, order), d = ref_dim(ct);
    if (nb < 0) return OR_ERR_UNSUPPORTED;
    for (int q = 0; q < nq; ++q)
        for (int i = 0; i < nb; ++i) shape_value_grad(ct, order, i, points + q * d, N[q * nb + i], dN + (q * nb + i) * d);
    return OR_OK;
}

// Element matrix of one cell (0-based cell index), Ke column-major ld x ld.
int or_element_matrix(const or_problem* p, const or_physics* ph, int64_t cell, double* Ke, double* fe, or_error* err) {
    Setup S;
    int rc = S.init(p);
    if (rc) return rc;
    const int s = S.cell_sdh[cell];
    if (s < 0) return OR_ERR_ARG;
    std::vector<double> x, ue;
    err->code = OR_OK;
    return element(S, S.cvs[s], s, cell, ph, Ke, fe, x, ue, err);
}

// nzval positions (1-based, 0 = missing) of the element entries of one cell, in the
// merge-walk order of assembler.jl:376-457: positions[J*ld + I] for Ke[I, J].
int or_index_map(const or_problem* p, int64_t cell, int64_t* positions) {
    Setup S;
    int rc = S.init(p);
    if (rc) return rc;
    const int s = S.cell_sdh[cell];
    if (s < 0) return OR_ERR_ARG;
    const int ld = S.ndpc[s];
    CSCView K{p->ndofs, p->colptr, p->rowval};
    std::vector<int64_t> sorted;
    std::vector<int> perm;
    const int64_t* dofs = p->cell_dofs + p->cell_dofs_offset[cell] - 1;
    for (int i = 0; i < ld * ld; ++i) positions[i] = 0;
    merge_walk(K, dofs, ld, sorted, perm,
               [&](int64_t R, int ker, int kec) { positions[kec * ld + ker] = R + 1; },
               [&](int64_t, int64_t, int, int) {});
    return OR_OK;
}

// CSR assembler of ext/FerriteSparseMatrixCSR.jl:9-96 (start_assemble for SparseMatrixCSR and
// its _assemble_inner!): per sorted row dof, a walk over the row's sorted columns (dense row and
// binary-search fast paths as for CSC), K[row, col] += Ke[row_local, col_local] with zeros
// skipped, a non-zero without a pattern entry reported as (row, col). The row walk is the CSC
// column walk on (rowptr, colval) with the element matrix read transposed.
int or_assemble_csr(const or_problem* p, const or_physics* ph, int32_t fillzero, const int64_t* rowptr,
                    const int64_t* colval, double* nzval, double* f, or_error* err) {
    Setup S;
    int rc = S.init(p);
    err->code = OR_OK;
    err->cell = 0;
    if (rc) { err->code = rc; return rc; }
    const int64_t nnz = rowptr[p->ndofs] - 1;
    if (fillzero) {
        if (nzval) std::memset(nzval, 0, nnz * sizeof(double));
        if (f) std::memset(f, 0, p->ndofs * sizeof(double));
    }
    CSCView rows{p->ndofs, rowptr, colval};
    std::vector<double> Ke, fe, x, ue;
    std::vector<int64_t> sorted;
    std::vector<int> perm;
    for (int s = 0; s < p->n_sdh; ++s)
        for (int64_t k = p->sdh_cellset_offset[s]; k < p->sdh_cellset_offset[s + 1]; ++k) {
            const int64_t c = p->sdh_cellset[k] - 1;
            const int ld = S.ndpc[s];
            Ke.resize(ld * ld);
            fe.resize(ld);
            int r = element(S, S.cvs[s], s, c, ph, Ke.data(), fe.data(), x, ue, err);
            if (r) return r;
            const int64_t* dofs = p->cell_dofs + p->cell_dofs_offset[c] - 1;
            if (f)
                for (int i = 0; i < ld; ++i) f[dofs[i] - 1] += fe[i];
            if (!nzval) continue;
            int miss_code = OR_OK;
            // walk row dofs[kerow]; kecol is the local index of the column found at R
            merge_walk(rows, dofs, ld, sorted, perm,
                       [&](int64_t R, int kecol, int kerow) {
                           const double v = Ke[kecol * ld + kerow];  // Ke[kerow, kecol], column-major
                           if (v != 0.0) nzval[R] += v;
                       },
                       [&](int64_t col, int64_t row, int kecol, int kerow) {
                           if (Ke[kecol * ld + kerow] != 0.0 && miss_code == OR_OK) {
                               miss_code = OR_ERR_PATTERN_MISSING;
                               err->code = OR_ERR_PATTERN_MISSING;
                               err->row = row;
                               err->col = col;
                               err->cell = c + 1;
                           }
                       });
            if (miss_code) return miss_code;
        }
    return OR_OK;
}

// Element-matrix product y (+)= sum_c A_c^T Ke_c A_c u in ascending cell order: the consumer
// of the element-assembly output of docs/src/literate-howto/gpu_assembly.jl:265-303 (Kes per
// cell, FP32 there), with explicit fused multiply-adds so the operation order is exact.
extern "C++" {
template <typename T>
static void element_matvec(const or_problem* p, const Setup& S, const T* ke, const int64_t* ks, const double* u,
                           double* y) {
    std::vector<T> ue, ye;
    for (int64_t c = 0; c < p->n_cells; ++c) {
        const int s = S.cell_sdh[c];
        if (s < 0) continue;
        const int n = S.ndpc[s];
        const int64_t* dofs = p->cell_dofs + p->cell_dofs_offset[c] - 1;
        ue.assign(n, T(0));
        ye.assign(n, T(0));
        for (int J = 0; J < n; ++J) ue[J] = (T)u[dofs[J] - 1];
        const T* kc = ke + c * ks[0];
        for (int J = 0; J < n; ++J)
            for (int I = 0; I < n; ++I) ye[I] = std::fma(kc[I * ks[1] + J * ks[2]], ue[J], ye[I]);
        for (int I = 0; I < n; ++I) y[dofs[I] - 1] += (double)ye[I];
    }
}
}

int or_element_matvec(const or_problem* p, int32_t fp64, const void* ke, const int64_t* ks, const double* u,
                      int32_t fillzero, double* y) {
    Setup S;
    int rc = S.init(p);
    if (rc) return rc;
    if (fillzero)
        for (int64_t i = 0; i < p->ndofs; ++i) y[i] = 0.0;
    if (fp64)
        element_matvec(p, S, (const double*)ke, ks, u, y);
    else
        element_matvec(p, S, (const float*)ke, ks, u, y);
    return OR_OK;
}

// Greedy node-sharing coloring in cell order (coloring.jl:47-143).
int or_greedy_coloring(const or_problem* p, int32_t* cell_color, int32_t* n_colors) {
    std::vector<int64_t> nptr(p->n_nodes + 1, 0);
    for (int64_t c = 0; c < p->n_cells; ++c)
        for (int64_t k = p->cell_nodes_offset[c]; k < p->cell_nodes_offset[c + 1]; ++k) nptr[p->cell_nodes[k]]++;
    for (int64_t v = 0; v < p->n_nodes; ++v) nptr[v + 1] += nptr[v];
    std::vector<int64_t> ncells(nptr[p->n_nodes]);
    {
        std::vector<int64_t> cur(nptr.begin(), nptr.end() - 1);
        for (int64_t c = 0; c < p->n_cells; ++c)
            for (int64_t k = p->cell_nodes_offset[c]; k < p->cell_nodes_offset[c + 1]; ++k)
                ncells[cur[p->cell_nodes[k] - 1]++] = c;
    }
    for (int64_t c = 0; c < p->n_cells; ++c) cell_color[c] = 0;
    int total = 0;
    std::vector<char> occupied;
    for (int64_t c = 0; c < p->n_cells; ++c) {
        std::fill(occupied.begin(), occupied.end(), 0);
        for (int64_t k = p->cell_nodes_offset[c]; k < p->cell_nodes_offset[c + 1]; ++k) {
            const int64_t v = p->cell_nodes[k] - 1;
            for (int64_t r = nptr[v]; r < nptr[v + 1]; ++r) {
                const int col = cell_color[ncells[r]];
                if (col) occupied[col - 1] = 1;
            }
        }
        int free_color = 0;
        for (int k = 0; k < total; ++k)
            if (!occupied[k]) { free_color = k + 1; break; }
        if (!free_color) {
            free_color = ++total;
            occupied.push_back(0);
        }
        cell_color[c] = free_color;
    }
    *n_colors = total;
    return OR_OK;
}

}  // extern "C"

namespace {

// Node-sharing cell incidence (create_incidence_matrix, coloring.jl:47-103): for each cell,
// the other cells sharing at least one node with it, ascending and without duplicates.
struct Incidence {
    std::vector<int64_t> ptr, adj;  // 0-based cell ids; ptr has n_cells + 1 entries
};
Incidence cell_incidence(const or_problem* p) {
    const int64_t n = p->n_cells;
    std::vector<int64_t> nptr(p->n_nodes + 1, 0);
    for (int64_t c = 0; c < n; ++c)
        for (int64_t k = p->cell_nodes_offset[c]; k < p->cell_nodes_offset[c + 1]; ++k) nptr[p->cell_nodes[k]]++;
    for (int64_t v = 0; v < p->n_nodes; ++v) nptr[v + 1] += nptr[v];
    std::vector<int64_t> ncells(nptr[p->n_nodes]);
    {
        std::vector<int64_t> cur(nptr.begin(), nptr.end() - 1);
        for (int64_t c = 0; c < n; ++c)
            for (int64_t k = p->cell_nodes_offset[c]; k < p->cell_nodes_offset[c + 1]; ++k)
                ncells[cur[p->cell_nodes[k] - 1]++] = c;
    }
    Incidence I;
    I.ptr.assign(n + 1, 0);
    std::vector<std::vector<int64_t>> rows(n);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < n; ++c) {
        std::vector<int64_t>& cand = rows[c];
        for (int64_t k = p->cell_nodes_offset[c]; k < p->cell_nodes_offset[c + 1]; ++k) {
            const int64_t v = p->cell_nodes[k] - 1;
            for (int64_t r = nptr[v]; r < nptr[v + 1]; ++r)
                if (ncells[r] != c) cand.push_back(ncells[r]);
        }
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    }
    for (int64_t c = 0; c < n; ++c) I.ptr[c + 1] = I.ptr[c] + (int64_t)rows[c].size();
    I.adj.resize(I.ptr[n]);
    for (int64_t c = 0; c < n; ++c) std::copy(rows[c].begin(), rows[c].end(), I.adj.begin() + I.ptr[c]);
    return I;
}

// _greedy_coloring! (coloring.jl:108-143) over `cells` in order, neighbours restricted to the
// cells for which member(c) holds; returns the color classes, cells in visiting order.
template <class Member>
std::vector<std::vector<int64_t>> greedy_classes(const Incidence& I, const std::vector<int64_t>& cells,
                                                 std::vector<int32_t>& cell_colors, Member member) {
    std::vector<std::vector<int64_t>> classes;
    std::vector<char> occupied;
    for (const int64_t c : cells) {
        std::fill(occupied.begin(), occupied.end(), 0);
        for (int64_t r = I.ptr[c]; r < I.ptr[c + 1]; ++r) {
            const int64_t nb = I.adj[r];
            if (!member(nb)) continue;
            const int32_t col = cell_colors[nb];
            if (col) occupied[col - 1] = 1;
        }
        int32_t free_color = 0;
        for (int32_t k = 0; k < (int32_t)classes.size(); ++k)
            if (!occupied[k]) { free_color = k + 1; break; }
        if (!free_color) {
            classes.emplace_back();
            occupied.push_back(0);
            free_color = (int32_t)classes.size();
        }
        cell_colors[c] = free_color;
        classes[free_color - 1].push_back(c);
    }
    return classes;
}

// workstream_coloring (coloring.jl:171-264, Turcksin et al. 2016 with greedy zone colorings),
// Ferrite's default create_coloring algorithm (coloring.jl:308), over all cells:
//  1. zones = levels of a breadth-first traversal from the lowest unvisited cell;
//  2. each zone colored greedily among its own cells;
//  3. the colors of the largest odd zone followed by those of the largest even zone are the
//     global colors; every other zone's colors, largest first, join the smallest global
//     color of its parity not yet used by that zone; each color is then sorted.
std::vector<std::vector<int64_t>> workstream_colors(const or_problem* p, const Incidence& I) {
    const int64_t n = p->n_cells;
    std::vector<std::vector<int64_t>> out;
    if (n == 0) return out;
    if (n == 1) return {{0}};
    std::vector<int64_t> zone_of(n, 0);
    std::vector<std::vector<int64_t>> zones;
    int64_t visited = 0, seed = 0;
    while (visited < n) {
        while (zone_of[seed] != 0) ++seed;
        zones.push_back({seed});
        zone_of[seed] = (int64_t)zones.size();
        ++visited;
        while (true) {
            std::vector<int64_t> s;
            const int64_t Z = (int64_t)zones.size() + 1;
            for (const int64_t c : zones.back())
                for (int64_t r = I.ptr[c]; r < I.ptr[c + 1]; ++r) {
                    const int64_t nb = I.adj[r];
                    if (zone_of[nb] == 0) {
                        zone_of[nb] = Z;
                        s.push_back(nb);
                    }
                }
            if (s.empty()) break;
            visited += (int64_t)s.size();
            zones.push_back(std::move(s));
        }
    }
    const int64_t nz = (int64_t)zones.size();
    std::vector<std::vector<std::vector<int64_t>>> zc(nz);
    std::vector<int32_t> cell_colors(n, 0);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t zi = 0; zi < nz; ++zi)  // zones touch disjoint parts of cell_colors
        zc[zi] = greedy_classes(I, zones[zi], cell_colors, [&](int64_t c) { return zone_of[c] == zi + 1; });
    // findmax over odd / even zone numbers (1-based), first maximum
    int64_t Nodd = -1, Zodd = -1, Neven = -1, Zeven = -1;
    for (int64_t z = 1; z <= nz; ++z) {
        const int64_t len = (int64_t)zc[z - 1].size();
        if (z & 1) {
            if (len > Nodd) { Nodd = len; Zodd = z; }
        } else if (len > Neven) {
            Neven = len;
            Zeven = z;
        }
    }
    if (Zeven < 0) Neven = 0;
    const int64_t N = Nodd + Neven;
    out = zc[Zodd - 1];
    if (Zeven > 0) out.insert(out.end(), zc[Zeven - 1].begin(), zc[Zeven - 1].end());
    std::vector<int64_t> sizes(N);
    for (int64_t x = 0; x < N; ++x) sizes[x] = (int64_t)out[x].size();
    std::vector<char> used(N);
    for (int64_t z = 1; z <= nz; ++z) {
        if (z == Zodd || z == Zeven) continue;
        const auto& zcv = zc[z - 1];
        const bool odd = z & 1;
        std::fill(used.begin(), used.end(), 0);
        std::vector<int64_t> order(zcv.size());
        for (size_t k = 0; k < order.size(); ++k) order[k] = (int64_t)k;
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return zcv[a].size() > zcv[b].size(); });
        for (const int64_t lc : order) {
            int64_t best = -1;
            for (int64_t x = 0; x < N; ++x) {
                const bool ok = (odd ? x + 1 <= Nodd : x + 1 > Nodd) && !used[x];
                if (ok && (best < 0 || sizes[x] < sizes[best])) best = x;
            }
            used[best] = 1;
            out[best].insert(out[best].end(), zcv[lc].begin(), zcv[lc].end());
            sizes[best] = (int64_t)out[best].size();
        }
    }
    for (auto& c : out) std::sort(c.begin(), c.end());
    return out;
}

// Greedy colors in cell order (greedy_coloring, coloring.jl:146-160), as classes.
std::vector<std::vector<int64_t>> greedy_colors(const or_problem* p) {
    std::vector<int32_t> color(p->n_cells);
    int32_t ncol = 0;
    or_greedy_coloring(p, color.data(), &ncol);
    std::vector<std::vector<int64_t>> colors(ncol);
    for (int s = 0; s < p->n_sdh; ++s)
        for (int64_t k = p->sdh_cellset_offset[s]; k < p->sdh_cellset_offset[s + 1]; ++k) {
            const int64_t c = p->sdh_cellset[k] - 1;
            colors[color[c] - 1].push_back(c);
        }
    return colors;
}

// One cell of the loop body of threaded_assembly.jl:232-265 / heat_equation.jl:186-206:
// reinit!, the element routine, then assemble! (f += fe; merge walk into nzval).
int assemble_cell(const or_problem* p, const Setup& S, const or_physics* ph, int64_t c, CellValues& cv,
                  std::vector<double>& Ke, std::vector<double>& fe, std::vector<double>& x, std::vector<double>& ue,
                  std::vector<int64_t>& sorted, std::vector<int>& perm, double* nzval, double* f, or_error& e) {
    const CSCView K{p->ndofs, p->colptr, p->rowval};
    const int s = S.cell_sdh[c];
    const int ld = S.ndpc[s];
    Ke.resize(ld * ld);
    fe.resize(ld);
    int r = element(S, cv, s, c, ph, Ke.data(), fe.data(), x, ue, &e);
    if (r) return r;
    const int64_t* dofs = p->cell_dofs + p->cell_dofs_offset[c] - 1;
    if (f)
        for (int i = 0; i < ld; ++i) f[dofs[i] - 1] += fe[i];
    if (!nzval) return OR_OK;
    int miss_code = OR_OK;
    merge_walk(K, dofs, ld, sorted, perm,
               [&](int64_t R, int ker, int kec) {
                   const double v = Ke[kec * ld + ker];
                   if (v != 0.0) nzval[R] += v;  // addindex! skips zeros (arrayutils.jl:100-107)
               },
               [&](int64_t row, int64_t col, int ker, int kec) {
                   if (Ke[kec * ld + ker] != 0.0 && miss_code == OR_OK) {
                       miss_code = OR_ERR_PATTERN_MISSING;
                       e.code = OR_ERR_PATTERN_MISSING;
                       e.row = row;
                       e.col = col;
                       e.cell = c + 1;
                   }
               });
    return miss_code;
}

// The colored loop of threaded_assembly.jl:232-265: colors in order, the cells of one color
// split into equal chunks over the threads (OhMyThreads' DynamicScheduler with ntasks = the
// thread count), each thread with its own CellValues copy and assembler buffers (ScratchData,
// created per task, 164-193). The first error by cell id is reported.
int assemble_colored(const or_problem* p, const Setup& S, const std::vector<std::vector<int64_t>>& colors,
                     const or_physics* ph, int32_t nthreads, double* nzval, double* f, or_error* err) {
    int status = OR_OK;
    or_error first_err{};
#ifdef _OPENMP
    omp_set_num_threads(nthreads);
#endif
    for (size_t col = 0; col < colors.size() && status == OR_OK; ++col) {
        const std::vector<int64_t>& cells = colors[col];
#pragma omp parallel
        {
            std::vector<CellValues> cvs = S.cvs;  // task-local CellValues copies
            std::vector<double> Ke, fe, x, ue;
            std::vector<int64_t> sorted;
            std::vector<int> perm;
            or_error e{};
#pragma omp for schedule(static)
            for (int64_t k = 0; k < (int64_t)cells.size(); ++k) {
                const int64_t c = cells[k];
                int r = assemble_cell(p, S, ph, c, cvs[S.cell_sdh[c]], Ke, fe, x, ue, sorted, perm, nzval, f, e);
                if (r) {
#pragma omp critical
                    {
                        if (status == OR_OK || e.cell < first_err.cell) {
                            status = r;
                            first_err = e;
                        }
                    }
                }
            }
        }
    }
    if (status) *err = first_err;
    return status;
}

}  // namespace

// A threaded assembly prepared once, as the how-to prepares it before its timed calls: the
// problem view, the CellValues and the coloring (create_coloring in create_cantilever_grid,
// threaded_assembly.jl:134-141); each or_threaded_assemble call is one assemble_global!.
struct or_threaded {
    or_problem p;
    Setup S;
    std::vector<std::vector<int64_t>> colors;
    int32_t nthreads;
};

extern "C" {

int or_threaded_create(const or_problem* p, int32_t nthreads, int32_t algorithm, or_threaded** out,
                       int32_t* n_colors) {
    if (!p || !out || nthreads <= 0) return OR_ERR_ARG;
    or_threaded* t = new or_threaded();
    t->p = *p;
    t->nthreads = nthreads;
    int rc = t->S.init(&t->p);
    if (rc) {
        delete t;
        return rc;
    }
#ifdef _OPENMP
    omp_set_num_threads(nthreads);
#endif
    if (algorithm == OR_COLORING_WORKSTREAM) {
        t->colors = workstream_colors(&t->p, cell_incidence(&t->p));
    } else if (algorithm == OR_COLORING_GREEDY) {
        t->colors = greedy_colors(&t->p);
    } else {
        delete t;
        return OR_ERR_ARG;
    }
    if (n_colors) *n_colors = (int32_t)t->colors.size();
    *out = t;
    return OR_OK;
}

int or_threaded_colors(const or_threaded* t, int32_t* cell_color) {
    for (size_t k = 0; k < t->colors.size(); ++k)
        for (const int64_t c : t->colors[k]) cell_color[c] = (int32_t)k + 1;
    return OR_OK;
}

int or_threaded_assemble(or_threaded* t, const or_physics* ph, double* nzval, double* f, or_error* err) {
    err->code = OR_OK;
    err->cell = 0;
    const or_problem* p = &t->p;
    // start_assemble(K, f) zeroes K and f (assembler.jl:287-291, arrayutils.jl:145-148)
    if (nzval) std::memset(nzval, 0, (p->colptr[p->ndofs] - 1) * sizeof(double));
    if (f) std::memset(f, 0, p->ndofs * sizeof(double));
    return assemble_colored(p, t->S, t->colors, ph, t->nthreads, nzval, f, err);
}

void or_threaded_destroy(or_threaded* t) { delete t; }

// Full assembly: start_assemble (zero K and f), then the cell loop with reinit!, the element
// routine and assemble!. nthreads == 0: sequential loop over the SubDofHandlers' cells in
// order (heat_equation.jl:186-206). nthreads > 0: greedy colors, cells of one color in
// parallel, one CellValues/assembler scratch per thread (threaded_assembly.jl:232-265).
int or_assemble(const or_problem* p, const or_physics* ph, int32_t nthreads, int32_t fillzero, double* nzval,
                double* f, or_error* err) {
    Setup S;
    int rc = S.init(p);
    err->code = OR_OK;
    err->cell = 0;
    if (rc) { err->code = rc; return rc; }
    const int64_t nnz = p->colptr[p->ndofs] - 1;
    if (fillzero) {  // fillzero! (arrayutils.jl:145-148)
        if (nzval) std::memset(nzval, 0, nnz * sizeof(double));
        if (f) std::memset(f, 0, p->ndofs * sizeof(double));
    }
    if (nthreads > 0) return assemble_colored(p, S, greedy_colors(p), ph, nthreads, nzval, f, err);
    std::vector<double> Ke, fe, x, ue;
    std::vector<int64_t> sorted;
    std::vector<int> perm;
    for (int s = 0; s < p->n_sdh; ++s)
        for (int64_t k = p->sdh_cellset_offset[s]; k < p->sdh_cellset_offset[s + 1]; ++k) {
            const int64_t c = p->sdh_cellset[k] - 1;
            int r = assemble_cell(p, S, ph, c, S.cvs[s], Ke, fe, x, ue, sorted, perm, nzval, f, *err);
            if (r) return r;
        }
    return OR_OK;
}


// ---------------------------------------------------------------------------------------
// Adjoint (vector-Jacobian products) of the heat and linear-elastic assembly, FP64. The
// formulas are derived from Phi = lambda^T (K u - f) with J = sum_k x_k (x) dM_k/dxi:
// d(dV) = dV tr(J^-1 dJ), d(grad v) = -grad(v) dJ J^-1, so dPhi/dJ = dV Sigma J^-T and
// dPhi/dx_k = dV Sigma (J^-T dM_k/dxi) (declaration in ferrite_oracle.h).
// ---------------------------------------------------------------------------------------
int or_adjoint(const or_problem* p, const or_physics* ph, const double* u, const double* lam, const double* dscale,
               double* d_cell, double* d_X, or_error* err) {
    Setup S;
    int rc = S.init(p);
    err->code = OR_OK;
    err->cell = 0;
    if (rc) { err->code = rc; return rc; }
    if (ph->physics != OR_HEAT && ph->physics != OR_LINEAR_ELASTIC) return OR_ERR_UNSUPPORTED;
    const int dim = p->dim;
    if (d_X) std::memset(d_X, 0, sizeof(double) * p->n_nodes * dim);
    std::vector<double> x;
    for (int s = 0; s < p->n_sdh; ++s) {
        CellValues& cv = S.cvs[s];
        const int nc = p->sdh_ncomp[s];
        const int nb = cv.nb, ng = cv.ng;
        if (ph->physics == OR_LINEAR_ELASTIC && nc != dim) return OR_ERR_ARG;
        if (ph->physics == OR_HEAT && nc != 1) return OR_ERR_ARG;
        for (int64_t kk = p->sdh_cellset_offset[s]; kk < p->sdh_cellset_offset[s + 1]; ++kk) {
            const int64_t c = p->sdh_cellset[kk] - 1;
            const int64_t off = p->cell_nodes_offset[c];
            x.resize(ng * dim);
            for (int k = 0; k < ng; ++k) {
                const int64_t nid = p->cell_nodes[off + k] - 1;
                for (int a = 0; a < dim; ++a) x[k * dim + a] = p->nodes[nid * p->dim + a];
            }
            double bad = 0;
            if (cv.reinit(x.data(), &bad)) {
                err->code = OR_ERR_DETJ;
                err->cell = c + 1;
                err->detJ = bad;
                return OR_ERR_DETJ;
            }
            const int64_t* dofs = p->cell_dofs + p->cell_dofs_offset[c] - 1;
            const double scale = ph->cell_scale ? ph->cell_scale[c] : 1.0;
            double m0 = 0, m1 = 0;  // unscaled material: heat k; elastic lambda, mu (E = p0)
            if (ph->physics == OR_HEAT) {
                m0 = ph->p0;
            } else {
                const double E = ph->p0, nu = ph->p1;
                m0 = E * nu / ((1 + nu) * (1 - 2 * nu));
                m1 = E / (2 * (1 + nu));
            }
            double gcell = 0.0;
            for (int q = 0; q < cv.nq; ++q) {
                const double dV = cv.detJdV[q];
                // gradients of u and lambda: G[c][d] = d v_c / d x_d; lambda at the point
                double Gu[9] = {0}, Gl[9] = {0}, lq[3] = {0};
                for (int i = 0; i < nb; ++i) {
                    const double* g = &cv.dNdx[(q * nb + i) * dim];
                    const double Ni = cv.N[q * nb + i];
                    for (int a = 0; a < nc; ++a) {
                        const double ui = u[dofs[i * nc + a] - 1], li = lam[dofs[i * nc + a] - 1];
                        lq[a] += Ni * li;
                        for (int d = 0; d < dim; ++d) {
                            Gu[a * dim + d] += ui * g[d];
                            Gl[a * dim + d] += li * g[d];
                        }
                    }
                }
                // fluxes / stresses with the unscaled material, then the scaled ones
                double Su[9] = {0}, Sl[9] = {0};
                if (ph->physics == OR_HEAT) {
                    for (int d = 0; d < dim; ++d) { Su[d] = m0 * Gu[d]; Sl[d] = m0 * Gl[d]; }
                } else {
                    double tu = 0, tl = 0;
                    for (int d = 0; d < dim; ++d) { tu += Gu[d * dim + d]; tl += Gl[d * dim + d]; }
                    for (int a = 0; a < dim; ++a)
                        for (int b = 0; b < dim; ++b) {
                            Su[a * dim + b] = m1 * (Gu[a * dim + b] + Gu[b * dim + a]) + (a == b ? m0 * tu : 0.0);
                            Sl[a * dim + b] = m1 * (Gl[a * dim + b] + Gl[b * dim + a]) + (a == b ? m0 * tl : 0.0);
                        }
                }
                double psi0 = 0;
                for (int t = 0; t < nc * dim; ++t) psi0 += Su[t] * Gl[t];
                gcell += dV * psi0;
                const double psi = scale * psi0;
                double fl = 0;
                if (ph->physics == OR_HEAT) fl = ph->p1 * lq[0];
                else for (int a = 0; a < nc; ++a) fl += lq[a] * ph->body[a];
                // Sigma = (psi - fl) I - Gu^T sigma(lambda) - Gl^T sigma(u), sigma scaled
                double Sg[9];
                for (int b = 0; b < dim; ++b)
                    for (int d = 0; d < dim; ++d) {
                        double v = (b == d) ? (psi - fl) : 0.0;
                        for (int a = 0; a < nc; ++a)
                            v -= scale * (Gu[a * dim + b] * Sl[a * dim + d] + Gl[a * dim + b] * Su[a * dim + d]);
                        Sg[b * dim + d] = v;
                    }
                if (d_X) {
                    // grad M_k = J^-T dM_k/dxi: recompute J^-1 for this point
                    double J[9] = {0}, Ji[9];
                    for (int k = 0; k < ng; ++k)
                        for (int a = 0; a < dim; ++a)
                            for (int b = 0; b < dim; ++b) J[a * dim + b] += x[k * dim + a] * cv.dMdxi[(q * ng + k) * dim + b];
                    inv_n(dim, J, det_n(dim, J), Ji);
                    for (int k = 0; k < ng; ++k) {
                        double gM[3] = {0, 0, 0};
                        for (int b = 0; b < dim; ++b)
                            for (int a = 0; a < dim; ++a) gM[b] += cv.dMdxi[(q * ng + k) * dim + a] * Ji[a * dim + b];
                        const int64_t nid = p->cell_nodes[off + k] - 1;
                        for (int b = 0; b < dim; ++b) {
                            double v = 0;
                            for (int d = 0; d < dim; ++d) v += Sg[b * dim + d] * gM[d];
                            d_X[nid * dim + b] += dV * v;
                        }
                    }
                }
            }
            if (d_cell) d_cell[c] = (dscale ? dscale[c] : 1.0) * gcell;
        }
    }
    return OR_OK;
}

// reference tangents u, v of facet `facet` (1-based): weighted_normal = (J u) x (J v) in 3D,
// rot(J u) = ((J u)_2, -(J u)_1) in 2D (facet_integrals.jl: quadrilateral 122-129, triangle
// 154-160, hexahedron 190-199, tetrahedron 226-234, prism 264-273)
static bool facet_tangents(int32_t ct, int32_t facet, double u[3], double v[3]) {
    for (int k = 0; k < 3; ++k) u[k] = v[k] = 0.0;
    auto e = [](double* x, int k, double s) { x[k] += s; };
    switch (ct) {
        case OR_QUADRILATERAL:
            if (facet == 1) e(u, 0, 1); else if (facet == 2) e(u, 1, 1); else if (facet == 3) e(u, 0, -1);
            else if (facet == 4) e(u, 1, -1); else return false;
            return true;
        case OR_TRIANGLE:
            if (facet == 1) { e(u, 0, -1); e(u, 1, 1); } else if (facet == 2) e(u, 1, -1); else if (facet == 3) e(u, 0, 1);
            else return false;
            return true;
        case OR_HEXAHEDRON: {
            static const int T[6][2] = {{1, 0}, {0, 2}, {1, 2}, {2, 0}, {2, 1}, {0, 1}};
            if (facet < 1 || facet > 6) return false;
            e(u, T[facet - 1][0], 1); e(v, T[facet - 1][1], 1);
            return true;
        }
        case OR_TETRAHEDRON:
            if (facet == 1) { e(u, 1, 1); e(v, 0, 1); }
            else if (facet == 2) { e(u, 0, 1); e(v, 2, 1); }
            else if (facet == 3) { e(u, 0, 1); e(u, 2, -1); e(v, 1, 1); e(v, 2, -1); }
            else if (facet == 4) { e(u, 2, 1); e(v, 1, 1); }
            else return false;
            return true;
        case OR_WEDGE:
            if (facet == 1) { e(u, 1, 1); e(v, 0, 1); }
            else if (facet == 2) { e(u, 0, 1); e(v, 2, 1); }
            else if (facet == 3) { e(u, 2, 1); e(v, 1, 1); }
            else if (facet == 4) { e(u, 1, 1); e(u, 0, -1); e(v, 2, 1); }
            else if (facet == 5) { e(u, 0, 1); e(v, 1, 1); }
            else return false;
            return true;
    }
    return false;
}

int or_facet_load(const or_problem* p, int64_t n, const int64_t* cells, const int32_t* facets, int32_t nf, int32_t nqp,
                  const double* w, const double* N, const double* dM, double pressure, const double* traction, double* f,
                  or_error* err) {
    const int dim = p->dim;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t c = cells[k] - 1;
        const int32_t fc = facets[k];
        if (c < 0 || c >= p->n_cells || fc < 1 || fc > nf) return OR_ERR_BOUNDS;
        const int32_t ct = p->cell_types[c];
        int sdh = -1;
        for (int s = 0; s < p->n_sdh && sdh < 0; ++s)
            for (int64_t t = p->sdh_cellset_offset[s]; t < p->sdh_cellset_offset[s + 1]; ++t)
                if (p->sdh_cellset[t] == c + 1) { sdh = s; break; }
        if (sdh < 0) return OR_ERR_ARG;
        const int nc = p->sdh_ncomp[sdh];
        const int nb = or_nbase(ct, p->sdh_ip_order[sdh]);
        const int64_t off = p->cell_nodes_offset[c];
        const int ng = (int)(p->cell_nodes_offset[c + 1] - off);
        double u[3], v[3];
        if (!facet_tangents(ct, fc, u, v)) return OR_ERR_ARG;
        std::vector<double> fe((size_t)nb * nc, 0.0);
        for (int q = 0; q < nqp; ++q) {
            const double* dMq = dM + ((size_t)(fc - 1) * nqp + q) * ng * dim;
            double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int j = 0; j < ng; ++j) {
                const double* x = p->nodes + (p->cell_nodes[off + j] - 1) * dim;
                for (int a = 0; a < dim; ++a)
                    for (int b = 0; b < dim; ++b) J[a * 3 + b] = J[a * 3 + b] + x[a] * dMq[j * dim + b];
            }
            double wn[3] = {0, 0, 0};
            if (dim == 2) {
                const double ju0 = J[0] * u[0] + J[1] * u[1], ju1 = J[3] * u[0] + J[4] * u[1];
                wn[0] = ju1;
                wn[1] = -ju0;
            } else {
                double ju[3], jv[3];
                for (int a = 0; a < 3; ++a) {
                    ju[a] = J[a * 3] * u[0] + J[a * 3 + 1] * u[1] + J[a * 3 + 2] * u[2];
                    jv[a] = J[a * 3] * v[0] + J[a * 3 + 1] * v[1] + J[a * 3 + 2] * v[2];
                }
                wn[0] = ju[1] * jv[2] - ju[2] * jv[1];
                wn[1] = ju[2] * jv[0] - ju[0] * jv[2];
                wn[2] = ju[0] * jv[1] - ju[1] * jv[0];
            }
            const double nrm = std::sqrt(wn[0] * wn[0] + wn[1] * wn[1] + wn[2] * wn[2]);
            if (!(nrm > 0.0)) {
                if (err) { err->code = OR_ERR_DETJ; err->cell = c + 1; err->detJ = nrm; }
                return OR_ERR_DETJ;
            }
            const double dG = nrm * w[(size_t)(fc - 1) * nqp + q];
            const double* Nq = N + ((size_t)(fc - 1) * nqp + q) * nb;
            for (int i = 0; i < nb; ++i)
                for (int a = 0; a < nc; ++a) {
                    const double t = nc == 1 ? pressure : pressure * (wn[a] / nrm) + traction[a];
                    const double s = Nq[i] * t;
                    fe[(size_t)i * nc + a] = fe[(size_t)i * nc + a] + s * dG;
                }
        }
        const int64_t* cd = p->cell_dofs + p->cell_dofs_offset[c] - 1;
        for (int I = 0; I < nb * nc; ++I) f[cd[I] - 1] = f[cd[I] - 1] + fe[I];
    }
    return OR_OK;
}

// apply! for Dirichlet constraints, ConstraintHandler.jl:711-744 step by step (no affine
// constraints: _condense! returns early for them, 803-805)
int or_apply(int64_t n, const int64_t* colptr, const int64_t* rowval, double* nzval, double* f, int64_t np,
             const int64_t* pd, const double* g, int32_t applyzero) {
    auto diag = [&](int64_t c) -> int64_t {  // nzval index of K[c, c] (0-based c), -1 if absent
        for (int64_t j = colptr[c] - 1; j < colptr[c + 1] - 1; ++j)
            if (rowval[j] == c + 1) return j;
        return -1;
    };
    // meandiag (944-955): sum of |K[i, i]| in order, divided by the size
    double z = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t j = diag(i);
        z += j >= 0 ? std::fabs(nzval[j]) : 0.0;
    }
    const double m = z / (double)n;
    // f -= K * g (add_inhomogeneities_csc!, 752-767)
    if (f && !applyzero)
        for (int64_t i = 0; i < np; ++i) {
            const int64_t d = pd[i] - 1;
            const double v = g[i];
            if (v != 0)
                for (int64_t j = colptr[d] - 1; j < colptr[d + 1] - 1; ++j) {
                    const double kv = nzval[j];
                    const double t = v * kv;
                    f[rowval[j] - 1] = f[rowval[j] - 1] - t;
                }
        }
    // zero_out_columns! (931-938), zero_out_rows! (940-949)
    std::vector<char> isc((size_t)n, 0);
    for (int64_t i = 0; i < np; ++i) isc[pd[i] - 1] = 1;
    for (int64_t i = 0; i < np; ++i) {
        const int64_t d = pd[i] - 1;
        for (int64_t j = colptr[d] - 1; j < colptr[d + 1] - 1; ++j) nzval[j] = 0.0;
    }
    for (int64_t j = 0; j < colptr[n] - 1; ++j)
        if (isc[rowval[j] - 1]) nzval[j] = 0.0;
    // meandiag on the constrained diagonals, f[d] = g_d m (735-742)
    for (int64_t i = 0; i < np; ++i) {
        const int64_t d = pd[i] - 1;
        const int64_t j = diag(d);
        if (j < 0) return OR_ERR_PATTERN_MISSING;
        nzval[j] = m;
        if (f) f[d] = (applyzero ? 0.0 : g[i]) * m;
    }
    return OR_OK;
}

}  // extern "C"
