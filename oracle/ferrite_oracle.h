/*
 * ferrite_oracle.h -- CPU FP64 restatement of Ferrite.jl's assembly path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the parity checker for the CUDA engine in
 * ferrite.jl_gb300/: only tests, __graft_entry__.smoke() and bench.py's CPU baseline leg
 * may load it. The product path never calls into it.
 *
 * It restates, in plain C++ with FP64 arithmetic, the Julia code of Ferrite.jl v1.6.0:
 *   grid generation      src/Grid/grid_generators.jl:78-112, 159-257, 474-559
 *   dof distribution     src/Dofs/DofHandler.jl:493-794, 829-1057
 *   sparsity pattern     src/Dofs/sparsity_pattern.jl:223-253, 549, 1136-1249
 *   quadrature           src/Quadrature/quadrature.jl:83-154, generate_quadrature.jl:93-112,
 *                        gaussquad_tet_table.jl (Jinyun/Keast), gaussquad_prism_table.jl:6-366
 *   shape functions      src/interpolations.jl:640-661, 891-913, 1038-1164, 1258-1280
 *   CellValues reinit!   src/FEValues/CellValues.jl:110-140, GeometryMapping.jl:124-130,
 *                        FunctionValues.jl:163, 186-192
 *   element kernels      docs/src/literate-tutorials/heat_equation.jl:143-164,
 *                        docs/src/literate-howto/threaded_assembly.jl:105-132,
 *                        docs/src/literate-tutorials/hyperelasticity.jl:157-276,
 *                        docs/src/literate-gallery/topology_optimization.jl:347-383
 *   CSC assembler        src/assembler.jl:287-291, 322-457, 513-576; src/arrayutils.jl:100-152
 *   CSR assembler        ext/FerriteSparseMatrixCSR.jl:9-96
 *   element product      y = sum_c A_c^T Ke_c A_c u over the element matrices of
 *                        docs/src/literate-howto/gpu_assembly.jl:265-303 (no reference code)
 *   greedy coloring      src/Grid/coloring.jl:47-143
 *   Dirichlet apply!     src/Dofs/ConstraintHandler.jl:711-767, 931-955
 *   facet loads          src/FEValues/FacetValues.jl:129-155, facet_integrals.jl:85-273,
 *                        benchmark/helper.jl:331-348
 *
 * Conventions follow Ferrite's memory layout: node coordinates AoS [n_nodes][dim],
 * connectivity, cell_dofs, cell_dofs_offset, colptr and rowval are 1-based Int64, nzval is
 * Float64 column-major CSC.
 */
#ifndef FERRITE_ORACLE_H
#define FERRITE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cell types (Ferrite: Triangle, Quadrilateral, Tetrahedron, Hexahedron, Wedge) */
enum { OR_TRIANGLE = 1, OR_QUADRILATERAL = 2, OR_TETRAHEDRON = 3, OR_HEXAHEDRON = 4, OR_WEDGE = 5 };
/* physics (element routines of the tutorials) */
enum { OR_HEAT = 1, OR_LINEAR_ELASTIC = 2, OR_NEO_HOOKE = 3 };
/* status codes, same meaning as the library's FE_* codes */
enum { OR_OK = 0, OR_ERR_ARG = 1, OR_ERR_BOUNDS = 2, OR_ERR_DETJ = 3, OR_ERR_PATTERN_MISSING = 4,
       OR_ERR_UNSUPPORTED = 5 };

typedef struct {
    int32_t dim;
    int64_t n_nodes;
    const double* nodes;              /* [n_nodes][dim] */
    int64_t n_cells;
    const int32_t* cell_types;        /* [n_cells] */
    const int64_t* cell_nodes_offset; /* [n_cells+1], 0-based into cell_nodes */
    const int64_t* cell_nodes;        /* 1-based node ids */
    int32_t n_sdh;                    /* SubDofHandlers, visited in this order */
    const int32_t* sdh_ip_order;      /* Lagrange order per sdh */
    const int32_t* sdh_ncomp;         /* 1 = scalar field, dim = ip^dim */
    const int32_t* sdh_qr_order;      /* QuadratureRule order per sdh */
    const int64_t* sdh_cellset_offset;/* [n_sdh+1] */
    const int64_t* sdh_cellset;       /* 1-based cell ids, ascending */
    int64_t ndofs;
    const int64_t* cell_dofs;         /* flat */
    const int64_t* cell_dofs_offset;  /* [n_cells], 1-based */
    const int64_t* colptr;            /* [ndofs+1], 1-based */
    const int64_t* rowval;            /* [nnz], 1-based */
} or_problem;

typedef struct {
    int32_t physics;
    double p0, p1;       /* heat: k, source; elastic: E, nu; neo-hooke: mu, lambda */
    double body[3];      /* body force (elastic, neo-hooke) */
    const double* cell_scale; /* optional per-cell factor on the material (E_e or rho^p); NULL = 1 */
    const double* u;     /* neo-hooke: current displacement [ndofs] */
} or_physics;

typedef struct {
    int32_t code;
    int64_t cell;        /* 1-based */
    double detJ;
    int64_t row, col;    /* 1-based, pattern miss */
} or_error;

int or_grid_counts(int32_t cell_type, const int64_t* nel, int64_t* n_nodes, int64_t* n_cells,
                   int32_t* nodes_per_cell, int32_t* dim);
int or_generate_grid(int32_t cell_type, const int64_t* nel, const double* left, const double* right,
                     double* nodes, int64_t* cells);

int or_nbase(int32_t cell_type, int32_t ip_order);
int or_close_dofhandler(const or_problem* p, int64_t* cell_dofs, int64_t* cell_dofs_offset,
                        int64_t* ndofs);
int or_sparsity_pattern(const or_problem* p, int64_t* colptr, int64_t* rowval, int64_t* nnz);

int or_quadrature(int32_t cell_type, int32_t order, int32_t* n_qp, double* weights, double* points);
int or_shape_tables(int32_t cell_type, int32_t ip_order, int32_t n_qp, const double* points,
                    double* N, double* dN);

int or_assemble(const or_problem* p, const or_physics* phys, int32_t nthreads, int32_t fillzero,
                double* nzval, double* f, or_error* err);
int or_element_matrix(const or_problem* p, const or_physics* phys, int64_t cell, double* Ke,
                      double* fe, or_error* err);
int or_index_map(const or_problem* p, int64_t cell, int64_t* positions);

/* Facet (Neumann) loads: for each facet (cell, local facet number) of the set, in the given
 * order, FacetValues reinit! (src/FEValues/FacetValues.jl:129-155: J = sum_k x_k (x) dM_k at the
 * facet point, wn = weighted_normal(J, refshape, facet) (src/FEValues/facet_integrals.jl),
 * dGamma = |wn| w, n = wn / |wn|, detJ = |wn| > 0) and f[celldofs] += fe with
 * fe[(i, a)] = sum_q (N_i(q) t_a) dGamma, t = pressure n + traction (benchmark/helper.jl:331-348;
 * hyperelasticity.jl:278-290 with pressure = -tn); scalar fields: t = pressure.
 * Tables per reference facet: w [nf][nqp], N [nf][nqp][n_base], dM [nf][nqp][n_geo][rdim]. */
int or_facet_load(const or_problem* p, int64_t n, const int64_t* cells, const int32_t* facets, int32_t n_ref_facets,
                  int32_t n_qp, const double* w, const double* N, const double* dM, double pressure,
                  const double* traction, double* f, or_error* err);

/* apply!(K, f, ch, applyzero) for Dirichlet constraints (src/Dofs/ConstraintHandler.jl:711-744):
 * m = meandiag(K) (944-955, before any change); unless applyzero, f -= K * g over the prescribed
 * columns (add_inhomogeneities_csc!, 752-767, prescribed dofs in ascending order, v != 0 only);
 * zero the prescribed columns (931-938) and rows (940-949); K[d, d] = m and f[d] = g_d m (0 for
 * apply_zero!). prescribed: 1-based, ascending, unique; f may be NULL (apply!(K, ch)).
 * Returns OR_ERR_PATTERN_MISSING if a prescribed diagonal is not in the pattern. */
int or_apply(int64_t n, const int64_t* colptr, const int64_t* rowval, double* nzval, double* f,
             int64_t n_prescribed, const int64_t* prescribed, const double* inhomogeneities, int32_t applyzero);
int or_greedy_coloring(const or_problem* p, int32_t* cell_color, int32_t* n_colors);

/* Threaded colored assembly prepared once (threaded_assembly.jl:134-141, 232-265): the
 * CellValues and the coloring are built by or_threaded_create, as the how-to builds them
 * before it assembles; each or_threaded_assemble is one assemble_global! call (start_assemble
 * zeroes K and f, then the colors in order, each color's cells in equal chunks over nthreads
 * threads with per-thread CellValues and assembler buffers). The problem's arrays must stay
 * valid until or_threaded_destroy. algorithm: OR_COLORING_WORKSTREAM (Ferrite's default,
 * coloring.jl:171-264, 308) or OR_COLORING_GREEDY (coloring.jl:108-160). */
enum { OR_COLORING_GREEDY = 1, OR_COLORING_WORKSTREAM = 2 };
typedef struct or_threaded or_threaded;
int or_threaded_create(const or_problem* p, int32_t nthreads, int32_t algorithm, or_threaded** out,
                       int32_t* n_colors);
int or_threaded_colors(const or_threaded* t, int32_t* cell_color);
int or_threaded_assemble(or_threaded* t, const or_physics* phys, double* nzval, double* f, or_error* err);
void or_threaded_destroy(or_threaded* t);

/* CSR assembly (ext/FerriteSparseMatrixCSR.jl:9-96, SparseMatrixCSR{1}): as or_assemble (serial,
 * cell order) into a CSR matrix with 1-based rowptr[ndofs+1] / colval[nnz] (columns ascending
 * within a row): K[row, col] += Ke[row_local, col_local]; a pattern miss reports (row, col). */
int or_assemble_csr(const or_problem* p, const or_physics* phys, int32_t fillzero, const int64_t* rowptr,
                    const int64_t* colval, double* nzval, double* f, or_error* err);

/* Matrix-free product with element matrices (the element-assembly technique of
 * docs/src/literate-howto/gpu_assembly.jl:265-303, Kes[cell, i, j]):
 *   y (+)= sum over cells c in ascending order, c in a SubDofHandler, of A_c^T (Ke_c (A_c u)).
 * Ke_c(I, J) = ke[c*ks[0] + I*ks[1] + J*ks[2]] (c, I, J 0-based; float if fp64 == 0, else
 * double). Per cell, u_e = u[celldofs] (rounded to float when fp64 == 0) and
 * ye_I = fma(Ke(I, n-1), u_{n-1}, ... fma(Ke(I, 0), u_0, 0)) in the element precision, J
 * ascending; then y[celldofs[I]] += (double) ye_I in FP64, I ascending. fillzero: y = 0 first. */
int or_element_matvec(const or_problem* p, int32_t fp64, const void* ke, const int64_t* ks, const double* u,
                      int32_t fillzero, double* y);

/* Adjoint of the assembly (heat, linear elasticity): for Phi = lambda^T (K(X, s) u - f(X)),
 *   d_cell[c] = dscale[c] * dPhi/ds_c   (s_c = cell_scale[c], the factor on the material;
 *                                        dscale NULL = 1: the derivative w.r.t. s_c itself)
 *   d_X[n*dim + a] = dPhi/dX_{n,a}      (node coordinates)
 * Per quadrature point, with psi = sigma(u) : grad(lambda) (heat: k grad u . grad lambda) and
 * the load density fl = lambda(x_q) . b (heat: source * lambda(x_q)):
 *   dPhi/ds = sum_q dV psi / s,   dPhi/dX_k = sum_q dV Sigma grad M_k,
 *   Sigma = (psi - fl) I - grad(u)^T sigma(lambda) - grad(lambda)^T sigma(u),
 * grad M_k the physical gradient of the geometric shape function of node k. */
int or_adjoint(const or_problem* p, const or_physics* phys, const double* u, const double* lambda,
               const double* dscale, double* d_cell, double* d_X, or_error* err);

#ifdef __cplusplus
}
#endif
#endif
