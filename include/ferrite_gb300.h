/*
 * ferrite_gb300.h -- C ABI of the GB300 (sm_103a) finite-element assembly engine.
 *
 * One call replaces Ferrite.jl's assembly hot path
 *
 *     assembler = start_assemble(K, f)                     # src/assembler.jl:287-291
 *     for cell in CellIterator(dh)                         # src/iterators.jl:248-274, 389-396
 *         reinit!(cellvalues, cell)                        # src/FEValues/CellValues.jl:122-140
 *         element_routine!(Ke, fe, cellvalues, ...)        # user code (tutorials)
 *         assemble!(assembler, celldofs(cell), Ke, fe)     # src/assembler.jl:322-457
 *     end
 *
 * with fe_assemble(), which fills the nzval of the same SparseMatrixCSC (pattern from
 * allocate_matrix(dh), src/Dofs/sparsity_pattern.jl:628-645) and the right-hand side f.
 * Everything a caller passes is plain memory in Ferrite's own layout: node coordinates as
 * Vector{Node{dim,Float64}} (AoS), connectivity / cell_dofs / cell_dofs_offset / colptr /
 * rowval as 1-based Int64, nzval and f as Float64. A Julia binding is in
 * ferrite.jl_gb300/julia/FerriteGB300.jl.
 *
 * Every function returns an int status (FE_OK = 0). Device-side failures never trap: the
 * kernels record the first failure in a status word and fe_assemble() returns its code;
 * fe_last_error() gives the details (cell id, detJ, row/col), mirroring the exceptions of
 * the reference (throw_detJ_not_pos, src/FEValues/common_values.jl:5; the missing pattern
 * entry error, src/assembler.jl:459-467; BoundsError / ArgumentError for bad input).
 *
 * Threading: like Ferrite's assemblers (src/assembler.jl:273-276) a handle is not
 * re-entrant; concurrent assemblies need separate handles. Work is queued on the stream
 * passed in fe_assemble_params.
 */
#ifndef FERRITE_GB300_H
#define FERRITE_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FE_ABI_VERSION 1

/* status codes */
#define FE_OK 0
#define FE_ERR_ARG 1             /* inconsistent sizes / bad argument (ArgumentError, DimensionMismatch) */
#define FE_ERR_BOUNDS 2          /* node / dof / cell index out of range (BoundsError) */
#define FE_ERR_DETJ 3            /* detJ <= 0 in some cell (throw_detJ_not_pos) */
#define FE_ERR_PATTERN_MISSING 4 /* a non-zero value has no entry in the pattern (assembler.jl:459-467) */
#define FE_ERR_UNSUPPORTED 5     /* element / dof layout this engine does not implement */
#define FE_ERR_CUDA 6            /* CUDA runtime error */
#define FE_ERR_OOM 7             /* device memory exhausted */
#define FE_ERR_STATE 8           /* call out of order (e.g. replay without capture) */

/* cell types (Ferrite: Triangle, Quadrilateral, Tetrahedron, Hexahedron, Wedge) */
#define FE_TRIANGLE 1
#define FE_QUADRILATERAL 2
#define FE_TETRAHEDRON 3
#define FE_HEXAHEDRON 4
#define FE_WEDGE 5

/* element routines: the ones of Ferrite's tutorials */
#define FE_HEAT 1           /* Ke += k (gradN_i . gradN_j) dOmega, fe += s N_i dOmega (heat_equation.jl:143-164) */
#define FE_LINEAR_ELASTIC 2 /* Ke += (eps_i : C : eps_j) dOmega, fe += (N_i . b) dOmega (threaded_assembly.jl:105-132) */
#define FE_NEO_HOOKE 3      /* tangent and residual of hyperelasticity.jl:157-276 (cell part) */

/* precision */
#define FE_PREC_MIXED 0 /* FP32 element math (FP64 Jacobians for flagged cells, FP64 Neo-Hooke points where the
                           deformation is near-singular or inverted); each entry's contributions summed
                           as a compensated FP32 pair (FP64-class) and rounded exactly to FP64; with FE_FP32_SUM
                           one plain FP32 sum per entry instead */
#define FE_PREC_FP64 1  /* the plain FP64 drop-in: all math and accumulation in FP64 */

/* fe_assemble flags */
#define FE_FILLZERO 1u /* zero K and f first, as start_assemble(K, f; fillzero=true) */
#define FE_NO_K 2u     /* skip K (nzval may be NULL) */
#define FE_NO_F 4u     /* skip f (f may be NULL) */
#define FE_ASYNC 8u    /* do not wait for the kernels; read the status later with fe_sync() */
#define FE_PROFILE 16u /* bracket the assembly kernel with CUDA events; read with fe_kernel_time() */
#define FE_COMPENSATED 32u /* FE_PREC_MIXED: sum each entry's contributions as a compensated FP32 pair
                              (TwoSum, FP64-class summation error) and round the pair exactly to FP64.
                              The default; the flag is accepted and changes nothing */
#define FE_TWO_PHASE 64u   /* element matrices first: one pass per cell writes Ke and fe to a device scratch
                              held by the handle, then the owner tiles load them instead of recomputing the
                              cell's geometry in every tile that owns one of its dofs. The default for
                              quadratic elements; results are bitwise those of the fused form */
#define FE_FUSED 128u      /* element math inside the owner tiles (the default for linear elements) */
#define FE_NO_TENSOR 256u  /* two-phase form: element matrices on the CUDA cores even where a tensor-core
                              kernel exists (27-node hexahedra, elasticity, mixed precision); the CUDA-core
                              form gives the fused form's bits, the tensor-core form (split TF32 products,
                              FP32 accumulation) differs from them by FP32 rounding */
#define FE_STAGED_OUTPUT 512u /* host nzval / f: assemble into a device buffer held by the handle and copy it back
                                 with the copy engine, also for page-locked memory (which by default the kernels
                                 write through its mapping); pageable memory is always staged */
#define FE_FP32_SUM 1024u     /* FE_PREC_MIXED: one plain FP32 sum per entry, rounded exactly to FP64, instead of
                                 the compensated pair (about a tenth faster; the summation error is then FP32's,
                                 ~1e-7 relative, where the element math's own FP32 rounding is of the same order) */

typedef struct fe_handle fe_handle;

typedef struct {
    int32_t dim;          /* spatial dimension, 2 or 3 */
    int64_t n_nodes;
    const double* nodes;  /* [n_nodes][dim]: the memory of grid.nodes */
    int64_t n_cells;      /* getncells(grid) */
} fe_grid_desc;

/* One SubDofHandler with its CellValues (dh.subdofhandlers[k], src/Dofs/DofHandler.jl:15-26). */
typedef struct {
    int32_t cell_type;    /* FE_* cell type of every cell in the set */
    int32_t ip_order;     /* Lagrange order of the field interpolation (1 or 2) */
    int32_t n_components; /* 1 = scalar field, dim = vectorized ip^dim (interleaved dofs) */
    int32_t n_qp;         /* quadrature points of the CellValues' QuadratureRule */
    const double* qr_weights; /* [n_qp] getweights(qr) */
    const double* N;      /* [n_qp][n_base] reference shape values (FunctionValues.Nxi of the scalar ip) */
    const double* dNdxi;  /* [n_qp][n_base][rdim] reference gradients (FunctionValues.dNdxi) */
    const double* M;      /* [n_qp][n_geo] geometric shape values (GeometryMapping.M) */
    const double* dMdxi;  /* [n_qp][n_geo][rdim] (GeometryMapping.dMdxi) */
    int64_t n_cells;
    const int64_t* cellset;    /* [n_cells] 1-based cell ids, ascending (sdh.cellset) */
    const int64_t* cell_nodes; /* [n_cells][n_geo] 1-based node ids of those cells (grid.cells[cellset]) */
} fe_subdomain_desc;

typedef struct {
    int64_t ndofs;
    const int64_t* cell_dofs;        /* dh.cell_dofs */
    const int64_t* cell_dofs_offset; /* [n_cells] 1-based, dh.cell_dofs_offset */
} fe_dof_desc;

typedef struct {
    int64_t n;             /* number of columns (= ndofs) */
    int64_t nnz;
    const int64_t* colptr; /* [n+1] 1-based (K.colptr) */
    const int64_t* rowval; /* [nnz] 1-based (K.rowval); read during fe_create only. Host or DEVICE
                              memory for fe_create (a device pattern from fe_sparsity_pattern_device or a
                              CuSparseMatrixCSC's colPtr / rowVal is copied to the host first); host
                              memory for fe_plan_dry_run */
} fe_csc_desc;
/* A SparseMatrixCSR{1} (ext/FerriteSparseMatrixCSR.jl:9-160) goes in as (K.rowptr, K.colval)
 * in place of (colptr, rowval), with its nzval as the output. Ferrite's pattern (cell
 * couplings plus the diagonal) is structurally symmetric, so its CSR arrays are its CSC
 * arrays, and every physics here has a symmetric K: the value written at row c of "column" r
 * is K[c, r], which is K[r, c] up to the rounding of Ke(I, J) against Ke(J, I). A pattern
 * miss is then reported with row and col swapped relative to the CSR (row, col). */

typedef struct {
    int32_t physics;       /* FE_HEAT, FE_LINEAR_ELASTIC, FE_NEO_HOOKE */
    int32_t precision;     /* FE_PREC_MIXED or FE_PREC_FP64 */
    uint32_t flags;        /* FE_FILLZERO | FE_NO_K | FE_NO_F | FE_ASYNC */
    double p0, p1;         /* heat: k, source; elastic: E, nu; neo-hooke: mu, lambda */
    double body[3];        /* body force b (elastic, neo-hooke) */
    const double* cell_scale; /* optional [n_cells]: per-cell factor on the material (E_e/E, rho^p), by cell id - 1 */
    const double* u;       /* neo-hooke: current solution [ndofs] */
    double cond_threshold; /* mixed precision: cells whose Jacobian condition number exceeds this
                              are recomputed in FP64 (<= 0: default 64) */
    void* stream;          /* cudaStream_t; NULL = legacy default stream */
} fe_assemble_params;

typedef struct {
    int32_t code;
    int64_t cell;          /* 1-based cell id (DETJ, PATTERN_MISSING) */
    double detJ;           /* DETJ */
    int64_t row, col;      /* PATTERN_MISSING, 1-based */
    char message[256];
} fe_error_info;

typedef struct {
    int64_t n_cells, ndofs, nnz;
    int64_t n_tiles;        /* owner tiles the nzval is partitioned into */
    int64_t n_cell_visits;  /* (cell, tile) pairs: geometry evaluations per assembly */
    int64_t n_items;        /* (cell, owned base function) work items per assembly */
    int64_t flagged_cells;  /* cell evaluations redone with FP64 Jacobians, plus Neo-Hooke quadrature points
                               redone in FP64, in the last mixed assembly (a cell is evaluated once per owner
                               tile it touches) */
    int64_t device_bytes;   /* device memory held by the handle */
    double create_seconds;  /* host time spent in fe_create */
    int32_t max_record_bytes;   /* largest tile record (shared-memory ring entry) */
    int32_t max_tile_nodes;     /* most nodes of one tile (gathered coordinates) */
    int32_t max_stage_values;   /* most staging values of one tile */
    int32_t max_out_doubles;    /* largest reduce output buffer of one tile */
    int32_t stage_cap;          /* staging capacity the plan was built with */
    uint32_t plan_checksum;     /* fe_plan_dry_run: digest of the tile records (FNV-1a 64 of each record,
                                   then of those in tile order, folded to 32 bits); equal plans, equal
                                   digests, whatever the host thread count. 0 from fe_get_info */
} fe_info;

/*
 * fe_create: validate and upload the problem, build the element-to-nzval index map
 * (bit-exact with Ferrite's assembler, src/assembler.jl:376-457) and the owner tiles.
 * Replaces the host side of start_assemble(K, f) (src/assembler.jl:287-291) together with
 * the device adaptation of grid/dh (ext/FerriteKAExt/adapt_core.jl:6-31,
 * ext/FerriteCudaExt.jl:44-48, 95-101). rowval is only read here.
 */
int fe_create(const fe_grid_desc* grid, int32_t n_subdomains, const fe_subdomain_desc* subdomains,
              const fe_dof_desc* dofs, const fe_csc_desc* pattern, fe_handle** out);

/*
 * fe_assemble: the whole `start_assemble` + `for cell in CellIterator(dh) ... assemble!`
 * loop (docs/src/literate-tutorials/heat_equation.jl:186-206,
 * docs/src/literate-howto/threaded_assembly.jl:232-265, ext/FerriteCudaExt.jl:50-93).
 * nzval [nnz] and f [ndofs] may be device or host pointers (host: staged through the
 * handle's device buffers). Same for params->u and params->cell_scale.
 */
int fe_assemble(fe_handle* h, const fe_assemble_params* params, double* nzval, double* f);

/*
 * fe_assemble_elements: element assembly without the global matrix, the "Element Assembly"
 * kernel of docs/src/literate-howto/gpu_assembly.jl:270-303 (per cell reinit!, fill!(Ke, 0),
 * assemble_element!(Ke, fe, cv) into Kes[cellid, :, :] and fes[cellid, :]). Every cell's Ke and
 * fe go to the caller's DEVICE arrays: Ke(c, I, J) at ke[c*ke_stride[0] + I*ke_stride[1] +
 * J*ke_stride[2]], fe(c, I) at fe[c*fe_stride[0] + I*fe_stride[1]], with c = cell id - 1 and
 * I, J = local dof index - 1 (Ferrite's order: vector dofs interleaved, I = n_components *
 * base function + component). Elements are float for FE_PREC_MIXED and double for
 * FE_PREC_FP64; strides count elements. The how-to's Kes = zeros(Float32, ncells, nbf, nbf)
 * (column-major) has ke_stride = {1, ncells, ncells*nbf} and fe_stride = {1, ncells}.
 * Physics, flags (FE_NO_K, FE_NO_F, FE_ASYNC, FE_PROFILE), cell_scale, u and errors (detJ) are
 * those of fe_assemble; entries of cells not in any subdomain are left untouched.
 */
typedef struct {
    int64_t ke_stride[3];
    int64_t fe_stride[2];
} fe_element_layout;

int fe_assemble_elements(fe_handle* h, const fe_assemble_params* params, void* ke, void* fe,
                         const fe_element_layout* layout);

/*
 * Matrix-free product with the element matrices of fe_assemble_elements (the element-assembly
 * technique of docs/src/literate-howto/gpu_assembly.jl:265-303, whose Kes the how-to leaves to
 * a user-written product): y (+)= sum over the cells of the handle's subdomains, in ascending
 * cell order, of A_c^T (Ke_c (A_c u)), A_c the gather of the cell's dofs.
 * fe_element_operator_create takes the element layout (ke_stride as in fe_assemble_elements;
 * fe_stride is ignored) and the precision: FE_PREC_MIXED for float Ke, FE_PREC_FP64 for double
 * Ke. It builds once the dof -> (cell, local dof) incidence in cell order and a scratch of one
 * value per (cell, local dof). fe_element_matvec, on DEVICE ke, u and y, asynchronous on
 * `stream`: per cell ye_I = sum_J Ke(I, J) u_J as fused multiply-adds in the element precision
 * (J ascending; u rounded to float for FE_PREC_MIXED), then y[dof_I] += (double) ye_I in FP64
 * in cell order; flags FE_FILLZERO sets y = 0 first. Deterministic, no atomics: bitwise the
 * serial loop over cells. fe_element_matvec only launches kernels (no host work, no
 * allocation), so a Krylov loop can capture it in a CUDA graph. The caller keeps ke covering
 * every cell the strides address.
 * Destroy the operator before its handle.
 */
typedef struct fe_element_operator fe_element_operator;
int fe_element_operator_create(fe_handle* h, const fe_element_layout* layout, int32_t precision,
                               fe_element_operator** out);
int fe_element_matvec(fe_element_operator* op, const void* ke, const double* u, double* y, uint32_t flags,
                      void* stream);
void fe_element_operator_destroy(fe_element_operator* op);

/*
 * Dirichlet constraints on the assembled matrix: apply!(K, f, ch) and apply_zero!(K, f, ch)
 * (src/Dofs/ConstraintHandler.jl:711-744; device form ext/FerriteKAExt/constraints.jl:40-148).
 * fe_dirichlet_create takes the closed handler's prescribed dofs (ch.prescribed_dofs: 1-based,
 * ascending, unique) and K.rowval (host, 1-based, the pattern of fe_create), and works out once
 * which nzval entries each step touches. fe_apply, on DEVICE nzval and f (f may be NULL, as in
 * apply!(K, ch)), in the reference's order: m = meandiag(K); unless applyzero,
 * f -= K * g over the prescribed columns (g = inhomogeneities, host or device, ch.inhomogeneities;
 * NULL: all zero); zero the prescribed columns and rows; K[d, d] = m; f[d] = g_d * m (0 for
 * apply_zero!). Asynchronous on `stream`; deterministic (no atomics); f -= K g is bitwise the
 * reference's per-row operation order, m is a fixed-order parallel sum. A prescribed dof
 * without a diagonal entry in the pattern is FE_ERR_PATTERN_MISSING at creation. Destroy the
 * constraints before their handle.
 */
/*
 * Facet (Neumann) loads: FacetValues on a facet set (src/FEValues/FacetValues.jl:129-155) and
 * f[celldofs] += fe, fe[(i, a)] = sum_q (N_i t_a) dGamma with t = pressure n + traction (vector
 * fields; the pressure load of benchmark/helper.jl:331-348, the traction of
 * hyperelasticity.jl:278-290 with pressure = -tn), t = pressure for scalar fields (a flux).
 * dGamma = |weighted normal| w and n its direction, the weighted normal being Ferrite's
 * (src/FEValues/facet_integrals.jl) from the cell's Jacobian at the facet point. The caller
 * passes the FacetValues tables per reference facet (pad a facet's rule with zero weights when
 * the facets' rules differ in length) and the set's (cell, local facet) pairs, all of one
 * subdomain. FP64; facets are added in the given order, so the result is that of a serial
 * FP64 loop. fe_assemble_facet_load: f is DEVICE memory; flags FE_FILLZERO; synchronous.
 */
typedef struct {
    int32_t n_qp;            /* points per facet (FacetQuadratureRule), <= 32 */
    int32_t n_ref_facets;    /* nfacets of the reference shape */
    const double* qr_weights;/* [n_ref_facets][n_qp] */
    const double* N;         /* [n_ref_facets][n_qp][n_base] field shape values at the facet points */
    const double* dMdxi;     /* [n_ref_facets][n_qp][n_geo][dim] geometric shape gradients there */
    int64_t n_facets;
    const int64_t* cells;    /* [n_facets] 1-based cell ids (FacetIndex) */
    const int32_t* facets;   /* [n_facets] 1-based local facet numbers */
} fe_facet_desc;
typedef struct fe_facet_set fe_facet_set;
int fe_facet_set_create(fe_handle* h, const fe_facet_desc* desc, fe_facet_set** out);
int fe_assemble_facet_load(fe_facet_set* set, double pressure, const double* traction, uint32_t flags, double* f, void* stream);
void fe_facet_set_destroy(fe_facet_set* set);

typedef struct fe_dirichlet fe_dirichlet;
int fe_dirichlet_create(fe_handle* h, const int64_t* rowval, int64_t n_prescribed, const int64_t* prescribed_dofs,
                        fe_dirichlet** out);
int fe_apply(fe_dirichlet* ch, double* nzval, double* f, const double* inhomogeneities, int32_t applyzero, void* stream);
void fe_dirichlet_destroy(fe_dirichlet* ch);

/* Wait for queued work of the handle and return the status of the last assembly. */
int fe_sync(fe_handle* h);

/* Details of the last failure (src/FEValues/common_values.jl:5, src/assembler.jl:459-467).
 * h == NULL: the last failed fe_create() of the calling thread. */
int fe_last_error(const fe_handle* h, fe_error_info* out);

int fe_get_info(const fe_handle* h, fe_info* out);

/*
 * fe_get_index_map: 1-based nzval positions of the element entries of one cell, in the
 * layout of Ke (positions[J*ld + I] for Ke[I, J], ld = ndofs_per_cell); 0 where the
 * pattern has no entry. Equals the positions Ferrite's merge walk
 * (src/assembler.jl:376-457) visits for celldofs(cell).
 */
int fe_get_index_map(const fe_handle* h, int64_t cell, int64_t* positions);

/*
 * fe_plan_dry_run: everything fe_create does on the host (validation, index map, owner
 * tiles and their bounds check) without touching a device; fills n_tiles, n_cell_visits,
 * n_items. Lets a caller check its arrays, or size a problem, on a machine without a GPU.
 */
int fe_plan_dry_run(const fe_grid_desc* grid, int32_t n_subdomains, const fe_subdomain_desc* subdomains,
                    const fe_dof_desc* dofs, const fe_csc_desc* pattern, fe_info* out);

/*
 * Host-side set-up in Ferrite's numbering, for callers that do not hold Ferrite objects.
 * Only cell_type, ip_order, n_components, n_cells, cellset and cell_nodes of the subdomain
 * descriptors are read (the reference tables may be NULL).
 *
 * fe_distribute_dofs: close!(dh) for one field (src/Dofs/DofHandler.jl:493-794). cell_dofs
 * must hold sum(n_cells * n_base * n_components) entries; cell_dofs_offset [grid->n_cells]
 * receives 1-based offsets (0 for cells in no subdomain).
 * fe_sparsity_pattern: allocate_matrix(dh) (src/Dofs/sparsity_pattern.jl:223-253, 549):
 * call with rowval == NULL to get colptr [ndofs+1] and nnz, then again with rowval [nnz].
 */
int fe_distribute_dofs(const fe_grid_desc* grid, int32_t n_subdomains, const fe_subdomain_desc* subdomains,
                       int64_t* cell_dofs, int64_t* cell_dofs_offset, int64_t* ndofs);
int fe_sparsity_pattern(const fe_grid_desc* grid, int32_t n_subdomains, const fe_subdomain_desc* subdomains,
                        const fe_dof_desc* dofs, int64_t* colptr, int64_t* rowval, int64_t* nnz);
/* fe_sparsity_pattern on the device: the same arrays (bit for bit), built by GPU kernels; colptr
 * and rowval may be host or device memory (device arrays are written in place, e.g. the
 * colPtr/rowVal of a CuSparseMatrixCSC). Same two-call protocol. */
int fe_sparsity_pattern_device(const fe_grid_desc* grid, int32_t n_subdomains, const fe_subdomain_desc* subdomains,
                               const fe_dof_desc* dofs, int64_t* colptr, int64_t* rowval, int64_t* nnz);

/* Device time of the assembly kernels launched with FE_PROFILE since the last call: waits
 * for them, returns the summed milliseconds and the number of launches, then resets. */
int fe_kernel_time(fe_handle* h, double* total_ms, int64_t* launches);

/*
 * fe_assemble_noalloc: fe_assemble for callers that cannot allocate device memory -- for
 * instance code running where cudaMalloc is forbidden or would synchronize the device, such
 * as an allocator-less embedding of the solver loop. No counterpart in the reference (Ferrite
 * has no device allocation concerns on this path).
 * It allocates nothing: nzval, f, u and cell_scale must already be device memory (host
 * buffers are rejected with FE_ERR_ARG, since they would need staging copies), and the FP32
 * copies of u and of cell_scale that mixed precision uses live in one static device array of
 * 4,194,304 floats (16 MiB) that every GPU loading this library holds until exit. Problems
 * needing more (ndofs for FE_NEO_HOOKE plus n_cells when cell_scale is given) are rejected
 * with FE_ERR_ARG. The call makes the handle's device current (cudaSetDevice); the first call
 * on a device looks up that array's address there (cudaGetSymbolAddress), so make that first
 * call before any stream capture. All calls share the array, which keeps the last call's
 * values (each call overwrites what it reads): calls that overlap on the GPU (other streams,
 * other handles) race on it. Without FE_ASYNC the call waits for its stream, so it returns
 * FE_ERR_STATE on a stream that is capturing; with FE_ASYNC its status is read at the next
 * fe_sync. An earlier FE_ASYNC assembly on the handle that failed returns its error here
 * before anything is launched. FE_PROFILE is not supported here.
 */
int fe_assemble_noalloc(fe_handle* h, const fe_assemble_params* params, double* nzval, double* f);

/* Adjoint of the assembly: vector-Jacobian products of Phi = lambda^T (K(X, s) u - f(X)).
 * No counterpart in the reference (Ferrite has no adjoint); the Julia binding exposes it as the
 * pullback of residual(h, K, s, u) = K(s) u - f (a ChainRulesCore.rrule), replacing
 * differentiation of the cell loop of docs/src/literate-gallery/topology_optimization.jl:347-383
 * (SIMP: s_e = rho_e^p).
 *   physics      FE_HEAT (p0 = k, p1 = source) or FE_LINEAR_ELASTIC (p0 = E, p1 = nu, body)
 *   cell_scale   per Ferrite cell material factor s_e (E_e = s_e p0; NULL = 1)
 *   dscale       per Ferrite cell ds_e/drho_e (NULL = 1: d_rho is then dPhi/ds_e)
 *   d_rho[n_cells]        = dscale_e * lambda_e^T (dK_e/ds_e) u_e  (0 for cells outside the subdomains)
 *   d_X[n_nodes * dim]    = dPhi/dX, node-major like grid.nodes (NULL: skipped)
 * Quadrature-point geometry is recomputed, not stored. FE_PREC_MIXED computes each cell in FP32
 * and sums the cells of a node in FP64; FE_PREC_FP64 is FP64 throughout. Deterministic. u,
 * lambda (ndofs), cell_scale, dscale and the outputs may be host or device memory. Errors:
 * FE_ERR_DETJ as fe_assemble; FE_ERR_UNSUPPORTED for element kinds without an adjoint kernel
 * (second-order elements, Neo-Hooke). */
typedef struct {
    int32_t physics;
    int32_t precision;
    uint32_t flags;           /* FE_ASYNC */
    double p0, p1;
    double body[3];
    const double* cell_scale;
    const double* dscale;
    void* stream;
} fe_adjoint_params;

int fe_assemble_adjoint(fe_handle* h, const fe_adjoint_params* params, const double* u, const double* lambda,
                        double* d_rho, double* d_X);

/* CUDA graphs of repeated assemblies (Newton-style re-assembly: the same pattern, new u).
 * fe_graph_capture records n_steps fe_assemble calls (steps[k] with nzval[k], f[k]; all
 * buffers device memory; different steps may use different u or outputs) into one CUDA graph on
 * `stream` (a created stream). It first runs each step once, uncaptured, so element errors are
 * reported here and the graph needs no allocation. fe_graph_replay launches the graph: it
 * re-reads the buffers' current contents, so updating u in place between replays re-assembles
 * with the new u. The device status (detJ, pattern misses) is reset at the start of a replay and
 * covers all its steps; fe_sync / a synchronous replay reports it. FE_ASYNC and FE_PROFILE
 * (bracketing the whole replay) are honoured by fe_graph_replay.
 * No counterpart in the reference: it replaces the repeated start_assemble + cell-loop passes of
 * a Newton iteration (docs/src/literate-tutorials/hyperelasticity.jl:386-420). */
int fe_graph_capture(fe_handle* h, void* stream, int32_t n_steps, const fe_assemble_params* steps, double* const* nzval,
                     double* const* f, int32_t* graph);
int fe_graph_replay(fe_handle* h, int32_t graph, void* stream, uint32_t flags);
int fe_graph_destroy(fe_handle* h, int32_t graph);

/* Autotuner of the tile plan and of the assembly form per cell type: for each candidate
 * staging capacity (values per tile, which sets the tile size and hence the cells recomputed
 * at tile borders and the CTAs that fit per SM), re-plan the handle and time `reps` assemblies
 * of `params` (after one warm-up) with CUDA events for each form mask: bit s set = subdomain s
 * (one SubDofHandler, one cell type) in the two-phase form, clear = fused. If params->flags
 * names FE_FUSED or FE_TWO_PHASE only that form is timed, else every mask. The fastest plan is
 * kept, and its form is used by later calls with the same physics and precision that name no
 * form. stage_caps NULL: a built-in candidate list. Per capacity, ms and form_mask are those
 * of its fastest form; candidates whose tiles do not fit shared memory are skipped (ms = -1).
 * nzval and f receive the assembled values. No counterpart in the reference. */
#define FE_TUNE_MAX 16
typedef struct {
    int32_t n_candidates;
    int32_t stage_cap[FE_TUNE_MAX];
    double ms[FE_TUNE_MAX];            /* per assembly, -1 = not run */
    int64_t n_tiles[FE_TUNE_MAX];
    int64_t n_cell_visits[FE_TUNE_MAX];
    int32_t best_stage_cap;
    double best_ms;
    uint32_t form_mask[FE_TUNE_MAX];   /* fastest form per capacity (bit s: subdomain s two-phase) */
    uint32_t best_form_mask;
} fe_tune_result;

int fe_autotune(fe_handle* h, const fe_assemble_params* params, double* nzval, double* f, int32_t n_candidates,
                const int32_t* stage_caps, int32_t reps, fe_tune_result* out);

void fe_destroy(fe_handle* h);

int fe_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
