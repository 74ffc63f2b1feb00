"""Test helpers: build an engine handle from oracle-generated Ferrite arrays.

The oracle (oracle/oracle.py) produces exactly the arrays a Julia caller would take from
Ferrite objects: grid nodes and cells, DofHandler cell_dofs / cell_dofs_offset, the
allocate_matrix pattern, and the CellValues reference tables.
"""
import numpy as np


def subdomain_specs(fg, O, prob):
    subs = []
    for sd in prob.subdomains:
        ct = int(prob.cell_types[sd.cellset[0] - 1])
        w, pts = O.quadrature(ct, sd.qr_order)
        N, dN = O.shape_tables(ct, sd.ip_order, pts)
        M, dM = O.shape_tables(ct, 1, pts)
        idx = sd.cellset - 1
        ng = O.nbase(ct, 1)
        starts = prob.cell_nodes_offset[idx]
        cn = prob.cell_nodes[starts[:, None] + np.arange(ng)[None, :]]
        subs.append(fg.Subdomain(ct, sd.ip_order, sd.ncomp, w, N, dN, M, dM, sd.cellset, cn))
    return subs


def make_handle(fg, O, prob):
    return fg.Handle(prob.nodes, subdomain_specs(fg, O, prob), prob.cell_dofs, prob.cell_dofs_offset,
                     prob.ndofs, prob.colptr, prob.rowval, prob.n_cells)


def rel_fro(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def facet_tables(O, ct, ip_order, order):
    """FacetValues tables per reference facet, as Ferrite builds them (FacetQuadratureRule:
    src/Quadrature/quadrature.jl:214-245 with facet_to_element_transformation,
    src/FEValues/facet_integrals.jl): returns (n_ref_facets, n_qp, w [nf, nq], N [nf, nq, nb],
    dM [nf, nq, ng, dim])."""
    if ct in (O.QUADRILATERAL, O.TRIANGLE):
        x, w = np.polynomial.legendre.leggauss(order)
        if ct == O.QUADRILATERAL:
            maps = [lambda p: (p, -1.0), lambda p: (1.0, p), lambda p: (-p, 1.0), lambda p: (-1.0, -p)]
        else:
            w = w / 2
            h = lambda p: (p + 1) / 2
            maps = [lambda p: (1 - h(p), h(p)), lambda p: (0.0, 1 - h(p)), lambda p: (h(p), 0.0)]
        pts = [np.array([m(p) for p in x]) for m in maps]
    elif ct == O.HEXAHEDRON:
        w, q = O.quadrature(O.QUADRILATERAL, order)
        maps = [lambda a, b: (b, a, -1.0), lambda a, b: (a, -1.0, b), lambda a, b: (1.0, a, b),
                lambda a, b: (-a, 1.0, b), lambda a, b: (-1.0, b, a), lambda a, b: (a, b, 1.0)]
        pts = [np.array([m(a, b) for a, b in q]) for m in maps]
    elif ct == O.TETRAHEDRON:
        w, q = O.quadrature(O.TRIANGLE, order)
        maps = [lambda a, b: (1 - a - b, b, 0.0), lambda a, b: (b, 0.0, 1 - a - b), lambda a, b: (a, b, 1 - a - b),
                lambda a, b: (0.0, 1 - a - b, b)]
        pts = [np.array([m(a, b) for a, b in q]) for m in maps]
    else:
        raise ValueError("facet tables for this cell type are not built here")
    nf, nq = len(pts), len(w)
    N = np.stack([O.shape_tables(ct, ip_order, p)[0] for p in pts])
    dM = np.stack([O.shape_tables(ct, 1, p)[1] for p in pts])
    W = np.tile(np.asarray(w, float), (nf, 1))
    return nf, nq, np.ascontiguousarray(W), np.ascontiguousarray(N), np.ascontiguousarray(dM)


# local nodes of each reference facet (1-based), Ferrite's reference-element topology
# (src/Grid/grid.jl): facet f of a cell of that type
FACET_NODES = {
    2: ((1, 2), (2, 3), (3, 4), (4, 1)),                                                    # quadrilateral
    1: ((1, 2), (2, 3), (3, 1)),                                                            # triangle
    4: ((1, 4, 3, 2), (1, 2, 6, 5), (2, 3, 7, 6), (3, 4, 8, 7), (1, 5, 8, 4), (5, 6, 7, 8)),  # hexahedron
    3: ((1, 3, 2), (1, 2, 4), (2, 3, 4), (1, 4, 3)),                                        # tetrahedron
    5: ((1, 3, 2), (1, 2, 5, 4), (3, 1, 4, 6), (2, 3, 6, 5), (4, 5, 6)),                    # wedge
}


def boundary_facets(prob, ct, on_boundary, nodes=None):
    """(cells, facets), 1-based, of the facets whose nodes all satisfy on_boundary(x)."""
    x = prob.nodes if nodes is None else nodes
    cells, facets = [], []
    for c in range(prob.n_cells):
        cn = prob.cells_of(c) - 1
        for f, loc in enumerate(FACET_NODES[ct]):
            if all(on_boundary(x[cn[k - 1]]) for k in loc):
                cells.append(c + 1)
                facets.append(f + 1)
    return np.array(cells, np.int64), np.array(facets, np.int32)
