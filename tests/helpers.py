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
