"""Host-side set-up mirroring Ferrite's API, for callers without Ferrite objects.

    grid = generate_grid(HEXAHEDRON, (128, 128, 128), (0, 0, 0), (1, 1, 1))   # grid_generators.jl
    dh = DofHandler(grid); dh.add(ip_order=1, n_components=3); dh.close()      # DofHandler.jl
    colptr, rowval = dh.allocate_matrix()                                     # sparsity_pattern.jl
    cv = CellValues(HEXAHEDRON, ip_order=1, qr_order=2)                       # CellValues.jl
    handle = dh.handle(cv)                                                    # -> fe_create

Grids are generated with numpy in Ferrite's node and cell numbering; dof distribution and the
pattern call the library's native fe_distribute_dofs / fe_sparsity_pattern. A Julia caller
passes Ferrite's own arrays to fe_create instead.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import (DofDesc, GridDesc, Handle, Subdomain, SubdomainDesc, FEError, ErrorInfo, lib, _as_f64, _as_i64,
               i64p, f64p, TRIANGLE, QUADRILATERAL, TETRAHEDRON, HEXAHEDRON, WEDGE, FE_OK)

REF_DIM = {TRIANGLE: 2, QUADRILATERAL: 2, TETRAHEDRON: 3, HEXAHEDRON: 3, WEDGE: 3}
N_GEO = {TRIANGLE: 3, QUADRILATERAL: 4, TETRAHEDRON: 4, HEXAHEDRON: 8, WEDGE: 6}


# ---------------------------------------------------------------------------------------
# grids (src/Grid/grid_generators.jl)
# ---------------------------------------------------------------------------------------
@dataclass
class Grid:
    cell_type: int
    nodes: np.ndarray   # [n_nodes, dim] float64
    cells: np.ndarray   # [n_cells, n_geo] int64, 1-based

    @property
    def dim(self):
        return self.nodes.shape[1]

    @property
    def n_cells(self):
        return self.cells.shape[0]


def _box_nodes(counts: Sequence[int], left, right):
    """_generate_nodes with the Q1 corner map: x = sum_k M_k(xi) corner_k, first index
    fastest; xi = 2*(i-1)/(n-1) - 1 per direction."""
    d = len(counts)
    left = np.asarray(left, float)
    right = np.asarray(right, float)
    A = (right - left) / 2.0
    if d == 2:
        refc = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], float)
    else:
        refc = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                         [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], float)
    corners = left[None, :] + A[None, :] * (refc + 1.0)
    axes = [2.0 * np.arange(n, dtype=float) / float(n - 1) - 1.0 for n in counts]
    mesh = np.meshgrid(*axes, indexing="ij")
    xi = [m.transpose(tuple(range(d))[::-1]).reshape(-1) for m in mesh]  # first index fastest
    x = np.zeros((xi[0].size, d))
    for k in range(len(refc)):
        M = np.ones_like(xi[0])
        for a in range(d):
            M = M * (1.0 + refc[k, a] * xi[a])
        M = M / (4.0 if d == 2 else 8.0)
        x += M[:, None] * corners[k][None, :]
    return x


def generate_grid(cell_type: int, nel: Sequence[int], left=None, right=None) -> Grid:
    """``generate_grid(CellType, nel, left, right)`` with Ferrite's node/cell numbering."""
    d = len(nel)
    left = np.full(d, -1.0) if left is None else np.asarray(left, float)
    right = np.full(d, 1.0) if right is None else np.asarray(right, float)
    nodes = _box_nodes([n + 1 for n in nel], left, right)
    if d == 2:
        nx = nel[0] + 1
        j, i = np.meshgrid(np.arange(nel[1]), np.arange(nel[0]), indexing="ij")
        i, j = i.reshape(-1), j.reshape(-1)
        n1 = i + j * nx + 1
        n2, n3, n4 = n1 + 1, n1 + 1 + nx, n1 + nx
        if cell_type == QUADRILATERAL:
            cells = np.stack([n1, n2, n3, n4], 1)
        elif cell_type == TRIANGLE:
            cells = np.stack([np.stack([n1, n2, n4], 1), np.stack([n2, n3, n4], 1)], 1).reshape(-1, 3)
        else:
            raise ValueError("2D cell type must be QUADRILATERAL or TRIANGLE")
        return Grid(cell_type, nodes, cells.astype(np.int64))
    nx, ny = nel[0] + 1, nel[1] + 1
    k, j, i = np.meshgrid(np.arange(nel[2]), np.arange(nel[1]), np.arange(nel[0]), indexing="ij")
    i, j, k = i.reshape(-1), j.reshape(-1), k.reshape(-1)
    base = i + j * nx + k * nx * ny + 1
    v = np.stack([base, base + 1, base + 1 + nx, base + nx,
                  base + nx * ny, base + 1 + nx * ny, base + 1 + nx + nx * ny, base + nx + nx * ny], 1)
    if cell_type == HEXAHEDRON:
        cells = v
    elif cell_type == TETRAHEDRON:  # 6 per cube (grid_generators.jl:506-511)
        T = np.array([[1, 2, 4, 8], [1, 5, 2, 8], [2, 3, 4, 8], [2, 7, 3, 8], [2, 5, 6, 8], [2, 6, 7, 8]]) - 1
        cells = v[:, T].reshape(-1, 4)
    elif cell_type == WEDGE:  # 2 per cube (grid_generators.jl:218-233)
        W = np.array([[1, 2, 4, 5, 6, 8], [2, 3, 4, 6, 7, 8]]) - 1
        cells = v[:, W].reshape(-1, 6)
    else:
        raise ValueError("unsupported 3D cell type")
    return Grid(cell_type, nodes, np.ascontiguousarray(cells, dtype=np.int64))


def perturb_interior(grid: Grid, nel, amplitude: float, seed: int, left=None, right=None) -> Grid:
    """Seeded i.i.d. uniform perturbation of the interior nodes, +-amplitude*h per axis."""
    x = grid.nodes.copy()
    d = x.shape[1]
    lo = x.min(0) if left is None else np.asarray(left, float)
    hi = x.max(0) if right is None else np.asarray(right, float)
    h = (hi - lo) / np.asarray(nel, float)
    tol = 1e-9 * (hi - lo)
    inner = np.all((x > lo + tol) & (x < hi - tol), axis=1)
    rng = np.random.default_rng(seed)
    x[inner] += rng.uniform(-1.0, 1.0, size=(int(inner.sum()), d)) * (amplitude * h)
    return Grid(grid.cell_type, x, grid.cells)


# ---------------------------------------------------------------------------------------
# quadrature and reference shape functions (src/Quadrature, src/interpolations.jl)
# ---------------------------------------------------------------------------------------
def quadrature_rule(cell_type: int, order: int):
    """``QuadratureRule{RefShape}(order)`` -> (weights [nq], points [nq, rdim])."""
    if cell_type in (QUADRILATERAL, HEXAHEDRON):
        p, w = np.polynomial.legendre.leggauss(order)
        d = REF_DIM[cell_type]
        idx = np.array(np.meshgrid(*[np.arange(order)] * d, indexing="ij")).reshape(d, -1)[::-1]  # xi_1 fastest
        pts = p[idx].T
        wts = np.prod(w[idx], axis=0)
        return wts, np.ascontiguousarray(pts)
    if cell_type == TETRAHEDRON:
        if order == 1:
            return np.array([1 / 6]), np.array([[0.25, 0.25, 0.25]])
        if order == 2:
            a, b = (5 + 3 * np.sqrt(5)) / 20, (5 - np.sqrt(5)) / 20
            return np.full(4, 1 / 24), np.array([[a, b, b], [b, a, b], [b, b, a], [b, b, b]])
    if cell_type == TRIANGLE:
        if order == 1:
            return np.array([0.5]), np.array([[1 / 3, 1 / 3]])
        if order == 2:
            return np.full(3, 1 / 6), np.array([[2 / 3, 1 / 6], [1 / 6, 2 / 3], [1 / 6, 1 / 6]])
    if cell_type == WEDGE:
        if order == 1:
            return np.array([0.5]), np.array([[1 / 3, 1 / 3, 0.5]])
        if order == 2:
            # Witherden & Vincent (2015) 5-point rule on [-1,1]^3, mapped to the unit prism
            t, z, w1 = -1 / 3, 0.99999999999999985119303811076522004183, 0.66666666666666686507594918564641756458
            a, b, w2 = -0.74158162379719638007464124598498266439, 0.48316324759439276014928249196996532878, \
                0.88888888888888875661603387623572162361
            xw = np.array([[t, t, -z, w1], [t, t, z, w1], [a, b, 0, w2], [b, a, 0, w2], [a, a, 0, w2]])
            return xw[:, 3] / 8.0, (xw[:, :3] + 1.0) / 2.0
    raise ValueError(f"no quadrature rule of order {order} for cell type {cell_type}")


def _phi(k, x):
    return [-x * (1 - x) / 2, (1 + x) * (1 - x), x * (1 + x) / 2][k]


def _dphi(k, x):
    return [x - 0.5, -2 * x, x + 0.5][k]


# vtkTriQuadraticHexahedron ordering (interpolations.jl:1073-1164): per node the 1D factors
_Q2HEX = [(0, 0, 0), (2, 0, 0), (2, 2, 0), (0, 2, 0), (0, 0, 2), (2, 0, 2), (2, 2, 2), (0, 2, 2),
          (1, 0, 0), (2, 1, 0), (1, 2, 0), (0, 1, 0), (1, 0, 2), (2, 1, 2), (1, 2, 2), (0, 1, 2),
          (0, 0, 1), (2, 0, 1), (2, 2, 1), (0, 2, 1),
          (1, 1, 0), (1, 0, 1), (2, 1, 1), (1, 2, 1), (0, 1, 1), (1, 1, 2), (1, 1, 1)]
_Q2QUAD = [(0, 0), (2, 0), (2, 2), (0, 2), (1, 0), (2, 1), (1, 2), (0, 1), (1, 1)]


def shape_tables(cell_type: int, order: int, points):
    """Reference values N [nq, nb] and gradients dN [nq, nb, rdim] of Lagrange{shape, order}."""
    P = np.asarray(points, float)
    nq = P.shape[0]
    x = P[:, 0]
    y = P[:, 1]
    z = P[:, 2] if P.shape[1] > 2 else None
    one, zero = np.ones(nq), np.zeros(nq)
    if cell_type == QUADRILATERAL and order == 1:
        s = [(-1, -1), (1, -1), (1, 1), (-1, 1)]
        N = [(1 + a * x) * (1 + b * y) / 4 for a, b in s]
        G = [[a * (1 + b * y) / 4, (1 + a * x) * b / 4] for a, b in s]
    elif cell_type == QUADRILATERAL and order == 2:
        N = [_phi(a, x) * _phi(b, y) for a, b in _Q2QUAD]
        G = [[_dphi(a, x) * _phi(b, y), _phi(a, x) * _dphi(b, y)] for a, b in _Q2QUAD]
    elif cell_type == HEXAHEDRON and order == 1:
        s = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]
        N = [(1 + a * x) * (1 + b * y) * (1 + c * z) / 8 for a, b, c in s]
        G = [[a * (1 + b * y) * (1 + c * z) / 8, (1 + a * x) * b * (1 + c * z) / 8,
              (1 + a * x) * (1 + b * y) * c / 8] for a, b, c in s]
    elif cell_type == HEXAHEDRON and order == 2:
        N = [_phi(a, x) * _phi(b, y) * _phi(c, z) for a, b, c in _Q2HEX]
        G = [[_dphi(a, x) * _phi(b, y) * _phi(c, z), _phi(a, x) * _dphi(b, y) * _phi(c, z),
              _phi(a, x) * _phi(b, y) * _dphi(c, z)] for a, b, c in _Q2HEX]
    elif cell_type == TETRAHEDRON and order == 1:
        N = [1 - x - y - z, x, y, z]
        G = [[-one, -one, -one], [one, zero, zero], [zero, one, zero], [zero, zero, one]]
    elif cell_type == TRIANGLE and order == 1:
        N = [x, y, 1 - x - y]
        G = [[one, zero], [zero, one], [-one, -one]]
    elif cell_type == WEDGE and order == 1:
        N = [1 - x - y - z * (1 - x - y), x * (1 - z), y * (1 - z), z * (1 - x - y), x * z, y * z]
        G = [[-1 + z, -1 + z, -(1 - x - y)], [1 - z, zero, -x], [zero, 1 - z, -y],
             [-z, -z, 1 - x - y], [z, zero, x], [zero, z, y]]
    else:
        raise ValueError("unsupported interpolation")
    Nt = np.stack([np.broadcast_to(n, (nq,)) for n in N], 1)
    Gt = np.stack([np.stack([np.broadcast_to(g, (nq,)) for g in gi], 1) for gi in G], 1)
    return np.ascontiguousarray(Nt, float), np.ascontiguousarray(Gt, float)


@dataclass
class CellValues:
    """``CellValues(qr, ip)``: the reference tables the engine needs."""
    cell_type: int
    ip_order: int
    qr_order: int

    def __post_init__(self):
        self.weights, self.points = quadrature_rule(self.cell_type, self.qr_order)
        self.N, self.dNdxi = shape_tables(self.cell_type, self.ip_order, self.points)
        self.M, self.dMdxi = shape_tables(self.cell_type, 1, self.points)


def _facet_points(cell_type: int, order: int):
    """FacetQuadratureRule{RefShape}(order) (src/Quadrature/quadrature.jl:214-245): per reference
    facet, (weights [nq], points [nq, rdim] in cell reference coordinates), the facet rule
    mapped by Ferrite's facet_to_element_transformation (src/FEValues/facet_integrals.jl)."""
    if cell_type in (QUADRILATERAL, TRIANGLE):
        x, w = np.polynomial.legendre.leggauss(order)
        if cell_type == QUADRILATERAL:
            maps = [lambda p: (p, -1.0), lambda p: (1.0, p), lambda p: (-p, 1.0), lambda p: (-1.0, -p)]
            return [(w, np.array([m(p) for p in x])) for m in maps]
        h = (x + 1) / 2  # the facet parameter on (0, 1): half the length, half the weights
        maps = [lambda t: (1 - t, t), lambda t: (0.0, 1 - t), lambda t: (t, 0.0)]
        return [(w / 2, np.array([m(t) for t in h])) for m in maps]
    if cell_type == HEXAHEDRON:
        w, q = quadrature_rule(QUADRILATERAL, order)
        maps = [lambda a, b: (b, a, -1.0), lambda a, b: (a, -1.0, b), lambda a, b: (1.0, a, b),
                lambda a, b: (-a, 1.0, b), lambda a, b: (-1.0, b, a), lambda a, b: (a, b, 1.0)]
        return [(w, np.array([m(a, b) for a, b in q])) for m in maps]
    if cell_type == TETRAHEDRON:
        w, q = quadrature_rule(TRIANGLE, order)
        maps = [lambda a, b: (1 - a - b, b, 0.0), lambda a, b: (b, 0.0, 1 - a - b), lambda a, b: (a, b, 1 - a - b),
                lambda a, b: (0.0, 1 - a - b, b)]
        return [(w, np.array([m(a, b) for a, b in q])) for m in maps]
    if cell_type == WEDGE:
        # triangle facets 1 and 5 take the triangle rule; quadrilateral facets 2-4 the Gauss rule
        # on (-1, 1)^2 mapped to (0, 1)^2, a quarter of the area, so a quarter of the weights
        # (src/Quadrature/quadrature.jl:240-249)
        wt, qt = quadrature_rule(TRIANGLE, order)
        wq, qq = quadrature_rule(QUADRILATERAL, order)
        tri = {1: lambda x, y: (1 - x - y, y, 0.0), 5: lambda x, y: (y, 1 - x - y, 1.0)}
        quad = {2: lambda x, y: ((1 + x) / 2, 0.0, (1 + y) / 2), 3: lambda x, y: (0.0, 1 - (1 + x) / 2, (1 + y) / 2),
                4: lambda x, y: (1 - (1 + x) / 2, (1 + x) / 2, (1 + y) / 2)}
        rules = []
        for fct in range(1, 6):
            if fct in tri:
                rules.append((np.asarray(wt, float), np.array([tri[fct](a, b) for a, b in qt])))
            else:
                rules.append((np.asarray(wq, float) / 4, np.array([quad[fct](a, b) for a, b in qq])))
        return _pad_rules(rules)
    raise ValueError(f"no facet rule for cell type {cell_type}")


def _pad_rules(rules):
    """Rules of different lengths padded to the longest with zero weights (the last point
    repeated), as fe_facet_set_create takes them."""
    nq = max(len(w) for w, _ in rules)
    out = []
    for w, p in rules:
        k = nq - len(w)
        out.append((np.concatenate([w, np.zeros(k)]), np.concatenate([p, np.repeat(p[-1:], k, axis=0)])))
    return out


def facet_values(cell_type: int, ip_order: int, qr_order: int):
    """``FacetValues(FacetQuadratureRule(qr_order), ip)``: the tables fe_facet_set_create takes,
    (n_ref_facets, n_qp, w [nf, nq], N [nf, nq, nb], dMdxi [nf, nq, ng, rdim])."""
    rules = _facet_points(cell_type, qr_order)
    nf, nq = len(rules), len(rules[0][0])
    W = np.stack([np.asarray(w, float) for w, _ in rules])
    N = np.stack([shape_tables(cell_type, ip_order, p)[0] for _, p in rules])
    dM = np.stack([shape_tables(cell_type, 1, p)[1] for _, p in rules])
    return nf, nq, np.ascontiguousarray(W), np.ascontiguousarray(N), np.ascontiguousarray(dM)


# ---------------------------------------------------------------------------------------
# DofHandler + pattern (native)
# ---------------------------------------------------------------------------------------
class DofHandler:
    """``DofHandler(grid)`` with one field over one or more SubDofHandlers."""

    def __init__(self, nodes, n_cells: int):
        self.nodes = _as_f64(nodes)
        self.n_cells = int(n_cells)
        self.subs: List[dict] = []
        self.cell_dofs = None
        self.cell_dofs_offset = None
        self.ndofs = 0

    @classmethod
    def from_grid(cls, grid: Grid, ip_order: int = 1, n_components: int = 1):
        dh = cls(grid.nodes, grid.n_cells)
        dh.add(grid.cell_type, grid.cells, np.arange(1, grid.n_cells + 1), ip_order, n_components)
        return dh

    def add(self, cell_type: int, cell_nodes, cellset, ip_order: int, n_components: int):
        self.subs.append(dict(cell_type=cell_type, cell_nodes=_as_i64(cell_nodes), cellset=_as_i64(cellset),
                              ip_order=ip_order, n_components=n_components))

    def _descs(self):
        d = (SubdomainDesc * len(self.subs))()
        for k, s in enumerate(self.subs):
            d[k].cell_type, d[k].ip_order, d[k].n_components = s["cell_type"], s["ip_order"], s["n_components"]
            d[k].n_cells = len(s["cellset"])
            d[k].cellset = s["cellset"].ctypes.data_as(i64p)
            d[k].cell_nodes = s["cell_nodes"].ctypes.data_as(i64p)
        g = GridDesc(self.nodes.shape[1], self.nodes.shape[0], self.nodes.ctypes.data_as(f64p), self.n_cells)
        return g, d

    def _nbase(self, s):
        ct, o = s["cell_type"], s["ip_order"]
        if o == 1:
            return N_GEO[ct]
        return {HEXAHEDRON: 27, QUADRILATERAL: 9}[ct]

    def close(self):
        """``close!(dh)`` via fe_distribute_dofs."""
        total = sum(self._nbase(s) * s["n_components"] * len(s["cellset"]) for s in self.subs)
        self.cell_dofs = np.zeros(total, np.int64)
        self.cell_dofs_offset = np.zeros(self.n_cells, np.int64)
        nd = ctypes.c_int64()
        g, d = self._descs()
        rc = lib().fe_distribute_dofs(ctypes.byref(g), len(self.subs), d, self.cell_dofs.ctypes.data_as(i64p),
                                      self.cell_dofs_offset.ctypes.data_as(i64p), ctypes.byref(nd))
        if rc != FE_OK:
            raise FEError(rc)
        self.ndofs = nd.value
        return self

    def allocate_matrix(self, device: bool = False):
        """``allocate_matrix(dh)`` via fe_sparsity_pattern: (colptr, rowval), 1-based Int64
        numpy arrays. device=True builds it with fe_sparsity_pattern_device (GPU kernels) into
        torch CUDA tensors."""
        g, d = self._descs()
        dd = DofDesc(self.ndofs, self.cell_dofs.ctypes.data_as(i64p), self.cell_dofs_offset.ctypes.data_as(i64p))
        nnz = ctypes.c_int64()
        L = lib()
        fn = L.fe_sparsity_pattern_device if device else L.fe_sparsity_pattern
        if device:
            import torch
            colptr = torch.zeros(self.ndofs + 1, dtype=torch.int64, device="cuda")
            ptr = lambda t: ctypes.cast(t.data_ptr(), i64p)
        else:
            colptr = np.zeros(self.ndofs + 1, np.int64)
            ptr = lambda t: t.ctypes.data_as(i64p)
        rc = fn(ctypes.byref(g), len(self.subs), d, ctypes.byref(dd), ptr(colptr), None, ctypes.byref(nnz))
        if rc != FE_OK:
            raise FEError(rc)
        if device:
            rowval = torch.empty(nnz.value, dtype=torch.int64, device="cuda")
        else:
            rowval = np.empty(nnz.value, np.int64)
        rc = fn(ctypes.byref(g), len(self.subs), d, ctypes.byref(dd), ptr(colptr), ptr(rowval), ctypes.byref(nnz))
        if rc != FE_OK:
            raise FEError(rc)
        return colptr, rowval

    def subdomains(self, cellvalues: Sequence[CellValues]) -> List[Subdomain]:
        out = []
        for s, cv in zip(self.subs, cellvalues):
            out.append(Subdomain(s["cell_type"], s["ip_order"], s["n_components"], cv.weights, cv.N, cv.dNdxi,
                                 cv.M, cv.dMdxi, s["cellset"], s["cell_nodes"]))
        return out

    def handle(self, cellvalues: Sequence[CellValues], colptr, rowval) -> Handle:
        """fe_create for this DofHandler, pattern and CellValues."""
        return Handle(self.nodes, self.subdomains(cellvalues), self.cell_dofs, self.cell_dofs_offset, self.ndofs,
                      colptr, rowval, self.n_cells)
