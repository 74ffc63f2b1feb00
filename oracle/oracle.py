"""Python front end of the CPU oracle (a restatement of Ferrite.jl's assembly path).

TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA engine and the timed CPU baseline.
Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline leg use it; the
product path (``ferrite.jl_gb300``) never imports it.

The heavy lifting is in ``ferrite_oracle.cpp`` (FP64, file:line citations of Ferrite.jl
v1.6.0 there). This module compiles it on first use (``g++``, no cmake), loads it with
ctypes and offers numpy-level helpers that produce the same arrays Ferrite holds:
node coordinates AoS, 1-based Int64 connectivity / cell_dofs / colptr / rowval.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "build")
LIB_PATH = os.path.join(BUILD_DIR, "libferrite_oracle.so")
SRC = os.path.join(HERE, "ferrite_oracle.cpp")

TRIANGLE, QUADRILATERAL, TETRAHEDRON, HEXAHEDRON, WEDGE = 1, 2, 3, 4, 5
HEAT, LINEAR_ELASTIC, NEO_HOOKE = 1, 2, 3
ERRORS = {0: "OK", 1: "ARG", 2: "BOUNDS", 3: "DETJ", 4: "PATTERN_MISSING", 5: "UNSUPPORTED"}

_lock = threading.Lock()
_lib = None

i32p = ctypes.POINTER(ctypes.c_int32)
i64p = ctypes.POINTER(ctypes.c_int64)
f64p = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> str:
    """Compile the oracle shared library (idempotent)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    hdr = os.path.join(HERE, "ferrite_oracle.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17",
           "-o", tmp, SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class _Problem(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("n_nodes", ctypes.c_int64), ("nodes", f64p),
                ("n_cells", ctypes.c_int64), ("cell_types", i32p), ("cell_nodes_offset", i64p),
                ("cell_nodes", i64p), ("n_sdh", ctypes.c_int32), ("sdh_ip_order", i32p),
                ("sdh_ncomp", i32p), ("sdh_qr_order", i32p), ("sdh_cellset_offset", i64p),
                ("sdh_cellset", i64p), ("ndofs", ctypes.c_int64), ("cell_dofs", i64p),
                ("cell_dofs_offset", i64p), ("colptr", i64p), ("rowval", i64p)]


class _Physics(ctypes.Structure):
    _fields_ = [("physics", ctypes.c_int32), ("p0", ctypes.c_double), ("p1", ctypes.c_double),
                ("body", ctypes.c_double * 3), ("cell_scale", f64p), ("u", f64p)]


class _Error(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int32), ("cell", ctypes.c_int64), ("detJ", ctypes.c_double),
                ("row", ctypes.c_int64), ("col", ctypes.c_int64)]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            L.or_grid_counts.argtypes = [ctypes.c_int32, i64p, i64p, i64p, i32p, i32p]
            L.or_generate_grid.argtypes = [ctypes.c_int32, i64p, f64p, f64p, f64p, i64p]
            L.or_nbase.argtypes = [ctypes.c_int32, ctypes.c_int32]
            L.or_close_dofhandler.argtypes = [ctypes.POINTER(_Problem), i64p, i64p, i64p]
            L.or_sparsity_pattern.argtypes = [ctypes.POINTER(_Problem), i64p, i64p, i64p]
            L.or_quadrature.argtypes = [ctypes.c_int32, ctypes.c_int32, i32p, f64p, f64p]
            L.or_shape_tables.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, f64p, f64p, f64p]
            L.or_assemble.argtypes = [ctypes.POINTER(_Problem), ctypes.POINTER(_Physics), ctypes.c_int32,
                                      ctypes.c_int32, f64p, f64p, ctypes.POINTER(_Error)]
            L.or_element_matrix.argtypes = [ctypes.POINTER(_Problem), ctypes.POINTER(_Physics),
                                            ctypes.c_int64, f64p, f64p, ctypes.POINTER(_Error)]
            L.or_index_map.argtypes = [ctypes.POINTER(_Problem), ctypes.c_int64, i64p]
            L.or_greedy_coloring.argtypes = [ctypes.POINTER(_Problem), i32p, i32p]
            L.or_facet_load.argtypes = [ctypes.POINTER(_Problem), ctypes.c_int64, i64p, i32p, ctypes.c_int32, ctypes.c_int32,
                                        f64p, f64p, f64p, ctypes.c_double, f64p, f64p, ctypes.POINTER(_Error)]
            L.or_apply.argtypes = [ctypes.c_int64, i64p, i64p, f64p, f64p, ctypes.c_int64, i64p, f64p, ctypes.c_int32]
            L.or_adjoint.argtypes = [ctypes.POINTER(_Problem), ctypes.POINTER(_Physics), f64p, f64p, f64p, f64p, f64p,
                                     ctypes.POINTER(_Error)]
            L.or_assemble_csr.argtypes = [ctypes.POINTER(_Problem), ctypes.POINTER(_Physics), ctypes.c_int32, i64p, i64p,
                                          f64p, f64p, ctypes.POINTER(_Error)]
            L.or_element_matvec.argtypes = [ctypes.POINTER(_Problem), ctypes.c_int32, ctypes.c_void_p, i64p, f64p,
                                            ctypes.c_int32, f64p]
            L.or_threaded_create.argtypes = [ctypes.POINTER(_Problem), ctypes.c_int32, ctypes.c_int32,
                                             ctypes.POINTER(ctypes.c_void_p), i32p]
            L.or_threaded_colors.argtypes = [ctypes.c_void_p, i32p]
            L.or_threaded_assemble.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Physics), f64p, f64p,
                                               ctypes.POINTER(_Error)]
            L.or_threaded_destroy.argtypes = [ctypes.c_void_p]
            L.or_threaded_destroy.restype = None
            _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else ctypes.cast(None, t)


def ref_dim(cell_type: int) -> int:
    return 2 if cell_type in (TRIANGLE, QUADRILATERAL) else 3


def nbase(cell_type: int, order: int) -> int:
    return lib().or_nbase(cell_type, order)


# ---------------------------------------------------------------------------------------
# grids, quadrature, shape tables
# ---------------------------------------------------------------------------------------
def generate_grid(cell_type: int, nel, left=None, right=None):
    """``generate_grid(CellType, nel, left, right)`` (grid_generators.jl). Returns
    (nodes [n_nodes, dim] float64, cells [n_cells, nodes_per_cell] int64 1-based)."""
    nel = np.ascontiguousarray(nel, dtype=np.int64)
    d = len(nel)
    left = np.ascontiguousarray(left if left is not None else -np.ones(d), dtype=np.float64)
    right = np.ascontiguousarray(right if right is not None else np.ones(d), dtype=np.float64)
    nn, nc = ctypes.c_int64(), ctypes.c_int64()
    npc, dim = ctypes.c_int32(), ctypes.c_int32()
    rc = lib().or_grid_counts(cell_type, _p(nel, i64p), ctypes.byref(nn), ctypes.byref(nc),
                              ctypes.byref(npc), ctypes.byref(dim))
    if rc:
        raise ValueError(f"unsupported cell type {cell_type}")
    nodes = np.empty((nn.value, dim.value), np.float64)
    cells = np.empty((nc.value, npc.value), np.int64)
    lib().or_generate_grid(cell_type, _p(nel, i64p), _p(left, f64p), _p(right, f64p),
                           _p(nodes, f64p), _p(cells, i64p))
    return nodes, cells


def quadrature(cell_type: int, order: int):
    """``QuadratureRule{RefShape}(order)``: (weights [nq], points [nq, rdim])."""
    nq = ctypes.c_int32()
    w = np.empty(512)
    pts = np.empty(512 * 3)
    rc = lib().or_quadrature(cell_type, order, ctypes.byref(nq), _p(w, f64p), _p(pts, f64p))
    if rc:
        raise ValueError("unsupported quadrature")
    n = nq.value
    return w[:n].copy(), pts[: n * ref_dim(cell_type)].reshape(n, ref_dim(cell_type)).copy()


def shape_tables(cell_type: int, order: int, points):
    """Reference shape values N[nq, nb] and gradients dN[nq, nb, rdim] (the tables
    ``FunctionValues`` / ``GeometryMapping`` precompute)."""
    points = np.ascontiguousarray(points, dtype=np.float64)
    nq = points.shape[0]
    nb = nbase(cell_type, order)
    rd = ref_dim(cell_type)
    N = np.empty((nq, nb))
    dN = np.empty((nq, nb, rd))
    rc = lib().or_shape_tables(cell_type, order, nq, _p(points, f64p), _p(N, f64p), _p(dN, f64p))
    if rc:
        raise ValueError("unsupported interpolation")
    return N, dN


def perturb_interior(nodes, nel, amplitude: float, seed: int, left=None, right=None):
    """Move every interior node of a structured box grid by i.i.d. uniform noise in
    [-amplitude*h_d, +amplitude*h_d] per coordinate (h_d = cell size along axis d).
    Seeded stand-in for the unseeded perturbation of test/test_utils.jl:282-293."""
    nodes = np.array(nodes, dtype=np.float64, copy=True)
    d = nodes.shape[1]
    lo = nodes.min(axis=0) if left is None else np.asarray(left, float)
    hi = nodes.max(axis=0) if right is None else np.asarray(right, float)
    h = (hi - lo) / np.asarray(nel, float)
    tol = 1e-9 * (hi - lo)
    interior = np.all((nodes > lo + tol) & (nodes < hi - tol), axis=1)
    rng = np.random.default_rng(seed)
    noise = rng.uniform(-1.0, 1.0, size=(int(interior.sum()), d)) * (amplitude * h)
    nodes[interior] += noise
    return nodes


# ---------------------------------------------------------------------------------------
# Problem: grid + SubDofHandlers + dofs + pattern
# ---------------------------------------------------------------------------------------
class Subdomain:
    """One SubDofHandler: a cellset with a single cell type and field interpolation."""

    def __init__(self, cellset, ip_order: int, ncomp: int, qr_order: int):
        self.cellset = np.ascontiguousarray(cellset, dtype=np.int64)  # 1-based
        self.ip_order = int(ip_order)
        self.ncomp = int(ncomp)
        self.qr_order = int(qr_order)


class Problem:
    """Grid + DofHandler + sparsity pattern, as arrays in Ferrite's layout."""

    def __init__(self, nodes, cell_types, cell_nodes_offset, cell_nodes, subdomains):
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self.dim = self.nodes.shape[1]
        self.cell_types = np.ascontiguousarray(cell_types, dtype=np.int32)
        self.cell_nodes_offset = np.ascontiguousarray(cell_nodes_offset, dtype=np.int64)
        self.cell_nodes = np.ascontiguousarray(cell_nodes, dtype=np.int64)
        self.subdomains = list(subdomains)
        self.n_cells = len(self.cell_types)
        self.cell_dofs = None
        self.cell_dofs_offset = None
        self.ndofs = 0
        self.colptr = None
        self.rowval = None
        self._keep = []

    @classmethod
    def single(cls, cell_type, nodes, cells, ip_order=1, ncomp=1, qr_order=2):
        cells = np.ascontiguousarray(cells, dtype=np.int64)
        n, npc = cells.shape
        prob = cls(nodes, np.full(n, cell_type, np.int32), np.arange(n + 1, dtype=np.int64) * npc,
                   cells.reshape(-1), [Subdomain(np.arange(1, n + 1), ip_order, ncomp, qr_order)])
        return prob

    def cells_of(self, c0: int):
        """1-based node ids of cell c0 (0-based index)."""
        return self.cell_nodes[self.cell_nodes_offset[c0]:self.cell_nodes_offset[c0 + 1]]

    def _struct(self):
        sd = self.subdomains
        ip = np.array([s.ip_order for s in sd], np.int32)
        nc = np.array([s.ncomp for s in sd], np.int32)
        qo = np.array([s.qr_order for s in sd], np.int32)
        off = np.zeros(len(sd) + 1, np.int64)
        off[1:] = np.cumsum([len(s.cellset) for s in sd])
        cs = np.concatenate([s.cellset for s in sd]).astype(np.int64)
        self._keep = [ip, nc, qo, off, cs]
        P = _Problem()
        P.dim = self.dim
        P.n_nodes = self.nodes.shape[0]
        P.nodes = _p(self.nodes, f64p)
        P.n_cells = self.n_cells
        P.cell_types = _p(self.cell_types, i32p)
        P.cell_nodes_offset = _p(self.cell_nodes_offset, i64p)
        P.cell_nodes = _p(self.cell_nodes, i64p)
        P.n_sdh = len(sd)
        P.sdh_ip_order = _p(ip, i32p)
        P.sdh_ncomp = _p(nc, i32p)
        P.sdh_qr_order = _p(qo, i32p)
        P.sdh_cellset_offset = _p(off, i64p)
        P.sdh_cellset = _p(cs, i64p)
        P.ndofs = self.ndofs
        P.cell_dofs = _p(self.cell_dofs, i64p)
        P.cell_dofs_offset = _p(self.cell_dofs_offset, i64p)
        P.colptr = _p(self.colptr, i64p)
        P.rowval = _p(self.rowval, i64p)
        return P

    def ndofs_per_cell(self, sdh: int) -> int:
        s = self.subdomains[sdh]
        ct = int(self.cell_types[s.cellset[0] - 1])
        return nbase(ct, s.ip_order) * s.ncomp

    def close(self):
        """``close!(dh)``: distribute dofs (DofHandler.jl:493-794)."""
        total = sum(self.ndofs_per_cell(k) * len(s.cellset) for k, s in enumerate(self.subdomains))
        self.cell_dofs = np.zeros(total, np.int64)
        self.cell_dofs_offset = np.zeros(self.n_cells, np.int64)
        nd = ctypes.c_int64()
        P = self._struct()
        rc = lib().or_close_dofhandler(ctypes.byref(P), _p(self.cell_dofs, i64p),
                                       _p(self.cell_dofs_offset, i64p), ctypes.byref(nd))
        if rc:
            raise RuntimeError(f"close_dofhandler failed: {ERRORS.get(rc, rc)}")
        self.ndofs = nd.value
        return self

    def allocate_matrix(self):
        """``allocate_matrix(dh)``: colptr/rowval (1-based Int64)."""
        self.colptr = np.zeros(self.ndofs + 1, np.int64)
        nnz = ctypes.c_int64()
        P = self._struct()
        lib().or_sparsity_pattern(ctypes.byref(P), _p(self.colptr, i64p), None, ctypes.byref(nnz))
        self.rowval = np.empty(nnz.value, np.int64)
        P = self._struct()
        rc = lib().or_sparsity_pattern(ctypes.byref(P), _p(self.colptr, i64p), _p(self.rowval, i64p),
                                       ctypes.byref(nnz))
        if rc:
            raise RuntimeError(f"sparsity pattern failed: {ERRORS.get(rc, rc)}")
        return self

    @property
    def nnz(self) -> int:
        return int(self.colptr[-1] - 1)

    def celldofs(self, c0: int):
        s = self._sdh_of(c0)
        o = self.cell_dofs_offset[c0] - 1
        return self.cell_dofs[o:o + self.ndofs_per_cell(s)]

    def _sdh_of(self, c0: int) -> int:
        for k, s in enumerate(self.subdomains):
            if np.any(s.cellset == c0 + 1):
                return k
        raise KeyError(c0)

    # -----------------------------------------------------------------------------------
    def _physics(self, physics, p0, p1, body, cell_scale, u):
        ph = _Physics()
        ph.physics = physics
        ph.p0 = p0
        ph.p1 = p1
        for k in range(3):
            ph.body[k] = body[k] if body is not None and k < len(body) else 0.0
        self._phys_keep = []
        if cell_scale is not None:
            cs = np.ascontiguousarray(cell_scale, np.float64)
            self._phys_keep.append(cs)
            ph.cell_scale = _p(cs, f64p)
        else:
            ph.cell_scale = ctypes.cast(None, f64p)
        if u is not None:
            uu = np.ascontiguousarray(u, np.float64)
            self._phys_keep.append(uu)
            ph.u = _p(uu, f64p)
        else:
            ph.u = ctypes.cast(None, f64p)
        return ph

    def assemble(self, physics, p0, p1, body=None, cell_scale=None, u=None, nthreads=0,
                 nzval=None, f=None, fillzero=True):
        """start_assemble + cell loop + assemble!; returns (nzval, f). Raises on errors with
        the same information Ferrite's exceptions carry."""
        if nzval is None:
            nzval = np.zeros(self.nnz)
        if f is None:
            f = np.zeros(self.ndofs)
        P = self._struct()
        ph = self._physics(physics, p0, p1, body, cell_scale, u)
        err = _Error()
        rc = lib().or_assemble(ctypes.byref(P), ctypes.byref(ph), int(nthreads), int(fillzero),
                               _p(nzval, f64p), _p(f, f64p), ctypes.byref(err))
        if rc:
            raise OracleError(rc, err)
        return nzval, f

    def csr_pattern(self):
        """allocate_matrix(SparseMatrixCSR, dh) (ext/FerriteSparseMatrixCSR.jl:124-160): the
        pattern's rows, columns ascending -- the transpose of the CSC pattern; returns 1-based
        (rowptr, colval)."""
        import scipy.sparse as sp
        A = sp.csc_matrix((np.ones(self.nnz), self.rowval - 1, self.colptr - 1), shape=(self.ndofs, self.ndofs)).tocsr()
        A.sort_indices()
        return A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1

    def assemble_csr(self, rowptr, colval, physics, p0, p1, body=None, cell_scale=None, u=None, fillzero=True):
        """start_assemble(K::SparseMatrixCSR, f) + cell loop + assemble! (serial, cell order);
        returns (nzval, f) of the CSR matrix."""
        rowptr = np.ascontiguousarray(rowptr, np.int64)
        colval = np.ascontiguousarray(colval, np.int64)
        nzval = np.zeros(len(colval))
        f = np.zeros(self.ndofs)
        P = self._struct()
        ph = self._physics(physics, p0, p1, body, cell_scale, u)
        err = _Error()
        rc = lib().or_assemble_csr(ctypes.byref(P), ctypes.byref(ph), int(fillzero), _p(rowptr, i64p), _p(colval, i64p),
                                   _p(nzval, f64p), _p(f, f64p), ctypes.byref(err))
        if rc:
            raise OracleError(rc, err)
        return nzval, f

    def element(self, c0: int, physics, p0, p1, body=None, cell_scale=None, u=None):
        s = self._sdh_of(c0)
        ld = self.ndofs_per_cell(s)
        Ke = np.zeros((ld, ld), order="F")
        fe = np.zeros(ld)
        P = self._struct()
        ph = self._physics(physics, p0, p1, body, cell_scale, u)
        err = _Error()
        rc = lib().or_element_matrix(ctypes.byref(P), ctypes.byref(ph), c0, _p(Ke, f64p), _p(fe, f64p),
                                     ctypes.byref(err))
        if rc:
            raise OracleError(rc, err)
        return Ke, fe

    def adjoint(self, physics, p0, p1, u, lam, body=None, cell_scale=None, dscale=None):
        """Vector-Jacobian products of Phi = lam^T (K u - f): (d_cell[n_cells], d_X[n_nodes, dim]),
        d_cell = dscale * dPhi/d(cell_scale) (dscale None: 1)."""
        P = self._struct()
        ph = self._physics(physics, p0, p1, body, cell_scale, None)
        uu = np.ascontiguousarray(u, np.float64)
        ll = np.ascontiguousarray(lam, np.float64)
        ds = None if dscale is None else np.ascontiguousarray(dscale, np.float64)
        d_cell = np.zeros(self.n_cells)
        d_X = np.zeros((self.nodes.shape[0], self.dim))
        err = _Error()
        rc = lib().or_adjoint(ctypes.byref(P), ctypes.byref(ph), _p(uu, f64p), _p(ll, f64p),
                              _p(ds, f64p) if ds is not None else ctypes.cast(None, f64p), _p(d_cell, f64p),
                              _p(d_X, f64p), ctypes.byref(err))
        if rc:
            raise OracleError(rc, err)
        return d_cell, d_X

    def facet_load(self, cells, facets, tables, pressure, traction=(0.0, 0.0, 0.0), f=None):
        """Facet loads over (cell, local facet) pairs (1-based), f += (in place; zeros if None).
        tables = (n_ref_facets, n_qp, w, N, dM) per reference facet."""
        nf, nq, w, N, dM = tables
        c = np.ascontiguousarray(cells, np.int64)
        fc = np.ascontiguousarray(facets, np.int32)
        if f is None:
            f = np.zeros(self.ndofs)
        t = np.ascontiguousarray(list(traction) + [0.0] * (3 - len(traction)), np.float64)
        P = self._struct()
        err = _Error()
        rc = lib().or_facet_load(ctypes.byref(P), len(c), _p(c, i64p), _p(fc, i32p), nf, nq,
                                 _p(np.ascontiguousarray(w, np.float64), f64p), _p(np.ascontiguousarray(N, np.float64), f64p),
                                 _p(np.ascontiguousarray(dM, np.float64), f64p), float(pressure), _p(t, f64p),
                                 _p(f, f64p), ctypes.byref(err))
        if rc:
            raise OracleError(rc, err)
        return f

    def apply(self, nzval, f, prescribed, inhomogeneities=None, applyzero=False):
        """apply!(K, f, ch) / apply_zero!(K, f, ch) for Dirichlet constraints, in place
        (ConstraintHandler.jl:711-744). prescribed: 1-based, ascending; f may be None."""
        pd = np.ascontiguousarray(prescribed, np.int64)
        g = np.ascontiguousarray(inhomogeneities if inhomogeneities is not None else np.zeros(len(pd)), np.float64)
        rc = lib().or_apply(self.ndofs, _p(self.colptr, i64p), _p(self.rowval, i64p), _p(nzval, f64p),
                            _p(f, f64p) if f is not None else None, len(pd), _p(pd, i64p), _p(g, f64p),
                            1 if applyzero else 0)
        if rc:
            raise OracleError(rc, _Error())
        return nzval, f

    def element_matvec(self, ke, u, y=None, fillzero=True):
        """y (+)= sum over cells in ascending order of A_c^T Ke_c A_c u, Ke_c = ke[c] (an array
        [n_cells, n, n], float32 or float64, any strides), with the operation order of
        or_element_matvec (fused multiply-adds in the element precision, FP64 sums)."""
        ke = np.asarray(ke)
        if ke.dtype not in (np.float32, np.float64) or ke.ndim != 3:
            raise ValueError("ke must be a float32 or float64 array [n_cells, n, n]")
        ks = np.array([st // ke.itemsize for st in ke.strides], np.int64)
        u = np.ascontiguousarray(u, np.float64)
        if y is None:
            y = np.zeros(self.ndofs, np.float64)
            fillzero = True
        P = self._struct()
        rc = lib().or_element_matvec(ctypes.byref(P), 1 if ke.dtype == np.float64 else 0,
                                     ctypes.c_void_p(ke.ctypes.data), _p(ks, i64p), _p(u, f64p),
                                     1 if fillzero else 0, _p(y, f64p))
        if rc:
            raise OracleError(rc, _Error())
        return y

    def index_map(self, c0: int):
        """1-based nzval positions of Ke entries of cell c0 ([ld, ld], Ke[I, J])."""
        s = self._sdh_of(c0)
        ld = self.ndofs_per_cell(s)
        pos = np.zeros((ld, ld), np.int64, order="F")
        P = self._struct()
        lib().or_index_map(ctypes.byref(P), c0, _p(pos, i64p))
        return pos

    def coloring(self):
        col = np.zeros(self.n_cells, np.int32)
        n = ctypes.c_int32()
        P = self._struct()
        lib().or_greedy_coloring(ctypes.byref(P), _p(col, i32p), ctypes.byref(n))
        return col, n.value

    def to_scipy(self, nzval):
        import scipy.sparse as sp
        return sp.csc_matrix((nzval, self.rowval - 1, self.colptr - 1), shape=(self.ndofs, self.ndofs))

    def threaded(self, nthreads, algorithm="workstream"):
        """The threaded colored assembly of threaded_assembly.jl, prepared once (CellValues and
        coloring at set-up); ``.assemble(...)`` is one assemble_global! call."""
        return Threaded(self, nthreads, algorithm)


class Threaded:
    """or_threaded_*: set-up (coloring) outside, the colored loop inside each call."""

    ALGORITHMS = {"greedy": 1, "workstream": 2}

    def __init__(self, prob, nthreads, algorithm="workstream"):
        self.prob, self.nthreads, self.algorithm = prob, int(nthreads), algorithm
        self._P = prob._struct()
        self._keep = list(prob._keep)  # the view's arrays live as long as the context
        ptr, n = ctypes.c_void_p(), ctypes.c_int32()
        t = time.perf_counter()
        rc = lib().or_threaded_create(ctypes.byref(self._P), self.nthreads, self.ALGORITHMS[algorithm],
                                      ctypes.byref(ptr), ctypes.byref(n))
        self.setup_s = time.perf_counter() - t
        if rc:
            raise OracleError(rc, _Error())
        self._h, self.n_colors = ptr, n.value

    def colors(self):
        col = np.zeros(self.prob.n_cells, np.int32)
        lib().or_threaded_colors(self._h, _p(col, i32p))
        return col

    def assemble(self, physics, p0, p1, body=None, cell_scale=None, u=None, nzval=None, f=None):
        prob = self.prob
        if nzval is None:
            nzval = np.zeros(prob.nnz)
        if f is None:
            f = np.zeros(prob.ndofs)
        ph = prob._physics(physics, p0, p1, body, cell_scale, u)
        err = _Error()
        rc = lib().or_threaded_assemble(self._h, ctypes.byref(ph), _p(nzval, f64p), _p(f, f64p), ctypes.byref(err))
        if rc:
            raise OracleError(rc, err)
        return nzval, f

    def close(self):
        if self._h:
            lib().or_threaded_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OracleError(RuntimeError):
    def __init__(self, code, err):
        self.code = code
        self.name = ERRORS.get(code, str(code))
        self.cell = err.cell
        self.detJ = err.detJ
        self.row = err.row
        self.col = err.col
        super().__init__(f"{self.name}: cell={self.cell} detJ={self.detJ} row={self.row} col={self.col}")


def box_problem(cell_type, nel, left=None, right=None, ip_order=1, ncomp=1, qr_order=2,
                perturb=0.0, seed=0, pattern=True):
    """generate_grid + DofHandler(add! one field) + close! + allocate_matrix."""
    nodes, cells = generate_grid(cell_type, nel, left, right)
    if perturb:
        nodes = perturb_interior(nodes, nel, perturb, seed, left, right)
    prob = Problem.single(cell_type, nodes, cells, ip_order, ncomp, qr_order).close()
    if pattern:
        prob.allocate_matrix()
    return prob


def lame(E: float, nu: float):
    return E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
