"""ferrite_gb300 -- Python host binding of libferrite_gb300.so, the GB300 (sm_103a)
finite-element assembly engine that replaces Ferrite.jl's assembly hot path.

The C ABI (include/ferrite_gb300.h) is the product; this module mirrors the Ferrite-level
interface on top of it so a Python caller (and the parity tests) reads like Ferrite code:

    handle = Handle(grid_nodes, [Subdomain(...)], dh_cell_dofs, dh_cell_dofs_offset, ndofs,
                    K_colptr, K_rowval, n_cells)            # allocate_matrix + CellValues data
    asm = start_assemble(handle, K_nzval, f)                 # src/assembler.jl:287-291
    assemble(asm, LinearElasticity(E, nu, body))             # the whole cell loop, one call
    K_nzval, f = finish_assemble(asm)                        # src/assembler.jl:299-301

nzval / f / u / cell_scale may be numpy arrays (host; staged through device buffers) or
torch CUDA tensors (device, written in place). Errors raise ``FEError`` carrying the same
information as Ferrite's exceptions (cell id and detJ, or the missing (row, col)).

There is no CPU fallback: if the shared library is missing or no GPU is present, calls fail.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libferrite_gb300.so")

# constants of include/ferrite_gb300.h
FE_OK, FE_ERR_ARG, FE_ERR_BOUNDS, FE_ERR_DETJ, FE_ERR_PATTERN_MISSING = 0, 1, 2, 3, 4
FE_ERR_UNSUPPORTED, FE_ERR_CUDA, FE_ERR_OOM, FE_ERR_STATE = 5, 6, 7, 8
ERROR_NAMES = {0: "OK", 1: "ARG", 2: "BOUNDS", 3: "DETJ", 4: "PATTERN_MISSING", 5: "UNSUPPORTED",
               6: "CUDA", 7: "OOM", 8: "STATE"}
TRIANGLE, QUADRILATERAL, TETRAHEDRON, HEXAHEDRON, WEDGE = 1, 2, 3, 4, 5
HEAT, LINEAR_ELASTIC, NEO_HOOKE = 1, 2, 3
PREC_MIXED, PREC_FP64 = 0, 1
FILLZERO, NO_K, NO_F, ASYNC, PROFILE, COMPENSATED, TWO_PHASE, FUSED, NO_TENSOR = 1, 2, 4, 8, 16, 32, 64, 128, 256
STAGED_OUTPUT = 512
FP32_SUM = 1024
_FORMS = {None: 0, "two_phase": TWO_PHASE, "fused": FUSED, "two_phase_cuda_cores": TWO_PHASE | NO_TENSOR}

EXPORTED = ["fe_abi_version", "fe_create", "fe_assemble", "fe_sync", "fe_last_error", "fe_get_info",
            "fe_get_index_map", "fe_plan_dry_run", "fe_distribute_dofs", "fe_sparsity_pattern", "fe_kernel_time", "fe_assemble_noalloc",
            "fe_assemble_adjoint", "fe_graph_capture", "fe_graph_replay", "fe_graph_destroy",
            "fe_autotune", "fe_assemble_elements", "fe_sparsity_pattern_device", "fe_facet_set_create", "fe_assemble_facet_load",
            "fe_facet_set_destroy", "fe_dirichlet_create", "fe_apply", "fe_dirichlet_destroy",
            "fe_element_operator_create", "fe_element_matvec", "fe_element_operator_destroy", "fe_destroy"]

i64p = ctypes.POINTER(ctypes.c_int64)
f64p = ctypes.POINTER(ctypes.c_double)
i32p = ctypes.POINTER(ctypes.c_int32)


class GridDesc(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("n_nodes", ctypes.c_int64), ("nodes", f64p), ("n_cells", ctypes.c_int64)]


class SubdomainDesc(ctypes.Structure):
    _fields_ = [("cell_type", ctypes.c_int32), ("ip_order", ctypes.c_int32), ("n_components", ctypes.c_int32),
                ("n_qp", ctypes.c_int32), ("qr_weights", f64p), ("N", f64p), ("dNdxi", f64p), ("M", f64p),
                ("dMdxi", f64p), ("n_cells", ctypes.c_int64), ("cellset", i64p), ("cell_nodes", i64p)]


class DofDesc(ctypes.Structure):
    _fields_ = [("ndofs", ctypes.c_int64), ("cell_dofs", i64p), ("cell_dofs_offset", i64p)]


class CscDesc(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("nnz", ctypes.c_int64), ("colptr", i64p), ("rowval", i64p)]


class AssembleParams(ctypes.Structure):
    _fields_ = [("physics", ctypes.c_int32), ("precision", ctypes.c_int32), ("flags", ctypes.c_uint32),
                ("p0", ctypes.c_double), ("p1", ctypes.c_double), ("body", ctypes.c_double * 3),
                ("cell_scale", ctypes.c_void_p), ("u", ctypes.c_void_p), ("cond_threshold", ctypes.c_double),
                ("stream", ctypes.c_void_p)]


class FacetDesc(ctypes.Structure):
    """fe_facet_desc: FacetValues tables per reference facet and the set's (cell, facet) pairs."""
    _fields_ = [("n_qp", ctypes.c_int32), ("n_ref_facets", ctypes.c_int32), ("qr_weights", f64p), ("N", f64p),
                ("dMdxi", f64p), ("n_facets", ctypes.c_int64), ("cells", i64p), ("facets", i32p)]


class ElementLayout(ctypes.Structure):
    """fe_element_layout: element strides of Ke(cell, I, J) and fe(cell, I)."""
    _fields_ = [("ke_stride", ctypes.c_int64 * 3), ("fe_stride", ctypes.c_int64 * 2)]


class AdjointParams(ctypes.Structure):
    _fields_ = [("physics", ctypes.c_int32), ("precision", ctypes.c_int32), ("flags", ctypes.c_uint32),
                ("p0", ctypes.c_double), ("p1", ctypes.c_double), ("body", ctypes.c_double * 3),
                ("cell_scale", ctypes.c_void_p), ("dscale", ctypes.c_void_p), ("stream", ctypes.c_void_p)]


TUNE_MAX = 16


class TuneResult(ctypes.Structure):
    _fields_ = [("n_candidates", ctypes.c_int32), ("stage_cap", ctypes.c_int32 * TUNE_MAX),
                ("ms", ctypes.c_double * TUNE_MAX), ("n_tiles", ctypes.c_int64 * TUNE_MAX),
                ("n_cell_visits", ctypes.c_int64 * TUNE_MAX), ("best_stage_cap", ctypes.c_int32),
                ("best_ms", ctypes.c_double), ("form_mask", ctypes.c_uint32 * TUNE_MAX),
                ("best_form_mask", ctypes.c_uint32)]


class ErrorInfo(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int32), ("cell", ctypes.c_int64), ("detJ", ctypes.c_double),
                ("row", ctypes.c_int64), ("col", ctypes.c_int64), ("message", ctypes.c_char * 256)]


class Info(ctypes.Structure):
    _fields_ = [("n_cells", ctypes.c_int64), ("ndofs", ctypes.c_int64), ("nnz", ctypes.c_int64),
                ("n_tiles", ctypes.c_int64), ("n_cell_visits", ctypes.c_int64), ("n_items", ctypes.c_int64),
                ("flagged_cells", ctypes.c_int64), ("device_bytes", ctypes.c_int64),
                ("create_seconds", ctypes.c_double), ("max_record_bytes", ctypes.c_int32),
                ("max_tile_nodes", ctypes.c_int32), ("max_stage_values", ctypes.c_int32),
                ("max_out_doubles", ctypes.c_int32), ("stage_cap", ctypes.c_int32), ("plan_checksum", ctypes.c_uint32)]


_lib = None


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile the CUDA library for sm_103a (ferrite.jl_gb300/build.py)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_fe_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(verbose=verbose, force=force)


def lib():
    """Load libferrite_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run ferrite_gb300.build() (nvcc, sm_103a) first")
        L = ctypes.CDLL(LIB_PATH)
        L.fe_abi_version.restype = ctypes.c_int
        L.fe_create.argtypes = [ctypes.POINTER(GridDesc), ctypes.c_int32, ctypes.POINTER(SubdomainDesc),
                                ctypes.POINTER(DofDesc), ctypes.POINTER(CscDesc), ctypes.POINTER(ctypes.c_void_p)]
        L.fe_assemble.argtypes = [ctypes.c_void_p, ctypes.POINTER(AssembleParams), ctypes.c_void_p, ctypes.c_void_p]
        L.fe_sync.argtypes = [ctypes.c_void_p]
        L.fe_last_error.argtypes = [ctypes.c_void_p, ctypes.POINTER(ErrorInfo)]
        L.fe_get_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(Info)]
        L.fe_get_index_map.argtypes = [ctypes.c_void_p, ctypes.c_int64, i64p]
        L.fe_plan_dry_run.argtypes = [ctypes.POINTER(GridDesc), ctypes.c_int32, ctypes.POINTER(SubdomainDesc),
                                      ctypes.POINTER(DofDesc), ctypes.POINTER(CscDesc), ctypes.POINTER(Info)]
        L.fe_distribute_dofs.argtypes = [ctypes.POINTER(GridDesc), ctypes.c_int32, ctypes.POINTER(SubdomainDesc),
                                         i64p, i64p, i64p]
        L.fe_sparsity_pattern.argtypes = [ctypes.POINTER(GridDesc), ctypes.c_int32, ctypes.POINTER(SubdomainDesc),
                                          ctypes.POINTER(DofDesc), i64p, i64p, i64p]
        L.fe_sparsity_pattern_device.argtypes = [ctypes.POINTER(GridDesc), ctypes.c_int32, ctypes.POINTER(SubdomainDesc),
                                          ctypes.POINTER(DofDesc), i64p, i64p, i64p]
        L.fe_kernel_time.argtypes = [ctypes.c_void_p, f64p, i64p]
        L.fe_assemble_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(AssembleParams), ctypes.c_void_p, ctypes.c_void_p]
        L.fe_facet_set_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(FacetDesc), ctypes.POINTER(ctypes.c_void_p)]
        L.fe_assemble_facet_load.argtypes = [ctypes.c_void_p, ctypes.c_double, f64p, ctypes.c_uint32, ctypes.c_void_p,
                                             ctypes.c_void_p]
        L.fe_facet_set_destroy.argtypes = [ctypes.c_void_p]
        L.fe_facet_set_destroy.restype = None
        L.fe_dirichlet_create.argtypes = [ctypes.c_void_p, i64p, ctypes.c_int64, i64p, ctypes.POINTER(ctypes.c_void_p)]
        L.fe_apply.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                               ctypes.c_void_p]
        L.fe_dirichlet_destroy.argtypes = [ctypes.c_void_p]
        L.fe_dirichlet_destroy.restype = None
        L.fe_element_operator_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(ElementLayout), ctypes.c_int32,
                                                 ctypes.POINTER(ctypes.c_void_p)]
        L.fe_element_matvec.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                        ctypes.c_void_p]
        L.fe_element_operator_destroy.argtypes = [ctypes.c_void_p]
        L.fe_element_operator_destroy.restype = None
        L.fe_assemble_elements.argtypes = [ctypes.c_void_p, ctypes.POINTER(AssembleParams), ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.POINTER(ElementLayout)]
        L.fe_assemble_adjoint.argtypes = [ctypes.c_void_p, ctypes.POINTER(AdjointParams), ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]
        L.fe_graph_capture.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(AssembleParams),
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                       ctypes.POINTER(ctypes.c_int32)]
        L.fe_graph_replay.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_uint32]
        L.fe_graph_destroy.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        L.fe_autotune.argtypes = [ctypes.c_void_p, ctypes.POINTER(AssembleParams), ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, ctypes.POINTER(TuneResult)]
        L.fe_destroy.argtypes = [ctypes.c_void_p]
        L.fe_destroy.restype = None
        _lib = L
    return _lib


class FEError(RuntimeError):
    """An FE_* status from the library, with Ferrite's exception details."""

    def __init__(self, code: int, info: Optional[ErrorInfo] = None):
        self.code = code
        self.name = ERROR_NAMES.get(code, str(code))
        self.cell = info.cell if info else 0
        self.detJ = info.detJ if info else 0.0
        self.row = info.row if info else 0
        self.col = info.col if info else 0
        msg = info.message.decode(errors="replace") if info else ""
        super().__init__(f"FE_ERR_{self.name}: {msg}")


def _as_i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def _as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(x):
    """Raw address of a numpy array or a torch tensor (None -> NULL)."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous:
            raise ValueError("array must be contiguous")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return x.data_ptr()
    raise TypeError(f"unsupported buffer type {type(x)}")


def _dtype(x) -> str:
    return str(x.dtype).replace("torch.", "")


def _numel(x) -> int:
    return int(x.size) if isinstance(x, np.ndarray) else int(x.numel())


def _check(x, name: str, dtype: str, n: int):
    """A buffer the library reads or writes n elements of: its element type and length. The C
    ABI takes bare pointers, so a wrong type or a short buffer would be accessed past its end."""
    if x is None:
        return
    if not isinstance(x, np.ndarray) and not hasattr(x, "data_ptr"):
        raise TypeError(f"{name}: unsupported buffer type {type(x)}")
    if _dtype(x) != dtype:
        raise TypeError(f"{name} must be {dtype}, got {_dtype(x)}")
    if _numel(x) < n:
        raise ValueError(f"{name} has {_numel(x)} elements; the call accesses {n}")


def _extent(n_cells: int, m: int, strides) -> int:
    """Elements spanned by per-cell arrays X(c, I[, J]) at c*s0 + I*s1 (+ J*s2), m dofs per cell."""
    st = [int(v) for v in strides]
    if any(v < 0 for v in st):
        raise ValueError("element strides must be non-negative")
    if n_cells == 0 or m == 0:
        return 0
    return (n_cells - 1) * st[0] + sum((m - 1) * v for v in st[1:]) + 1


def _max_dofs_per_cell(subdomains) -> int:
    """Most dofs of one cell over the subdomains: base functions (N is [n_qp, n_base]) times
    components."""
    return max(((np.asarray(sd.N).size // max(len(np.asarray(sd.qr_weights)), 1)) * int(sd.n_components)
                for sd in subdomains), default=0)


def _elem_dtype(precision: int) -> str:
    return "float64" if precision == PREC_FP64 else "float32"


@dataclass
class Subdomain:
    """One SubDofHandler + its CellValues data (the arrays a Julia caller extracts from
    ``dh.subdofhandlers[k]``, ``cv.fun_values`` and ``cv.geo_mapping``)."""
    cell_type: int
    ip_order: int
    n_components: int
    qr_weights: np.ndarray
    N: np.ndarray        # [nq, nb]
    dNdxi: np.ndarray    # [nq, nb, rdim]
    M: np.ndarray        # [nq, ng]
    dMdxi: np.ndarray    # [nq, ng, rdim]
    cellset: np.ndarray  # [n] 1-based
    cell_nodes: np.ndarray  # [n, ng] 1-based
    _keep: list = field(default_factory=list, repr=False)

    def desc(self) -> SubdomainDesc:
        arrs = [_as_f64(self.qr_weights), _as_f64(self.N), _as_f64(self.dNdxi), _as_f64(self.M),
                _as_f64(self.dMdxi), _as_i64(self.cellset), _as_i64(self.cell_nodes)]
        self._keep = arrs
        d = SubdomainDesc()
        d.cell_type, d.ip_order, d.n_components = self.cell_type, self.ip_order, self.n_components
        d.n_qp = len(arrs[0])
        d.qr_weights, d.N, d.dNdxi, d.M, d.dMdxi = [a.ctypes.data_as(f64p) for a in arrs[:5]]
        d.n_cells = len(arrs[5])
        d.cellset = arrs[5].ctypes.data_as(i64p)
        d.cell_nodes = arrs[6].ctypes.data_as(i64p)
        return d


def _descs(nodes, subdomains, cell_dofs, cell_dofs_offset, ndofs, colptr, rowval, n_cells):
    nodes = _as_f64(nodes)
    g = GridDesc(nodes.shape[1], nodes.shape[0], nodes.ctypes.data_as(f64p), int(n_cells))
    subs = (SubdomainDesc * len(subdomains))(*[s.desc() for s in subdomains])
    cd, co = _as_i64(cell_dofs), _as_i64(cell_dofs_offset)
    dd = DofDesc(int(ndofs), cd.ctypes.data_as(i64p), co.ctypes.data_as(i64p))
    cp, rv = _as_i64(colptr), _as_i64(rowval)
    pd = CscDesc(int(ndofs), int(len(rv)), cp.ctypes.data_as(i64p), rv.ctypes.data_as(i64p))
    return (g, subs, dd, pd), (nodes, cd, co, cp, rv)


def plan_dry_run(nodes, subdomains, cell_dofs, cell_dofs_offset, ndofs, colptr, rowval, n_cells) -> dict:
    """fe_plan_dry_run: validate the arrays and build the index map and owner tiles on the
    host only (no GPU needed)."""
    (g, subs, dd, pd), _keep = _descs(nodes, subdomains, cell_dofs, cell_dofs_offset, ndofs, colptr, rowval, n_cells)
    info = Info()
    L = lib()
    rc = L.fe_plan_dry_run(ctypes.byref(g), len(subdomains), subs, ctypes.byref(dd), ctypes.byref(pd), ctypes.byref(info))
    if rc != FE_OK:
        e = ErrorInfo()
        L.fe_last_error(None, ctypes.byref(e))
        raise FEError(rc, e)
    return {k: getattr(info, k) for k, _ in Info._fields_}


class Handle:
    """fe_create/fe_destroy: the device-resident problem (grid, dofs, pattern, index map,
    owner tiles)."""

    def __init__(self, nodes, subdomains: Sequence[Subdomain], cell_dofs, cell_dofs_offset, ndofs: int,
                 colptr, rowval, n_cells: int):
        L = lib()
        nodes = _as_f64(nodes)
        g = GridDesc(nodes.shape[1], nodes.shape[0], nodes.ctypes.data_as(f64p), int(n_cells))
        subs = (SubdomainDesc * len(subdomains))(*[s.desc() for s in subdomains])
        cd, co = _as_i64(cell_dofs), _as_i64(cell_dofs_offset)
        dd = DofDesc(int(ndofs), cd.ctypes.data_as(i64p), co.ctypes.data_as(i64p))
        if getattr(colptr, "is_cuda", False) or getattr(rowval, "is_cuda", False):
            # a device pattern (allocate_matrix(device=True)): fe_create copies it to the host
            for x, name, n in ((colptr, "colptr", int(ndofs) + 1), (rowval, "rowval", 0)):
                if not getattr(x, "is_cuda", False):
                    raise TypeError("colptr and rowval must both be CUDA tensors or both host arrays")
                _check(x, name, "int64", n)
                if not x.is_contiguous():
                    raise ValueError(f"{name} must be contiguous")
            cp, rv = colptr, rowval
            nnz = int(rowval.numel())
            pd = CscDesc(int(ndofs), nnz, ctypes.cast(colptr.data_ptr(), i64p), ctypes.cast(rowval.data_ptr(), i64p))
        else:
            cp, rv = _as_i64(colptr), _as_i64(rowval)
            nnz = int(len(rv))
            pd = CscDesc(int(ndofs), nnz, cp.ctypes.data_as(i64p), rv.ctypes.data_as(i64p))
        h = ctypes.c_void_p()
        rc = L.fe_create(ctypes.byref(g), len(subdomains), subs, ctypes.byref(dd), ctypes.byref(pd), ctypes.byref(h))
        if rc != FE_OK:
            info = ErrorInfo()
            L.fe_last_error(None, ctypes.byref(info))
            raise FEError(rc, info)
        self._h = h
        self.ndofs = int(ndofs)
        self.nnz = nnz
        self.n_cells = int(n_cells)
        self.n_nodes, self.dim = int(nodes.shape[0]), int(nodes.shape[1])
        self.ndofs_per_cell = {}
        self._subdomains = list(subdomains)
        self.max_dofs_per_cell = _max_dofs_per_cell(subdomains)

    def _check_fields(self, u=None, cell_scale=None):
        _check(u, "u", "float64", self.ndofs)
        _check(cell_scale, "cell_scale", "float64", self.n_cells)

    def _check_outputs(self, nzval, f):
        _check(nzval, "nzval", "float64", self.nnz)
        _check(f, "f", "float64", self.ndofs)

    @property
    def ptr(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            lib().fe_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _raise(self, rc):
        info = ErrorInfo()
        lib().fe_last_error(self._h, ctypes.byref(info))
        raise FEError(rc, info)

    def assemble(self, nzval, f, physics: int, p0: float, p1: float, body=(0.0, 0.0, 0.0), cell_scale=None, u=None,
                 precision: int = PREC_MIXED, fillzero: bool = True, stream=None, sync: bool = True,
                 cond_threshold: float = 0.0, profile: bool = False, compensated: bool = True, form=None,
                 staged_output: bool = False):
        """One fe_assemble call. ``stream`` is a torch.cuda.Stream, a raw handle or None.
        ``compensated`` (mixed precision): sum each entry as a compensated FP32 pair (FP64-class, the
        default); False: one plain FP32 sum per entry (FE_FP32_SUM).
        ``staged_output``: host outputs through a device buffer and the copy engine, also when
        they are page-locked (default there: written by the kernels through the mapping).
        ``form``: None (the engine's choice), "two_phase" (element matrices first; on the tensor
        cores where a kernel exists), "two_phase_cuda_cores" or "fused"."""
        self._check_outputs(nzval, f)
        self._check_fields(u, cell_scale)
        p = AssembleParams()
        p.physics, p.precision = physics, precision
        flags = FILLZERO if fillzero else 0
        if nzval is None:
            flags |= NO_K
        if f is None:
            flags |= NO_F
        if not sync:
            flags |= ASYNC
        if profile:
            flags |= PROFILE
        if not compensated:
            flags |= FP32_SUM
        if staged_output:
            flags |= STAGED_OUTPUT
        flags |= _FORMS[form]
        p.flags = flags
        p.p0, p.p1 = float(p0), float(p1)
        for k in range(3):
            p.body[k] = float(body[k]) if k < len(body) else 0.0
        p.cell_scale = _ptr(cell_scale)
        p.u = _ptr(u)
        p.cond_threshold = float(cond_threshold)
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        p.stream = stream
        rc = lib().fe_assemble(self._h, ctypes.byref(p), _ptr(nzval), _ptr(f))
        if rc != FE_OK:
            self._raise(rc)
        return nzval, f

    def assemble_elements(self, ke, fe, physics: int, p0: float, p1: float, ke_stride=None, fe_stride=None,
                          stream=None, sync: bool = True, **kw):
        """fe_assemble_elements: every cell's Ke and fe into device arrays (torch CUDA tensors,
        float32 for mixed precision, float64 for FP64). Default layout: ke[n_cells, nbf, nbf] and
        fe[n_cells, nbf] row-major, i.e. ke[c, I, J] (the strides of ke.stride() / fe.stride())."""
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        p = self._params(physics, p0, p1, stream=stream, **kw)
        if ke is None:
            p.flags |= NO_K
        if fe is None:
            p.flags |= NO_F
        if not sync:
            p.flags |= ASYNC
        lay = ElementLayout()
        ks = ke_stride if ke_stride is not None else (tuple(ke.stride()) if ke is not None else (0, 0, 0))
        fs = fe_stride if fe_stride is not None else (tuple(fe.stride()) if fe is not None else (0, 0))
        for k in range(3):
            lay.ke_stride[k] = int(ks[k])
        for k in range(2):
            lay.fe_stride[k] = int(fs[k])
        dt = _elem_dtype(kw.get("precision", PREC_MIXED))
        m = self.max_dofs_per_cell
        if ke is not None:
            _check(ke, "ke", dt, _extent(self.n_cells, m, ks))
        if fe is not None:
            _check(fe, "fe", dt, _extent(self.n_cells, m, fs))
        self._check_fields(kw.get("u"), kw.get("cell_scale"))
        rc = lib().fe_assemble_elements(self._h, ctypes.byref(p), _ptr(ke), _ptr(fe), ctypes.byref(lay))
        if rc != FE_OK:
            self._raise(rc)
        return ke, fe

    def facet_set(self, cells, facets, tables):
        """fe_facet_set_create: (cell, local facet) pairs (1-based) of one subdomain and the
        FacetValues tables (n_ref_facets, n_qp, w, N, dM) per reference facet."""
        nf, nq, w, N, dM = tables
        keep = [np.ascontiguousarray(cells, np.int64), np.ascontiguousarray(facets, np.int32),
                np.ascontiguousarray(w, np.float64), np.ascontiguousarray(N, np.float64), np.ascontiguousarray(dM, np.float64)]
        d = FacetDesc(int(nq), int(nf), keep[2].ctypes.data_as(f64p), keep[3].ctypes.data_as(f64p), keep[4].ctypes.data_as(f64p),
                      len(keep[0]), keep[0].ctypes.data_as(i64p), keep[1].ctypes.data_as(i32p))
        out = ctypes.c_void_p()
        rc = lib().fe_facet_set_create(self._h, ctypes.byref(d), ctypes.byref(out))
        if rc != FE_OK:
            self._raise(rc)
        return FacetSet(self, out)

    def dirichlet(self, rowval, prescribed):
        """fe_dirichlet_create: Dirichlet constraints of this handle's pattern (K.rowval, host,
        1-based) on the 1-based ascending prescribed dofs (ch.prescribed_dofs)."""
        rv = np.ascontiguousarray(rowval, np.int64)
        pd = np.ascontiguousarray(prescribed, np.int64)
        out = ctypes.c_void_p()
        rc = lib().fe_dirichlet_create(self._h, rv.ctypes.data_as(i64p), len(pd), pd.ctypes.data_as(i64p),
                                       ctypes.byref(out))
        if rc != FE_OK:
            self._raise(rc)
        return Dirichlet(self, out, len(pd))

    def element_operator(self, ke_stride, precision: int = PREC_MIXED):
        """fe_element_operator_create: the matrix-free product y (+)= sum_c A_c^T Ke_c A_c u over
        element matrices laid out with ke_stride (elements, Ke(c, I, J) at c*s0 + I*s1 + J*s2;
        float32 for PREC_MIXED, float64 for PREC_FP64)."""
        lay = ElementLayout()
        for k in range(3):
            lay.ke_stride[k] = int(ke_stride[k])
        out = ctypes.c_void_p()
        rc = lib().fe_element_operator_create(self._h, ctypes.byref(lay), int(precision), ctypes.byref(out))
        if rc != FE_OK:
            self._raise(rc)
        return ElementOperator(self, out, precision, tuple(int(v) for v in ke_stride))

    def adjoint(self, u, lam, d_rho, d_X, physics: int, p0: float, p1: float, body=(0.0, 0.0, 0.0), cell_scale=None,
                dscale=None, precision: int = PREC_MIXED, stream=None, sync: bool = True):
        """fe_assemble_adjoint: d_rho[n_cells] = dscale * lam^T (dK/ds) u and d_X[n_nodes*dim] =
        lam^T d(K u - f)/dX, written in place (numpy or torch CUDA buffers; d_X may be None)."""
        _check(u, "u", "float64", self.ndofs)
        _check(lam, "lam", "float64", self.ndofs)
        _check(d_rho, "d_rho", "float64", self.n_cells)
        _check(d_X, "d_X", "float64", self.n_nodes * self.dim)
        _check(cell_scale, "cell_scale", "float64", self.n_cells)
        _check(dscale, "dscale", "float64", self.n_cells)
        p = AdjointParams()
        p.physics, p.precision = physics, precision
        p.flags = 0 if sync else ASYNC
        p.p0, p.p1 = float(p0), float(p1)
        for k in range(3):
            p.body[k] = float(body[k]) if k < len(body) else 0.0
        p.cell_scale = _ptr(cell_scale)
        p.dscale = _ptr(dscale)
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        p.stream = stream
        rc = lib().fe_assemble_adjoint(self._h, ctypes.byref(p), _ptr(u), _ptr(lam), _ptr(d_rho), _ptr(d_X))
        if rc != FE_OK:
            self._raise(rc)
        return d_rho, d_X

    @staticmethod
    def _params(physics, p0, p1, body=(0.0, 0.0, 0.0), cell_scale=None, u=None, precision=PREC_MIXED, fillzero=True,
                cond_threshold=0.0, compensated=True, stream=None, form=None):
        p = AssembleParams()
        p.physics, p.precision = physics, precision
        p.flags = (FILLZERO if fillzero else 0) | (0 if compensated else FP32_SUM) | _FORMS[form]
        p.p0, p.p1 = float(p0), float(p1)
        for k in range(3):
            p.body[k] = float(body[k]) if k < len(body) else 0.0
        p.cell_scale = _ptr(cell_scale)
        p.u = _ptr(u)
        p.cond_threshold = float(cond_threshold)
        p.stream = stream
        return p

    def autotune(self, nzval, f, stage_caps=None, reps: int = 3, stream=None, **assemble_kw):
        """fe_autotune: re-plan with each candidate staging capacity, time every form mask (bit s:
        subdomain s two-phase) unless ``form`` names one, keep the fastest plan and form.
        Returns {"best_stage_cap", "best_ms", "best_form_mask", "candidates": [(cap, ms, tiles,
        visits, form_mask), ...]} (per capacity its fastest form)."""
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        self._check_outputs(nzval, f)
        self._check_fields(assemble_kw.get("u"), assemble_kw.get("cell_scale"))
        p = self._params(stream=stream, **assemble_kw)
        caps = None
        n = 0
        if stage_caps:
            n = len(stage_caps)
            caps = (ctypes.c_int32 * n)(*[int(c) for c in stage_caps])
        res = TuneResult()
        rc = lib().fe_autotune(self._h, ctypes.byref(p), _ptr(nzval), _ptr(f), n, caps, int(reps), ctypes.byref(res))
        if rc != FE_OK:
            self._raise(rc)
        cands = [(res.stage_cap[k], res.ms[k], res.n_tiles[k], res.n_cell_visits[k], res.form_mask[k])
                 for k in range(res.n_candidates)]
        return {"best_stage_cap": res.best_stage_cap, "best_ms": res.best_ms, "best_form_mask": res.best_form_mask,
                "candidates": cands}

    def graph_capture(self, steps, nzvals, fs, stream):
        """fe_graph_capture: steps = list of dicts of assemble() keywords (physics, p0, p1, body,
        cell_scale, u, precision, ...); nzvals / fs = device buffers per step. Returns the graph id."""
        n = len(steps)
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        if len(nzvals) != n or len(fs) != n:
            raise ValueError("one nzval and one f per step")
        for st, nz, fv in zip(steps, nzvals, fs):
            self._check_outputs(nz, fv)
            self._check_fields(st.get("u"), st.get("cell_scale"))
        arr = (AssembleParams * n)(*[self._params(stream=stream, **st) for st in steps])
        nz = (ctypes.c_void_p * n)(*[_ptr(x) for x in nzvals])
        ff = (ctypes.c_void_p * n)(*[_ptr(x) for x in fs])
        gid = ctypes.c_int32()
        rc = lib().fe_graph_capture(self._h, stream, n, arr, nz, ff, ctypes.byref(gid))
        if rc != FE_OK:
            self._raise(rc)
        return gid.value

    def graph_replay(self, graph: int, stream=None, sync: bool = True, profile: bool = False):
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        flags = (0 if sync else ASYNC) | (PROFILE if profile else 0)
        rc = lib().fe_graph_replay(self._h, int(graph), stream, flags)
        if rc != FE_OK:
            self._raise(rc)

    def graph_destroy(self, graph: int):
        rc = lib().fe_graph_destroy(self._h, int(graph))
        if rc != FE_OK:
            self._raise(rc)

    def sync(self):
        rc = lib().fe_sync(self._h)
        if rc != FE_OK:
            self._raise(rc)

    def kernel_time(self):
        """(total ms, launches) of the FE_PROFILE launches since the last call."""
        ms, n = ctypes.c_double(), ctypes.c_int64()
        rc = lib().fe_kernel_time(self._h, ctypes.byref(ms), ctypes.byref(n))
        if rc != FE_OK:
            self._raise(rc)
        return ms.value, n.value

    def info(self) -> dict:
        i = Info()
        lib().fe_get_info(self._h, ctypes.byref(i))
        return {k: getattr(i, k) for k, _ in Info._fields_}

    def index_map(self, cell: int, ld: int):
        """1-based nzval positions of Ke entries of a (1-based) cell: array [ld, ld], Ke[I, J]."""
        out = np.zeros((ld, ld), np.int64, order="F")
        rc = lib().fe_get_index_map(self._h, int(cell), out.ctypes.data_as(i64p))
        if rc != FE_OK:
            self._raise(rc)
        return out


# ---------------------------------------------------------------------------------------
# Ferrite-style front end
# ---------------------------------------------------------------------------------------
@dataclass
class Heat:
    """heat_equation.jl:143-164: Ke += k gradN_i.gradN_j dOmega, fe += source N_i dOmega."""
    k: float = 1.0
    source: float = 1.0
    cell_scale: object = None

    def args(self):
        return dict(physics=HEAT, p0=self.k, p1=self.source, cell_scale=self.cell_scale)


@dataclass
class LinearElasticity:
    """threaded_assembly.jl:105-132 (isotropic C from E, nu); cell_scale multiplies E per cell
    (SIMP, topology_optimization.jl:347-383)."""
    E: float
    nu: float
    body: tuple = (0.0, 0.0, 0.0)
    cell_scale: object = None

    def args(self):
        return dict(physics=LINEAR_ELASTIC, p0=self.E, p1=self.nu, body=self.body, cell_scale=self.cell_scale)


@dataclass
class NeoHooke:
    """hyperelasticity.jl:157-276 (cell part): tangent K and residual g at displacement u."""
    mu: float
    lam: float
    u: object = None
    body: tuple = (0.0, 0.0, 0.0)

    def args(self):
        return dict(physics=NEO_HOOKE, p0=self.mu, p1=self.lam, body=self.body, u=self.u)


class GPUAssembler:
    """What ``start_assemble(K, f)`` returns (src/assembler.jl:287-291), for the device engine."""

    def __init__(self, handle: Handle, nzval, f, fillzero: bool = True, precision: int = PREC_MIXED, stream=None):
        self.handle, self.nzval, self.f = handle, nzval, f
        self.fillzero, self.precision, self.stream = fillzero, precision, stream


def start_assemble(handle: Handle, nzval, f=None, fillzero: bool = True, precision: int = PREC_MIXED, stream=None):
    return GPUAssembler(handle, nzval, f, fillzero, precision, stream)


def assemble(asm: GPUAssembler, element, sync: bool = True):
    """The whole ``for cell in CellIterator(dh); reinit!; element!; assemble!; end`` loop."""
    asm.handle.assemble(asm.nzval, asm.f, precision=asm.precision, fillzero=asm.fillzero, stream=asm.stream,
                        sync=sync, **element.args())
    asm.fillzero = False  # later calls accumulate, like a second loop over the same assembler
    return asm


def finish_assemble(asm: GPUAssembler):
    return asm.nzval, asm.f


class Dirichlet:
    """Dirichlet constraints on a handle's pattern: apply!(K, f, ch) / apply_zero!(K, f, ch)
    on device buffers (torch CUDA tensors). Close it before its handle."""

    def __init__(self, handle, ptr, n_prescribed):
        self._handle = handle
        self._c = ptr
        self.n_prescribed = n_prescribed

    def apply(self, nzval, f=None, inhomogeneities=None, applyzero: bool = False, stream=None, sync: bool = True):
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        g = inhomogeneities
        if isinstance(g, np.ndarray):
            g = np.ascontiguousarray(g, np.float64)
        self._handle._check_outputs(nzval, f)
        _check(g, "inhomogeneities", "float64", self.n_prescribed)
        rc = lib().fe_apply(self._c, _ptr(nzval), _ptr(f), _ptr(g), 1 if applyzero else 0, stream)
        if rc != FE_OK:
            self._handle._raise(rc)
        if sync:
            import torch
            torch.cuda.synchronize()
        return nzval, f

    def apply_zero(self, nzval, f=None, stream=None, sync: bool = True):
        return self.apply(nzval, f, None, True, stream, sync)

    def close(self):
        if self._c:
            lib().fe_dirichlet_destroy(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ElementOperator:
    """y (+)= sum_c A_c^T Ke_c A_c u with element matrices (fe_element_matvec) on device buffers
    (torch CUDA tensors). Close it before its handle."""

    def __init__(self, handle, ptr, precision, ke_stride):
        self._handle = handle
        self._c = ptr
        self.precision = precision
        self.ke_stride = ke_stride

    def matvec(self, ke, u, y, fillzero: bool = True, stream=None, sync: bool = True):
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        h = self._handle
        _check(ke, "ke", _elem_dtype(self.precision), _extent(h.n_cells, h.max_dofs_per_cell, self.ke_stride))
        _check(u, "u", "float64", h.ndofs)
        _check(y, "y", "float64", h.ndofs)
        rc = lib().fe_element_matvec(self._c, _ptr(ke), _ptr(u), _ptr(y), FILLZERO if fillzero else 0, stream)
        if rc != FE_OK:
            self._handle._raise(rc)
        if sync:
            import torch
            torch.cuda.synchronize()
        return y

    def close(self):
        if self._c:
            lib().fe_element_operator_destroy(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FacetSet:
    """Facet loads over a facet set (fe_assemble_facet_load) into a device f (torch CUDA)."""

    def __init__(self, handle, ptr):
        self._handle = handle
        self._c = ptr

    def load(self, f, pressure: float, traction=(0.0, 0.0, 0.0), fillzero: bool = False, stream=None):
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        _check(f, "f", "float64", self._handle.ndofs)
        t = (ctypes.c_double * 3)(*[float(x) for x in list(traction) + [0.0] * (3 - len(traction))])
        rc = lib().fe_assemble_facet_load(self._c, float(pressure), ctypes.cast(t, f64p), FILLZERO if fillzero else 0,
                                          _ptr(f), stream)
        if rc != FE_OK:
            self._handle._raise(rc)
        return f

    def close(self):
        if self._c:
            lib().fe_facet_set_destroy(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
