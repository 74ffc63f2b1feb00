"""fe_assemble_noalloc: the allocation-free entry point, for callers that cannot allocate
device memory (its FP32 input copies live in a static 16 MiB device array instead of buffers
the library would cudaMalloc on first use).

Called through the C ABI directly and compared with fe_assemble on the same handle, twice in
a row (the static array keeps the previous call's contents; each call must overwrite what it
reads). Both entry points run the same kernel on the same FP32 inputs, so the outputs must be
equal bit for bit. Collected last so that a failure here cannot hide the results of the other
tests.
"""
import ctypes

import numpy as np
import pytest

from helpers import make_handle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def noalloc(fg, h, nz, f, physics, p0, p1, u=None, cell_scale=None, body=(0.0, 0.0, 0.0), stream=None, flags=None):
    p = fg.AssembleParams()
    p.physics, p.precision, p.flags = physics, fg.PREC_MIXED, fg.FILLZERO if flags is None else flags
    p.p0, p.p1 = p0, p1
    for k in range(3):
        p.body[k] = body[k]
    p.u = u.data_ptr() if u is not None else None
    p.cell_scale = cell_scale.data_ptr() if cell_scale is not None else None
    p.cond_threshold = 0.0
    p.stream = stream.cuda_stream if stream is not None else None
    return fg.lib().fe_assemble_noalloc(h.ptr, ctypes.byref(p), ctypes.c_void_p(nz.data_ptr()), ctypes.c_void_p(f.data_ptr()))


def _pair(torch, prob):
    ref = (torch.zeros(prob.nnz, dtype=torch.float64, device="cuda"),
           torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda"))
    out = (torch.full((prob.nnz,), float("nan"), dtype=torch.float64, device="cuda"),
           torch.full((prob.ndofs,), float("nan"), dtype=torch.float64, device="cuda"))
    return ref, out


def test_noalloc_matches_fe_assemble_twice(fg, oracle, torch_cuda):
    torch, O = torch_cuda, oracle
    fg.build()
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(3)
    # Neo-Hooke with u and a cell factor in one call: the FP32 copy of u and then the cell
    # factors share the static scratch, so a wrong offset of the second would overwrite the
    # first and change K and f
    prob = O.box_problem(O.HEXAHEDRON, (5, 4, 3), [0, 0, 0], [1, 1, 1], ip_order=1, ncomp=3, qr_order=2,
                         perturb=0.15, seed=8)
    h = make_handle(fg, O, prob)
    for call in range(2):
        u = torch.tensor(0.05 * rng.uniform(-1, 1, prob.ndofs), dtype=torch.float64, device="cuda")
        scale = torch.tensor(rng.uniform(0.5, 2.0, prob.n_cells), dtype=torch.float64, device="cuda")
        (ref_nz, ref_f), (nz, f) = _pair(torch, prob)
        h.assemble(ref_nz, ref_f, physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, u=u, cell_scale=scale, stream=stream)
        assert noalloc(fg, h, nz, f, fg.NEO_HOOKE, 1.0, 10.0, u=u, cell_scale=scale, stream=stream) == fg.FE_OK
        torch.cuda.synchronize()
        assert torch.equal(nz, ref_nz), call
        assert torch.equal(f, ref_f), call
    # SIMP-style per-cell modulus: the FP32 copy of the cell factors goes to the scratch too
    prob = O.box_problem(O.HEXAHEDRON, (4, 4, 4), [0, 0, 0], [1, 1, 1], ip_order=1, ncomp=3, qr_order=2,
                         perturb=0.1, seed=9)
    h = make_handle(fg, O, prob)
    for call in range(2):
        scale = torch.tensor(rng.uniform(0.01, 1.0, prob.n_cells) ** 3, dtype=torch.float64, device="cuda")
        (ref_nz, ref_f), (nz, f) = _pair(torch, prob)
        h.assemble(ref_nz, ref_f, physics=fg.LINEAR_ELASTIC, p0=1.0, p1=0.3, cell_scale=scale, body=(0, 0, -1),
                   stream=stream)
        assert noalloc(fg, h, nz, f, fg.LINEAR_ELASTIC, 1.0, 0.3, cell_scale=scale, body=(0.0, 0.0, -1.0),
                       stream=stream) == fg.FE_OK
        torch.cuda.synchronize()
        assert torch.equal(nz, ref_nz), call
        assert torch.equal(f, ref_f), call


def test_noalloc_rejects_host_buffers(fg, oracle, torch_cuda):
    O = oracle
    fg.build()
    prob = O.box_problem(O.QUADRILATERAL, (4, 4), qr_order=2)
    h = make_handle(fg, O, prob)
    p = fg.AssembleParams()
    p.physics, p.precision, p.flags, p.p0, p.p1 = fg.HEAT, fg.PREC_MIXED, fg.FILLZERO, 1.0, 1.0
    nz, f = np.zeros(prob.nnz), np.zeros(prob.ndofs)
    rc = fg.lib().fe_assemble_noalloc(h.ptr, ctypes.byref(p), ctypes.c_void_p(nz.ctypes.data), ctypes.c_void_p(f.ctypes.data))
    assert rc == fg.FE_ERR_ARG


def test_noalloc_refuses_a_synchronous_call_on_a_capturing_stream(fg, oracle, torch_cuda):
    torch, O = torch_cuda, oracle
    fg.build()
    prob = O.box_problem(O.QUADRILATERAL, (4, 4), qr_order=2)
    h = make_handle(fg, O, prob)
    (ref_nz, ref_f), (nz, f) = _pair(torch, prob)
    side = torch.cuda.Stream()
    # the first call on this device resolves the scratch address outside any capture
    assert noalloc(fg, h, nz, f, fg.HEAT, 1.0, 1.0, stream=side) == fg.FE_OK
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
        rc = noalloc(fg, h, nz, f, fg.HEAT, 1.0, 1.0, stream=side)
    assert rc == fg.FE_ERR_STATE
    # the handle still works afterwards, with the same bits as fe_assemble
    assert noalloc(fg, h, nz, f, fg.HEAT, 1.0, 1.0, stream=side) == fg.FE_OK
    h.assemble(ref_nz, ref_f, physics=fg.HEAT, p0=1.0, p1=1.0, stream=side)
    torch.cuda.synchronize()
    assert torch.equal(nz, ref_nz)
    assert torch.equal(f, ref_f)
