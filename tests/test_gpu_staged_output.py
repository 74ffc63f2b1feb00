"""FE_STAGED_OUTPUT: page-locked host nzval/f assembled into a device buffer held by the handle
and copied back by the copy engine (instead of the kernels storing through the host mapping):
the same bits as device outputs, with and without fill-zero."""
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


def test_staged_pinned_outputs_equal_device_outputs(fg, oracle, torch_cuda):
    torch = torch_cuda
    fg.build()
    O = oracle
    prob = O.box_problem(O.HEXAHEDRON, (6, 5, 4), ncomp=3, perturb=0.2, seed=51)
    h = make_handle(fg, O, prob)
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0))
    nz_d = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    f_d = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    h.assemble(nz_d, f_d, **kw)
    nz_p = torch.full((prob.nnz,), float("nan"), dtype=torch.float64).pin_memory()
    f_p = torch.full((prob.ndofs,), float("nan"), dtype=torch.float64).pin_memory()
    h.assemble(nz_p, f_p, staged_output=True, **kw)
    assert torch.equal(nz_p, nz_d.cpu()) and torch.equal(f_p, f_d.cpu())
    h.assemble(nz_p, f_p, fillzero=False, staged_output=True, **kw)
    h.assemble(nz_d, f_d, fillzero=False, **kw)
    assert torch.equal(nz_p, nz_d.cpu()) and torch.equal(f_p, f_d.cpu())
    h.close()
