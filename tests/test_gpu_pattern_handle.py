"""fe_create on a device-resident pattern (the output of fe_sparsity_pattern_device, as a
CuSparseMatrixCSC's colPtr / rowVal would be): the handle assembles bitwise the same as one made
from the host pattern."""
import pytest

from test_gpu_pattern import single

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def host(fg, torch_cuda):
    fg.build()
    return __import__("ferrite_gb300.host", fromlist=["host"])


def test_handle_on_device_pattern(fg, host, torch_cuda):
    """The device pattern goes straight into fe_create (a CuSparseMatrixCSC-style flow: pattern,
    set-up and nzval all on the device); the assembly is bitwise that of a host-pattern handle."""
    torch = torch_cuda
    dh = single(host, host.HEXAHEDRON, (6, 5, 4), 1, 3, 0.2)
    cvs = [host.CellValues(host.HEXAHEDRON, 1, 2)]
    cp_h, rv_h = dh.allocate_matrix()
    cp_d, rv_d = dh.allocate_matrix(device=True)
    h_h = dh.handle(cvs, cp_h, rv_h)
    h_d = dh.handle(cvs, cp_d, rv_d)
    assert h_d.nnz == h_h.nnz == len(rv_h)
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0))
    out = []
    for h in (h_h, h_d):
        nz = torch.zeros(h.nnz, dtype=torch.float64, device="cuda")
        f = torch.zeros(dh.ndofs, dtype=torch.float64, device="cuda")
        h.assemble(nz, f, **kw)
        out.append((nz, f))
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])
    h_h.close()
    h_d.close()
