"""fe_create on a device-resident pattern (the output of fe_sparsity_pattern_device, as a
CuSparseMatrixCSC's colPtr / rowVal would be): only colptr comes to the host; the entity-blocked
pattern check and the rank tables (the element -> nzval index map) are built on the device. The
handle has the same plan (digest), the same index map and assembles bitwise the same as one made
from the host pattern; a pattern that is not entity-blocked is refused the same way."""
import numpy as np
import pytest

from test_gpu_pattern import mixed, single

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


def _case(host, case):
    if case == "hex_q1_vec":
        return single(host, host.HEXAHEDRON, (6, 5, 4), 1, 3, 0.2), [host.CellValues(host.HEXAHEDRON, 1, 2)], 3
    if case == "hex_q2_vec":
        return single(host, host.HEXAHEDRON, (3, 3, 2), 2, 3), [host.CellValues(host.HEXAHEDRON, 2, 3)], 3
    if case == "quad_q1_heat":
        return single(host, host.QUADRILATERAL, (20, 15), 1, 1), [host.CellValues(host.QUADRILATERAL, 1, 2)], 1
    dh = mixed(host)
    return dh, [host.CellValues(host.HEXAHEDRON, 1, 2), host.CellValues(host.TETRAHEDRON, 1, 1),
                host.CellValues(host.WEDGE, 1, 2)], 3


@pytest.mark.parametrize("case", ["hex_q1_vec", "hex_q2_vec", "quad_q1_heat", "mixed"])
def test_handle_on_device_pattern(fg, host, torch_cuda, case):
    """The device pattern goes straight into fe_create (a CuSparseMatrixCSC-style flow: pattern,
    set-up and nzval all on the device); plan digest, index map and assembly are those of a
    host-pattern handle."""
    torch = torch_cuda
    dh, cvs, nc = _case(host, case)
    cp_h, rv_h = dh.allocate_matrix()
    cp_d, rv_d = dh.allocate_matrix(device=True)
    h_h = dh.handle(cvs, cp_h, rv_h)
    h_d = dh.handle(cvs, cp_d, rv_d)
    assert h_d.nnz == h_h.nnz == len(rv_h)
    assert h_d.info()["plan_checksum"] == h_h.info()["plan_checksum"]
    ld = max(h_h.max_dofs_per_cell, 1)
    for cell in np.linspace(1, dh.n_cells, 7).astype(int):
        assert np.array_equal(h_d.index_map(int(cell), ld), h_h.index_map(int(cell), ld)), cell
    kw = (dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0)[:3]) if nc > 1
          else dict(physics=fg.HEAT, p0=1.0, p1=1.0))
    out = []
    for h in (h_h, h_d):
        nz = torch.zeros(h.nnz, dtype=torch.float64, device="cuda")
        f = torch.zeros(dh.ndofs, dtype=torch.float64, device="cuda")
        h.assemble(nz, f, **kw)
        out.append((nz, f))
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])
    h_h.close()
    h_d.close()


def test_device_pattern_not_entity_blocked_is_refused(fg, host, torch_cuda):
    """Two rows of one column swapped: the host check and the device check both refuse the
    pattern (FE_ERR_UNSUPPORTED, the failing column reported)."""
    torch = torch_cuda
    dh, cvs, _ = _case(host, "hex_q1_vec")
    cp_h, rv_h = dh.allocate_matrix()
    bad_h = rv_h.copy()
    k = int(cp_h[10]) - 1  # column 10 (0-based 9): its first two rows swapped
    bad_h[k], bad_h[k + 1] = bad_h[k + 1], bad_h[k]
    bad_d = torch.as_tensor(bad_h, device="cuda")
    cp_d = torch.as_tensor(cp_h, device="cuda")
    errs = []
    for cp, rv in ((cp_h, bad_h), (cp_d, bad_d)):
        with pytest.raises(fg.FEError) as ei:
            dh.handle(cvs, cp, rv)
        errs.append(ei.value)
    assert errs[0].code == errs[1].code == fg.FE_ERR_UNSUPPORTED
    assert errs[0].col == errs[1].col == 10  # the failing entity's first column, 1-based
