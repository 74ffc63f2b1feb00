"""allocate_matrix(dh) on the device (fe_sparsity_pattern_device) against the host
fe_sparsity_pattern (itself checked bit for bit against the oracle's restatement of
sparsity_pattern.jl in tests/test_host.py): identical colptr and rowval."""
import numpy as np
import pytest

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


def single(host, ct, nel, order, nc, perturb=0.0):
    d = len(nel)
    g = host.generate_grid(ct, nel, (0,) * d, (1,) * d)
    if perturb:
        g = host.perturb_interior(g, nel, perturb, 3, (0,) * d, (1,) * d)
    return host.DofHandler.from_grid(g, ip_order=order, n_components=nc).close()


def mixed(host):
    nx, ny, nz = 6, 3, 3
    g = host.generate_grid(host.HEXAHEDRON, (nx, ny, nz), (0, 0, 0), (2, 1, 1))
    cubes = g.cells
    ix = np.arange(cubes.shape[0]) % nx
    T = np.array([[1, 2, 4, 8], [1, 5, 2, 8], [2, 3, 4, 8], [2, 7, 3, 8], [2, 5, 6, 8], [2, 6, 7, 8]]) - 1
    W = np.array([[1, 2, 4, 5, 6, 8], [2, 3, 4, 6, 7, 8]]) - 1
    hexes = cubes[ix < 2]
    tets = cubes[(ix >= 2) & (ix < 4)][:, T].reshape(-1, 4)
    wedges = cubes[ix >= 4][:, W].reshape(-1, 6)
    dh = host.DofHandler(g.nodes, len(hexes) + len(tets) + len(wedges))
    o = 0
    for ct, cn in ((host.HEXAHEDRON, hexes), (host.TETRAHEDRON, tets), (host.WEDGE, wedges)):
        dh.add(ct, np.ascontiguousarray(cn, np.int64), np.arange(o + 1, o + len(cn) + 1, dtype=np.int64), 1, 3)
        o += len(cn)
    return dh.close()


@pytest.mark.parametrize("case", ["hex_q1_vec", "hex_q2_vec", "quad_q1", "quad_q2", "tet_vec", "tri", "mixed"])
def test_device_pattern_equals_host(host, torch_cuda, case):
    torch = torch_cuda
    if case == "hex_q1_vec":
        dh = single(host, host.HEXAHEDRON, (7, 6, 5), 1, 3, 0.2)
    elif case == "hex_q2_vec":
        dh = single(host, host.HEXAHEDRON, (3, 3, 2), 2, 3)
    elif case == "quad_q1":
        dh = single(host, host.QUADRILATERAL, (20, 15), 1, 1)
    elif case == "quad_q2":
        dh = single(host, host.QUADRILATERAL, (9, 7), 2, 1)
    elif case == "tet_vec":
        dh = single(host, host.TETRAHEDRON, (4, 3, 3), 1, 3)
    elif case == "tri":
        dh = single(host, host.TRIANGLE, (8, 5), 1, 1)
    else:
        dh = mixed(host)
    cp_h, rv_h = dh.allocate_matrix()
    cp_d, rv_d = dh.allocate_matrix(device=True)
    assert np.array_equal(cp_d.cpu().numpy(), cp_h)
    assert np.array_equal(rv_d.cpu().numpy(), rv_h)

