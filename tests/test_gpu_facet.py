"""Facet (Neumann) loads on the device (fe_facet_set_create / fe_assemble_facet_load) against
the oracle's restatement of FacetValues reinit! and the facet-load loop (FP64 both, same
operation order): equal to the last bit, checked with a 1e-15 relative margin."""
import numpy as np
import pytest

from helpers import boundary_facets, facet_tables, make_handle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def built(fg, torch_cuda):
    fg.build()
    return fg


def shaken(O, ct, nel, ip, nc, qo, seed):
    """A box problem with every node moved (facets curved and tilted)."""
    d = len(nel)
    prob = O.box_problem(ct, nel, [0.0] * d, [1.0] * d, ip_order=ip, ncomp=nc, qr_order=qo)
    base = prob.nodes.copy()
    h = 1.0 / max(nel)
    prob.nodes = np.ascontiguousarray(base + np.random.default_rng(seed).uniform(-0.15 * h, 0.15 * h, base.shape))
    return prob, base


@pytest.mark.parametrize("case", ["hex_q1", "hex_q2", "tet", "quad_heat", "tri_heat"])
def test_facet_loads_against_oracle(built, oracle, torch_cuda, case):
    torch = torch_cuda
    fg, O = built, oracle
    if case == "hex_q1":
        ct, nel, ip, nc, qo, fq = O.HEXAHEDRON, (4, 3, 3), 1, 3, 2, 2
    elif case == "hex_q2":
        ct, nel, ip, nc, qo, fq = O.HEXAHEDRON, (2, 2, 2), 2, 3, 3, 3
    elif case == "tet":
        ct, nel, ip, nc, qo, fq = O.TETRAHEDRON, (3, 2, 2), 1, 3, 1, 2
    elif case == "quad_heat":
        ct, nel, ip, nc, qo, fq = O.QUADRILATERAL, (6, 5), 1, 1, 2, 3
    else:
        ct, nel, ip, nc, qo, fq = O.TRIANGLE, (5, 4), 1, 1, 2, 2
    prob, base = shaken(O, ct, nel, ip, nc, qo, seed=70 + len(case))
    # two sides of the box, selected on the unperturbed nodes
    sel = [boundary_facets(prob, ct, lambda X: abs(X[0] - 1.0) < 1e-12, base),
           boundary_facets(prob, ct, lambda X: abs(X[1]) < 1e-12, base)]
    cells = np.concatenate([c for c, _ in sel])
    facets = np.concatenate([f for _, f in sel])
    tabs = facet_tables(O, ct, ip, fq)
    h = make_handle(fg, O, prob)
    fs = h.facet_set(cells, facets, tabs)
    t = (0.3, -1.2, 0.7)
    f0 = np.random.default_rng(1).normal(size=prob.ndofs)
    ref = prob.facet_load(cells, facets, tabs, pressure=-2.5, traction=t, f=f0.copy())
    fd = torch.as_tensor(f0.copy(), device="cuda")
    fs.load(fd, pressure=-2.5, traction=t)
    got = fd.cpu().numpy()
    assert np.allclose(got, ref, rtol=1e-15, atol=0), np.abs(got - ref).max()
    # fill-zero: the loads alone
    fs.load(fd, pressure=-2.5, traction=t, fillzero=True)
    ref0 = prob.facet_load(cells, facets, tabs, pressure=-2.5, traction=t)
    assert np.allclose(fd.cpu().numpy(), ref0, rtol=1e-15, atol=0)
    fs.close()


def test_facet_set_errors(built, oracle, torch_cuda):
    fg, O = built, oracle
    prob = O.box_problem(O.QUADRILATERAL, (3, 3), qr_order=2)
    h = make_handle(fg, O, prob)
    tabs = facet_tables(O, O.QUADRILATERAL, 1, 2)
    with pytest.raises(fg.FEError) as e:
        h.facet_set(np.array([1], np.int64), np.array([5], np.int32), tabs)
    assert e.value.name == "BOUNDS"
    with pytest.raises(fg.FEError) as e:
        h.facet_set(np.array([prob.n_cells + 1], np.int64), np.array([1], np.int32), tabs)
    assert e.value.name == "BOUNDS"


def test_empty_facet_set(built, oracle, torch_cuda):
    torch = torch_cuda
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (2, 2, 2), ncomp=3)
    h = make_handle(fg, O, prob)
    fs = h.facet_set(np.zeros(0, np.int64), np.zeros(0, np.int32), facet_tables(O, O.HEXAHEDRON, 1, 2))
    f = torch.ones(prob.ndofs, dtype=torch.float64, device="cuda")
    fs.load(f, pressure=1.0)
    assert bool((f == 1).all())
    fs.load(f, pressure=1.0, fillzero=True)
    assert bool((f == 0).all())
