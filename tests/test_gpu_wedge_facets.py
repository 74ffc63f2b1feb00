"""Facet loads on wedges (RefPrism): triangle facets 1 and 5 with the triangle rule,
quadrilateral facets 2-4 with a quarter of the Gauss weights, padded to one length
(host.facet_values). Device against the oracle's serial FP64 loop with the same tables, equal to
the last bit (1e-15 relative margin), on a box whose every node is moved."""
import numpy as np
import pytest

from helpers import boundary_facets, make_handle
from test_gpu_facet import shaken

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_wedge_facet_loads_against_oracle(fg, oracle, torch_cuda):
    torch = torch_cuda
    fg.build()
    O = oracle
    host = __import__("ferrite_gb300.host", fromlist=["host"])
    ct, nel, ip, nc, qo = O.WEDGE, (3, 3, 2), 1, 3, 2
    prob, base = shaken(O, ct, nel, ip, nc, qo, seed=75)
    # two sides (quadrilateral facets) and the top (triangle facets), on the unperturbed nodes
    sel = [boundary_facets(prob, ct, lambda X: abs(X[0] - 1.0) < 1e-12, base),
           boundary_facets(prob, ct, lambda X: abs(X[1]) < 1e-12, base),
           boundary_facets(prob, ct, lambda X: abs(X[2] - 1.0) < 1e-12, base)]
    cells = np.concatenate([c for c, _ in sel])
    facets = np.concatenate([f for _, f in sel])
    assert {2, 5} <= set(facets.tolist())
    tabs = host.facet_values(ct, ip, 2)
    h = make_handle(fg, O, prob)
    fs = h.facet_set(cells, facets, tabs)
    t = (0.3, -1.2, 0.7)
    f0 = np.random.default_rng(1).normal(size=prob.ndofs)
    ref = prob.facet_load(cells, facets, tabs, pressure=-2.5, traction=t, f=f0.copy())
    fd = torch.as_tensor(f0.copy(), device="cuda")
    fs.load(fd, pressure=-2.5, traction=t)
    got = fd.cpu().numpy()
    assert np.allclose(got, ref, rtol=1e-15, atol=0), np.abs(got - ref).max()
    fs.close()
    h.close()
