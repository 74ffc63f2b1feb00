"""GPU adjoint (fe_assemble_adjoint, through the C ABI) against the oracle's FP64 adjoint, which
tests/test_oracle_adjoint.py pins to central finite differences of the assembly.

Tolerances, max abs error relative to the largest entry of each output:
  FE_PREC_FP64 <= 1e-11; FE_PREC_MIXED (FP32 per cell, FP64 node sums) <= 2e-5 for d_X, whose
  node sums cancel strongly (the per-cell terms are ~100x the sums), 2e-6 for d_rho."""
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


@pytest.fixture(scope="module")
def built(fg, torch_cuda):
    fg.build()
    return fg


def rel_max(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def run_case(fg, O, prob, phys_fg, phys_or, p0, p1, body, seed, tol_mixed=(2e-6, 2e-5)):
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.01, 1.0, prob.n_cells)
    scale, dscale = rho ** 3, 3 * rho ** 2
    u = rng.normal(0, 1e-3, prob.ndofs)
    lam = rng.normal(0, 1e-3, prob.ndofs)
    ref_cell, ref_X = prob.adjoint(phys_or, p0, p1, u, lam, body=body, cell_scale=scale, dscale=dscale)
    h = make_handle(fg, O, prob)
    out = {}
    for prec, (t_cell, t_X) in ((1, (1e-11, 1e-11)), (0, tol_mixed)):
        d_rho = np.full(prob.n_cells, np.nan)
        d_X = np.full(prob.nodes.shape[0] * prob.dim, np.nan)
        h.adjoint(u, lam, d_rho, d_X, phys_fg, p0, p1, body=body or (0.0, 0.0, 0.0), cell_scale=scale, dscale=dscale,
                  precision=prec)
        assert rel_max(d_rho, ref_cell) <= t_cell, (prec, rel_max(d_rho, ref_cell))
        assert rel_max(d_X, ref_X.ravel()) <= t_X, (prec, rel_max(d_X, ref_X.ravel()))
        out[prec] = (d_rho, d_X)
    return h, out, (u, lam, scale, dscale)


def test_adjoint_hex_elastic_cantilever(built, oracle):
    """SIMP cantilever slab (the benchmark's (96,48,48) on [0,2]x[0,1]^2, scaled down)."""
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (12, 6, 6), [0, 0, 0], [2, 1, 1], ncomp=3, perturb=0.2, seed=4)
    run_case(fg, O, prob, fg.LINEAR_ELASTIC, O.LINEAR_ELASTIC, 1.0, 0.3, (0.0, 0.0, -1.0), 21)


def test_adjoint_tet_elastic(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.TETRAHEDRON, (4, 3, 3), ncomp=3, qr_order=1, perturb=0.15, seed=8)
    run_case(fg, O, prob, fg.LINEAR_ELASTIC, O.LINEAR_ELASTIC, 2.0, 0.25, (0.5, 0.0, -1.0), 3)


def test_adjoint_heat_quad(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.QUADRILATERAL, (20, 15), ncomp=1, perturb=0.2, seed=6)
    run_case(fg, O, prob, fg.HEAT, O.HEAT, 1.0, 1.0, None, 5)


def test_adjoint_reproducible_and_device_buffers(built, oracle, torch_cuda):
    torch = torch_cuda
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (6, 5, 4), ncomp=3, perturb=0.2, seed=2)
    h, out, (u, lam, scale, dscale) = run_case(fg, O, prob, fg.LINEAR_ELASTIC, O.LINEAR_ELASTIC, 1.0, 0.3,
                                               (0.0, 0.0, -1.0), 9)
    dev = lambda a: torch.as_tensor(a, device="cuda")
    d_rho = torch.empty(prob.n_cells, dtype=torch.float64, device="cuda")
    d_X = torch.empty(prob.nodes.shape[0] * 3, dtype=torch.float64, device="cuda")
    h.adjoint(dev(u), dev(lam), d_rho, d_X, fg.LINEAR_ELASTIC, 1.0, 0.3, body=(0.0, 0.0, -1.0), cell_scale=dev(scale),
              dscale=dev(dscale), precision=0)
    assert np.array_equal(d_rho.cpu().numpy(), out[0][0])
    assert np.array_equal(d_X.cpu().numpy(), out[0][1])


def test_adjoint_unsupported_physics(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (2, 2, 2), ncomp=3)
    h = make_handle(fg, O, prob)
    z = np.zeros(prob.ndofs)
    with pytest.raises(fg.FEError) as e:
        h.adjoint(z, z, np.zeros(prob.n_cells), None, fg.NEO_HOOKE, 1.0, 10.0)
    assert e.value.code == 5
