"""Dirichlet constraints on the device (fe_dirichlet_create / fe_apply) against the oracle's
apply! (ConstraintHandler.jl:711-744) on the same assembled matrix.

Every entry except the prescribed diagonals (m = meandiag(K)) and f at the prescribed dofs
(g m) must agree bitwise: zeroing is exact and f -= K g follows the reference's per-row
operation order. m is a fixed-order parallel sum here and a serial sum in the reference:
relative difference <= 1e-14."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

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


def boundary_dofs(O, prob, which):
    """1-based dofs (ascending) of the nodes selected by which(x) (vertex dofs only)."""
    x = prob.nodes
    nc = prob.ndofs_per_cell(0) // len(prob.cells_of(0))
    out = set()
    for c in range(prob.n_cells):
        nodes = prob.cells_of(c) - 1
        d = prob.celldofs(c)
        for k, n in enumerate(nodes):
            comps = which(x[n])
            for a in comps:
                out.add(int(d[k * nc + a]))
    return np.array(sorted(out), np.int64)


def run_case(fg, O, torch, prob, kw_f, pd, g, applyzero, with_f=True, form=None):
    h = make_handle(fg, O, prob)
    nz = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    f = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    h.assemble(nz, f, precision=fg.PREC_FP64, form=form, **kw_f)
    nz_o, f_o = nz.cpu().numpy().copy(), f.cpu().numpy().copy()
    ch = h.dirichlet(prob.rowval, pd)
    ch.apply(nz, f if with_f else None, g, applyzero=applyzero)
    prob.apply(nz_o, f_o if with_f else None, pd, g, applyzero=applyzero)
    nz_d, f_d = nz.cpu().numpy(), f.cpu().numpy()
    # the prescribed diagonals
    dpos = np.array([np.searchsorted(prob.rowval[prob.colptr[d - 1] - 1:prob.colptr[d] - 1], d) + prob.colptr[d - 1] - 1
                     for d in pd])
    mask = np.ones(prob.nnz, bool)
    mask[dpos] = False
    assert np.array_equal(nz_d[mask], nz_o[mask])
    assert np.allclose(nz_d[dpos], nz_o[dpos], rtol=1e-14, atol=0)
    if with_f:
        free = np.ones(prob.ndofs, bool)
        free[pd - 1] = False
        assert np.array_equal(f_d[free], f_o[free])
        assert np.allclose(f_d[pd - 1], f_o[pd - 1], rtol=1e-14, atol=0)
    else:
        assert np.array_equal(f.cpu().numpy(), f_o)  # untouched
    ch.close()
    return nz_d, f_d


def test_apply_heat_inhomogeneous(built, oracle, torch_cuda):
    fg, O, torch = built, oracle, torch_cuda
    prob = O.box_problem(O.QUADRILATERAL, (12, 10), qr_order=2, perturb=0.2, seed=41)
    pd = boundary_dofs(O, prob, lambda x: [0] if abs(abs(x[0]) - 1) < 1e-12 or abs(abs(x[1]) - 1) < 1e-12 else [])
    g = np.random.default_rng(1).normal(size=len(pd))
    nz, f = run_case(fg, O, torch, prob, dict(physics=fg.HEAT, p0=1.0, p1=1.0), pd, g, False)
    u = spla.spsolve(prob.to_scipy(nz).tocsc(), f)
    assert np.allclose(u[pd - 1], g, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("applyzero,with_f", [(False, True), (True, True), (False, False)])
def test_apply_elastic_componentwise(built, oracle, torch_cuda, applyzero, with_f):
    """Clamped x = -1 face (all components), u_z prescribed on z = 1 (one component)."""
    fg, O, torch = built, oracle, torch_cuda
    prob = O.box_problem(O.HEXAHEDRON, (5, 4, 4), ncomp=3, perturb=0.2, seed=42)

    def sel(x):
        c = []
        if abs(x[0] + 1) < 1e-12:
            c = [0, 1, 2]
        elif abs(x[2] - 1) < 1e-12:
            c = [2]
        return c
    pd = boundary_dofs(O, prob, sel)
    g = np.where(np.arange(len(pd)) % 3 == 0, 0.0, 0.01 * np.arange(len(pd)))
    run_case(fg, O, torch, prob, dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0)), pd, g,
             applyzero, with_f)


def test_apply_q2_two_phase(built, oracle, torch_cuda):
    fg, O, torch = built, oracle, torch_cuda
    prob = O.box_problem(O.HEXAHEDRON, (3, 2, 2), ip_order=2, ncomp=3, qr_order=3, perturb=0.2, seed=43)
    rng = np.random.default_rng(2)
    pd = np.sort(rng.choice(prob.ndofs, 40, replace=False)) + 1
    g = rng.normal(size=len(pd))
    run_case(fg, O, torch, prob, dict(physics=fg.LINEAR_ELASTIC, p0=1.0, p1=0.3, body=(0.0, 1.0, 0.0)), pd, g, False)


def test_apply_errors(built, oracle, torch_cuda):
    fg, O = built, oracle
    prob = O.box_problem(O.QUADRILATERAL, (3, 3), qr_order=2)
    h = make_handle(fg, O, prob)
    with pytest.raises(fg.FEError) as e:
        h.dirichlet(prob.rowval, np.array([3, 2], np.int64))
    assert e.value.name == "ARG"
    with pytest.raises(fg.FEError) as e:
        h.dirichlet(prob.rowval, np.array([1, prob.ndofs + 1], np.int64))
    assert e.value.name == "BOUNDS"


def test_apply_without_prescribed_dofs(built, oracle, torch_cuda):
    torch = torch_cuda
    fg, O = built, oracle
    prob = O.box_problem(O.QUADRILATERAL, (4, 3), qr_order=2)
    h = make_handle(fg, O, prob)
    nz = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    f = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    h.assemble(nz, f, physics=fg.HEAT, p0=1.0, p1=1.0)
    nz0, f0 = nz.clone(), f.clone()
    ch = h.dirichlet(prob.rowval, np.zeros(0, np.int64))
    ch.apply(nz, f, None)
    assert torch.equal(nz, nz0) and torch.equal(f, f0)
    ch.close()
