"""Element assembly (fe_assemble_elements): every cell's Ke and fe into device arrays, the
"Element Assembly" kernel of the GPU how-to (gpu_assembly.jl:270-303), against the oracle's
element routine (or_element_matrix) cell by cell.

Tolerances (relative Frobenius norm over all cells): FP64 1e-12, mixed (FP32 output) 1e-6."""
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


def oracle_elements(prob, n_cells, nbf, **kw):
    Ke = np.zeros((n_cells, nbf, nbf))
    fe = np.zeros((n_cells, nbf))
    for c in range(n_cells):
        k, f = prob.element(c, **kw)
        Ke[c], fe[c] = k, f
    return Ke, fe


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("case", ["hex_q1_elastic", "hex_q2_elastic_scaled", "quad_heat", "tet_neo"])
def test_elements_against_oracle(built, oracle, torch_cuda, case):
    torch = torch_cuda
    fg, O = built, oracle
    if case == "hex_q1_elastic":
        prob = O.box_problem(O.HEXAHEDRON, (4, 3, 3), ncomp=3, perturb=0.2, seed=31)
        kf = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0))
        ko = dict(physics=O.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0))
    elif case == "hex_q2_elastic_scaled":
        prob = O.box_problem(O.HEXAHEDRON, (2, 2, 2), ip_order=2, ncomp=3, qr_order=3, perturb=0.2, seed=32)
        sc = np.random.default_rng(4).lognormal(0.0, 0.5, prob.n_cells)
        kf = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 1.0, 0.0), cell_scale=sc)
        ko = dict(physics=O.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 1.0, 0.0), cell_scale=sc)
    elif case == "quad_heat":
        prob = O.box_problem(O.QUADRILATERAL, (7, 5), perturb=0.2, seed=33)
        kf = dict(physics=fg.HEAT, p0=1.0, p1=1.0)
        ko = dict(physics=O.HEAT, p0=1.0, p1=1.0)
    else:
        prob = O.box_problem(O.TETRAHEDRON, (3, 2, 2), ncomp=3, qr_order=1, perturb=0.15, seed=34)
        u = 0.05 * np.random.default_rng(5).uniform(-1, 1, prob.ndofs)
        kf = dict(physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, u=u)
        ko = dict(physics=O.NEO_HOOKE, p0=1.0, p1=10.0, u=u)
    h = make_handle(fg, O, prob)
    n, nbf = prob.n_cells, prob.ndofs_per_cell(0)
    Ke_ref, fe_ref = oracle_elements(prob, n, nbf, **ko)
    for prec, dt, tol in ((fg.PREC_FP64, torch.float64, 1e-12), (fg.PREC_MIXED, torch.float32, 1e-6)):
        # row-major [cell, I, J] (per-cell contiguous)
        ke = torch.full((n, nbf, nbf), float("nan"), dtype=dt, device="cuda")
        fe = torch.full((n, nbf), float("nan"), dtype=dt, device="cuda")
        h.assemble_elements(ke, fe, precision=prec, **kf)
        assert rel(ke.double().cpu().numpy(), Ke_ref) <= tol, (prec, rel(ke.double().cpu().numpy(), Ke_ref))
        assert rel(fe.double().cpu().numpy(), fe_ref) <= tol
        # the how-to's layout: Kes[ncells, nbf, nbf] in Julia (column-major): cell fastest
        kj = torch.full((nbf * nbf * n,), float("nan"), dtype=dt, device="cuda")
        fj = torch.full((nbf * n,), float("nan"), dtype=dt, device="cuda")
        h.assemble_elements(kj, fj, precision=prec, ke_stride=(1, n, n * nbf), fe_stride=(1, n), **kf)
        kj = kj.reshape(nbf, nbf, n).permute(2, 1, 0)  # [J][I][c] memory -> [c, I, J]
        fj = fj.reshape(nbf, n).permute(1, 0)
        assert torch.equal(kj, ke) and torch.equal(fj, fe)


def test_elements_sum_to_global_assembly(built, oracle, torch_cuda):
    """Scattering the element matrices by the index map reproduces fe_assemble's K (FP64)."""
    torch = torch_cuda
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (3, 3, 2), ncomp=3, perturb=0.2, seed=35)
    h = make_handle(fg, O, prob)
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=1.0, p1=0.3, body=(0.0, 0.0, -1.0), precision=fg.PREC_FP64)
    n, nbf = prob.n_cells, prob.ndofs_per_cell(0)
    ke = torch.zeros((n, nbf, nbf), dtype=torch.float64, device="cuda")
    fe = torch.zeros((n, nbf), dtype=torch.float64, device="cuda")
    h.assemble_elements(ke, fe, **kw)
    nz = np.zeros(prob.nnz)
    f = np.zeros(prob.ndofs)
    h.assemble(nz, f, **kw)
    ke, fe = ke.cpu().numpy(), fe.cpu().numpy()
    nz2 = np.zeros(prob.nnz)
    f2 = np.zeros(prob.ndofs)
    for c in range(n):
        pos = h.index_map(c + 1, nbf)
        np.add.at(nz2, pos.ravel(order="F") - 1, ke[c].ravel(order="F"))
        np.add.at(f2, prob.celldofs(c) - 1, fe[c])
    assert np.allclose(nz2, nz, rtol=1e-12, atol=1e-12 * np.abs(nz).max())
    assert np.allclose(f2, f, rtol=1e-12, atol=1e-15)


def test_elements_detj_error(built, oracle, torch_cuda):
    torch = torch_cuda
    fg, O = built, oracle
    nodes, cells = O.generate_grid(O.QUADRILATERAL, (3, 3))
    cells[4] = cells[4][[1, 0, 3, 2]]
    prob = O.Problem.single(O.QUADRILATERAL, nodes, cells).close().allocate_matrix()
    h = make_handle(fg, O, prob)
    ke = torch.zeros((9, 4, 4), dtype=torch.float32, device="cuda")
    fe = torch.zeros((9, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(fg.FEError) as ei:
        h.assemble_elements(ke, fe, physics=fg.HEAT, p0=1.0, p1=1.0)
    assert ei.value.name == "DETJ" and ei.value.cell == 5


def test_elements_without_k_or_f(built, oracle, torch_cuda):
    torch = torch_cuda
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (2, 2, 1), ncomp=3, perturb=0.2, seed=36)
    h = make_handle(fg, O, prob)
    n, nbf = prob.n_cells, prob.ndofs_per_cell(0)
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=1.0, p1=0.3, body=(0.0, 0.0, -1.0))
    ke = torch.zeros((n, nbf, nbf), dtype=torch.float32, device="cuda")
    fe = torch.zeros((n, nbf), dtype=torch.float32, device="cuda")
    h.assemble_elements(ke, fe, **kw)
    ke2 = torch.full_like(ke, 7.0)
    h.assemble_elements(ke2, None, fe_stride=(0, 0), **kw)
    assert torch.equal(ke2, ke)
    fe2 = torch.full_like(fe, 7.0)
    h.assemble_elements(None, fe2, ke_stride=(0, 0, 0), **kw)
    assert torch.equal(fe2, fe)
