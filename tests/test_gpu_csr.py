"""CSR output (SparseMatrixCSR{1} of ext/FerriteSparseMatrixCSR.jl): the engine fills a CSR
matrix given as (rowptr, colval) in place of (colptr, rowval). Checked against the oracle's CSR
assembler (or_assemble_csr, the extension's _assemble_inner!) at the engine's tolerances
(mixed 1e-6, FP64 1e-12 relative Frobenius), for heat, elasticity and Neo-Hooke on mixed cells."""
import numpy as np
import pytest

from helpers import rel_fro, subdomain_specs
from test_gpu_parity import mixed_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(fg):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    fg.build()
    return fg


@pytest.mark.parametrize("case", ["quad_heat", "hex_elastic", "hex27_elastic", "mixed_neo"])
def test_csr_against_oracle(built, oracle, case):
    fg, O = built, oracle
    if case == "quad_heat":
        prob = O.box_problem(O.QUADRILATERAL, (9, 7), perturb=0.2, seed=41)
        kf, ko = dict(physics=fg.HEAT, p0=1.0, p1=1.0), dict(physics=O.HEAT, p0=1.0, p1=1.0)
    elif case == "hex_elastic":
        prob = O.box_problem(O.HEXAHEDRON, (5, 4, 3), ncomp=3, perturb=0.2, seed=42)
        kf = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0))
        ko = dict(physics=O.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0))
    elif case == "hex27_elastic":
        prob = O.box_problem(O.HEXAHEDRON, (2, 2, 2), ip_order=2, ncomp=3, qr_order=3, perturb=0.2, seed=43)
        kf = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 1.0, 0.0))
        ko = dict(physics=O.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 1.0, 0.0))
    else:
        prob = mixed_problem(O)
        u = 0.002 * np.random.default_rng(3).uniform(-1, 1, prob.ndofs)
        kf, ko = dict(physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, u=u), dict(physics=O.NEO_HOOKE, p0=1.0, p1=10.0, u=u)
    rowptr, colval = prob.csr_pattern()
    h = fg.Handle(prob.nodes, subdomain_specs(fg, O, prob), prob.cell_dofs, prob.cell_dofs_offset, prob.ndofs,
                  rowptr, colval, prob.n_cells)
    nz_ref, f_ref = prob.assemble_csr(rowptr, colval, **ko)
    for prec, tol in ((fg.PREC_FP64, 1e-12), (fg.PREC_MIXED, 1e-6)):
        nz = np.full(len(colval), np.nan)
        f = np.full(prob.ndofs, np.nan)
        h.assemble(nz, f, precision=prec, **kf)
        assert rel_fro(nz, nz_ref) <= tol, (case, prec, rel_fro(nz, nz_ref))
        assert rel_fro(f, f_ref) <= tol, (case, prec)
    h.close()
