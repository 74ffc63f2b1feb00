"""Element kernels instantiated from the verified template for three more cell / physics
combinations, each device assembly against the FP64 oracle (mixed 1e-6, FP64 1e-12 relative
Frobenius):
- plane linear elasticity on P1 triangles, the element of the linear-elasticity tutorial
  (docs/src/literate-tutorials/linear_elasticity.jl: Lagrange{RefTriangle, 1}^2 with
  QuadratureRule{RefTriangle}(1)), and with the 3-point rule, with a per-cell modulus;
- heat on P1 wedges with 1 and 5 points (the RefPrism polyquad rules);
- plane linear elasticity on Q2 quadrilaterals with 3x3 Gauss."""
import numpy as np
import pytest

from helpers import make_handle, rel_fro

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(fg):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    fg.build()
    return fg


@pytest.mark.parametrize("qo", [1, 2])
def test_triangle_elasticity_against_oracle(built, oracle, qo):
    fg, O = built, oracle
    prob = O.box_problem(O.TRIANGLE, (12, 9), [0.0, 0.0], [2.0, 1.0], ip_order=1, ncomp=2, qr_order=qo,
                         perturb=0.15, seed=60 + qo)
    scale = np.random.default_rng(qo).lognormal(0.0, 0.5, prob.n_cells)
    E, nu, b = 200e3, 0.3, (0.0, -1.0, 0.0)
    h = make_handle(fg, O, prob)
    nz_ref, f_ref = prob.assemble(O.LINEAR_ELASTIC, E, nu, body=list(b), cell_scale=scale)
    for prec, tol in ((fg.PREC_FP64, 1e-12), (fg.PREC_MIXED, 1e-6)):
        nz = np.full(prob.nnz, np.nan)
        f = np.full(prob.ndofs, np.nan)
        h.assemble(nz, f, physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, body=b, cell_scale=scale, precision=prec)
        assert rel_fro(nz, nz_ref) <= tol, (qo, prec, rel_fro(nz, nz_ref))
        assert rel_fro(f, f_ref) <= tol, (qo, prec, rel_fro(f, f_ref))
    h.close()


@pytest.mark.parametrize("qo", [1, 2])
def test_wedge_heat_against_oracle(built, oracle, qo):
    fg, O = built, oracle
    prob = O.box_problem(O.WEDGE, (4, 3, 3), [0.0, 0.0, 0.0], [2.0, 1.0, 1.0], ip_order=1, ncomp=1, qr_order=qo,
                         perturb=0.15, seed=64 + qo)
    h = make_handle(fg, O, prob)
    nz_ref, f_ref = prob.assemble(O.HEAT, 1.0, 1.0)
    for prec, tol in ((fg.PREC_FP64, 1e-12), (fg.PREC_MIXED, 1e-6)):
        nz = np.full(prob.nnz, np.nan)
        f = np.full(prob.ndofs, np.nan)
        h.assemble(nz, f, physics=fg.HEAT, p0=1.0, p1=1.0, precision=prec)
        assert rel_fro(nz, nz_ref) <= tol, (qo, prec, rel_fro(nz, nz_ref))
        assert rel_fro(f, f_ref) <= tol, (qo, prec, rel_fro(f, f_ref))
    h.close()


def test_quad9_elasticity_against_oracle(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.QUADRILATERAL, (6, 5), [0.0, 0.0], [2.0, 1.0], ip_order=2, ncomp=2, qr_order=3,
                         perturb=0.15, seed=67)
    E, nu, b = 200e3, 0.3, (0.5, -1.0, 0.0)
    h = make_handle(fg, O, prob)
    nz_ref, f_ref = prob.assemble(O.LINEAR_ELASTIC, E, nu, body=list(b))
    for prec, tol in ((fg.PREC_FP64, 1e-12), (fg.PREC_MIXED, 1e-6)):
        nz = np.full(prob.nnz, np.nan)
        f = np.full(prob.ndofs, np.nan)
        h.assemble(nz, f, physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, body=b, precision=prec)
        assert rel_fro(nz, nz_ref) <= tol, (prec, rel_fro(nz, nz_ref))
        assert rel_fro(f, f_ref) <= tol, (prec, rel_fro(f, f_ref))
    h.close()
