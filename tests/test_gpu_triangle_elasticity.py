"""Plane linear elasticity on P1 triangles, the element of the linear-elasticity tutorial
(docs/src/literate-tutorials/linear_elasticity.jl: Lagrange{RefTriangle, 1}^2 with
QuadratureRule{RefTriangle}(1)), and with the 3-point rule: device assembly against the FP64
oracle (mixed 1e-6, FP64 1e-12 relative Frobenius), including a per-cell modulus."""
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
