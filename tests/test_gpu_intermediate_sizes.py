"""GPU parity at intermediate sizes, between the small unit cases and the benchmark sizes: the
same generators and physics as the benchmark configurations, with enough cells that every
kernel form runs many tiles on every SM, checked against the oracle's FP64 assembly.

  * 32^3 Q1 hexahedra, linear elasticity on the perturbed unit cube (the 128^3 workload's
    generator), compensated and plain FP32 sums;
  * 12^3 Q2 hexahedra, linear elasticity with a lognormal per-cell modulus, tensor-core and
    CUDA-core element matrices;
  * a 30x10x10 hexahedron / tetrahedron / wedge box (1,000 + 6,000 + 2,000 cells), Neo-Hooke,
    fused and two-phase, with a moderate displacement and with one that inverts some elements;
  * the SIMP adjoint on a (24,12,12) cantilever slab.

Tolerances are those of the unit cases: relative Frobenius error of nzval and f <= 1e-6 for
the mixed forms (2e-6 for Neo-Hooke), max error relative to the largest entry for the adjoint.
"""
import numpy as np
import pytest

from helpers import make_handle, rel_fro
from test_gpu_adjoint import run_case
from test_gpu_parity import mixed_problem

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


def _run(fg, O, prob, element_args, oracle_args, variants, tol):
    nz_ref, f_ref = prob.assemble(**oracle_args)
    h = make_handle(fg, O, prob)
    for kw in variants:
        nz = np.full(prob.nnz, np.nan)
        f = np.full(prob.ndofs, np.nan)
        h.assemble(nz, f, precision=0, **element_args, **kw)
        assert rel_fro(nz, nz_ref) <= tol, (kw, rel_fro(nz, nz_ref))
        assert rel_fro(f, f_ref) <= tol, (kw, rel_fro(f, f_ref))


def test_q1_elasticity_32cubed(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (32, 32, 32), [0, 0, 0], [1, 1, 1], ip_order=1, ncomp=3, qr_order=2,
                         perturb=0.2, seed=20261203)
    E, nu, b = 200e3, 0.3, (0.0, 0.0, -1.0)
    _run(fg, O, prob, dict(physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, body=b),
         dict(physics=O.LINEAR_ELASTIC, p0=E, p1=nu, body=b),
         [dict(), dict(compensated=False), dict(form="two_phase_cuda_cores")], 1e-6)


def test_q2_elasticity_12cubed(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (12, 12, 12), [0, 0, 0], [1, 1, 1], ip_order=2, ncomp=3, qr_order=3,
                         perturb=0.2, seed=31)
    scale = np.random.default_rng(32).lognormal(0.0, 0.5, prob.n_cells)
    E, nu = 200e3, 0.3
    _run(fg, O, prob, dict(physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, cell_scale=scale),
         dict(physics=O.LINEAR_ELASTIC, p0=E, p1=nu, cell_scale=scale),
         [dict(), dict(form="two_phase_cuda_cores"), dict(form="fused")], 1e-6)


def test_neo_hooke_mixed_30x10x10(built, oracle):
    fg, O = built, oracle
    prob = mixed_problem(O, nel=(30, 10, 10), seed=41)
    # displacement amplitude scaled to the cell size (h = 1/15 along x) as in the unit cases:
    # det F stays within [0.67, 1.47], no element near inversion
    u = 0.01 * np.random.default_rng(42).uniform(-1, 1, prob.ndofs)
    _run(fg, O, prob, dict(physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, u=u, body=(0.0, -0.5, 0.0)),
         dict(physics=O.NEO_HOOKE, p0=1.0, p1=10.0, u=u, body=(0.0, -0.5, 0.0)),
         [dict(), dict(form="fused"), dict(form="two_phase")], 2e-6)


def test_neo_hooke_near_singular_points(built, oracle):
    """A displacement of amplitude 0.05 on the same mix (h = 1/15 along x) drives det F down to
    -0.64 at about 1.6 % of the hexahedron points (inverted elements; Ferrite's J = sqrt(det C)
    maps them to |det F|). The FP32 point math flags those points and recomputes them in FP64,
    so the mixed forms still match the FP64 oracle."""
    fg, O = built, oracle
    prob = mixed_problem(O, nel=(30, 10, 10), seed=41)
    u = 0.05 * np.random.default_rng(42).uniform(-1, 1, prob.ndofs)
    nz_ref, f_ref = prob.assemble(physics=O.NEO_HOOKE, p0=1.0, p1=10.0, u=u, body=(0.0, -0.5, 0.0))
    assert np.isfinite(nz_ref).all() and np.isfinite(f_ref).all()
    h = make_handle(fg, O, prob)
    for kw in (dict(), dict(form="fused"), dict(form="two_phase")):
        nz = np.full(prob.nnz, np.nan)
        f = np.full(prob.ndofs, np.nan)
        h.assemble(nz, f, precision=0, physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, u=u, body=(0.0, -0.5, 0.0), **kw)
        assert np.isfinite(nz).all() and np.isfinite(f).all(), kw
        assert rel_fro(nz, nz_ref) <= 2e-6, (kw, rel_fro(nz, nz_ref))
        assert rel_fro(f, f_ref) <= 2e-6, (kw, rel_fro(f, f_ref))
        assert h.info()["flagged_cells"] > 0, kw


def test_adjoint_cantilever_24x12x12(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (24, 12, 12), [0, 0, 0], [2, 1, 1], ncomp=3, perturb=0.2, seed=43)
    run_case(fg, O, prob, fg.LINEAR_ELASTIC, O.LINEAR_ELASTIC, 1.0, 0.3, (0.0, 0.0, -1.0), 44)
