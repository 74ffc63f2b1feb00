"""The oracle's adjoint (vector-Jacobian products of lam^T (K u - f)) against central finite
differences of the oracle's own assembly, h = 1e-6 (the FD step of the adjoint benchmark).

These pin the adjoint formulas that the GPU adjoint kernel is then compared with: d/d(rho) of
a SIMP modulus E = rho^3 E0 per cell, and d/dX of every node coordinate."""
import numpy as np
import pytest

import oracle as orc

H = 1e-6


def phi(prob, physics, p0, p1, body, scale, u, lam):
    nz, f = prob.assemble(physics, p0, p1, body=body, cell_scale=scale)
    return lam @ (prob.to_scipy(nz) @ u - f)


def fd_check(prob, physics, p0, p1, body, rho, u, lam, tol):
    scale, dscale = rho ** 3, 3 * rho ** 2
    d_cell, d_X = prob.adjoint(physics, p0, p1, u, lam, body=body, cell_scale=scale, dscale=dscale)
    # cells
    fd_cell = np.zeros_like(d_cell)
    for c in range(prob.n_cells):
        rp, rm = rho.copy(), rho.copy()
        rp[c] += H
        rm[c] -= H
        fd_cell[c] = (phi(prob, physics, p0, p1, body, rp ** 3, u, lam) - phi(prob, physics, p0, p1, body, rm ** 3, u, lam)) / (2 * H)
    # node coordinates (perturbed in place; the dof numbering and pattern do not change)
    fd_X = np.zeros_like(d_X)
    for n in range(prob.nodes.shape[0]):
        for a in range(prob.dim):
            x0 = prob.nodes[n, a]
            prob.nodes[n, a] = x0 + H
            pp = phi(prob, physics, p0, p1, body, scale, u, lam)
            prob.nodes[n, a] = x0 - H
            pm = phi(prob, physics, p0, p1, body, scale, u, lam)
            prob.nodes[n, a] = x0
            fd_X[n, a] = (pp - pm) / (2 * H)
    assert np.max(np.abs(d_cell - fd_cell)) <= tol * np.max(np.abs(fd_cell))
    assert np.max(np.abs(d_X - fd_X)) <= tol * np.max(np.abs(fd_X))
    return d_cell, d_X


def test_adjoint_elastic_hex_fd():
    prob = orc.box_problem(orc.HEXAHEDRON, (3, 2, 2), (0, 0, 0), (2, 1, 1), ncomp=3, perturb=0.2, seed=7)
    rng = np.random.default_rng(11)
    rho = rng.uniform(0.01, 1.0, prob.n_cells)
    u = rng.normal(0, 1e-3, prob.ndofs)
    lam = rng.normal(0, 1e-3, prob.ndofs)
    fd_check(prob, orc.LINEAR_ELASTIC, 1.0, 0.3, (0.0, 0.0, -1.0), rho, u, lam, 2e-6)


def test_adjoint_elastic_tet_fd():
    prob = orc.box_problem(orc.TETRAHEDRON, (2, 1, 1), ncomp=3, perturb=0.15, seed=3)
    rng = np.random.default_rng(5)
    rho = rng.uniform(0.1, 1.0, prob.n_cells)
    u = rng.normal(0, 1.0, prob.ndofs)
    lam = rng.normal(0, 1.0, prob.ndofs)
    fd_check(prob, orc.LINEAR_ELASTIC, 2.0, 0.25, (0.5, 0.0, -1.0), rho, u, lam, 2e-6)


def test_adjoint_heat_quad_fd():
    prob = orc.box_problem(orc.QUADRILATERAL, (3, 3), ncomp=1, perturb=0.2, seed=2)
    rng = np.random.default_rng(9)
    rho = rng.uniform(0.2, 1.0, prob.n_cells)
    u = rng.normal(0, 1.0, prob.ndofs)
    lam = rng.normal(0, 1.0, prob.ndofs)
    fd_check(prob, orc.HEAT, 1.0, 1.0, None, rho, u, lam, 2e-6)


def test_adjoint_linear_in_lambda_and_zero_for_rigid_translation():
    """d_cell is bilinear: zero lam gives zero; a rigid translation u leaves K u = 0, so only the
    load term remains in d_X and d_cell vanishes."""
    prob = orc.box_problem(orc.HEXAHEDRON, (2, 2, 2), ncomp=3, perturb=0.2, seed=1)
    n = prob.ndofs
    d_cell, d_X = prob.adjoint(orc.LINEAR_ELASTIC, 1.0, 0.3, np.ones(n), np.zeros(n))
    assert not d_cell.any() and not d_X.any()
    u = np.tile([1.0, -2.0, 0.5], n // 3)
    lam = np.random.default_rng(0).normal(size=n)
    d_cell, _ = prob.adjoint(orc.LINEAR_ELASTIC, 1.0, 0.3, u, lam)
    assert np.max(np.abs(d_cell)) < 1e-12
