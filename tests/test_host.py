"""The library's own host-side set-up (numpy grids, native dof distribution and pattern,
reference tables) against the oracle's restatement of Ferrite: bit-exact dofs and patterns."""
import importlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def host(fg):
    fg.build()
    return importlib.import_module("ferrite_gb300.host")


CASES = [(2, (7, 5), 1, 1), (2, (4, 3), 2, 1), (1, (5, 4), 1, 1), (4, (5, 4, 3), 1, 3), (4, (3, 3, 2), 2, 3),
         (3, (3, 2, 2), 1, 3), (5, (3, 3, 2), 1, 3), (4, (4, 4, 4), 1, 1),
         (1, (4, 3), 1, 2), (2, (3, 3), 2, 2), (5, (3, 2, 2), 1, 1)]


@pytest.mark.parametrize("ct,nel,ip,nc", CASES)
def test_grid_dofs_pattern_match_oracle(host, oracle, ct, nel, ip, nc):
    O = oracle
    d = len(nel)
    left, right = np.zeros(d), np.arange(1, d + 1, dtype=float)
    g = host.generate_grid(ct, nel, left, right)
    nodes, cells = O.generate_grid(ct, nel, left, right)
    assert np.array_equal(g.nodes, nodes)
    assert np.array_equal(g.cells, cells)
    dh = host.DofHandler.from_grid(g, ip, nc).close()
    prob = O.Problem.single(ct, nodes, cells, ip, nc, 2).close().allocate_matrix()
    assert dh.ndofs == prob.ndofs
    assert np.array_equal(dh.cell_dofs, prob.cell_dofs)
    assert np.array_equal(dh.cell_dofs_offset, prob.cell_dofs_offset)
    colptr, rowval = dh.allocate_matrix()
    assert np.array_equal(colptr, prob.colptr) and np.array_equal(rowval, prob.rowval)


def test_mixed_subdomains_match_oracle(host, oracle):
    from test_gpu_parity import mixed_problem
    prob = mixed_problem(oracle)
    dh = host.DofHandler(prob.nodes, prob.n_cells)
    for sd in prob.subdomains:
        ct = int(prob.cell_types[sd.cellset[0] - 1])
        ng = oracle.nbase(ct, 1)
        cn = prob.cell_nodes[prob.cell_nodes_offset[sd.cellset - 1][:, None] + np.arange(ng)[None, :]]
        dh.add(ct, cn, sd.cellset, 1, 3)
    dh.close()
    assert np.array_equal(dh.cell_dofs, prob.cell_dofs)
    colptr, rowval = dh.allocate_matrix()
    assert np.array_equal(colptr, prob.colptr) and np.array_equal(rowval, prob.rowval)


@pytest.mark.parametrize("ct,orders", [(2, [1, 2, 3]), (4, [1, 2, 3]), (3, [1, 2]), (5, [1, 2]), (1, [1, 2])])
def test_tables_match_oracle(host, oracle, ct, orders):
    for qo in orders:
        w, p = host.quadrature_rule(ct, qo)
        w2, p2 = oracle.quadrature(ct, qo)
        assert np.allclose(w, w2, rtol=0, atol=2e-16) and np.allclose(p, p2, rtol=0, atol=2e-16)
        ips = [1, 2] if ct in (2, 4) else [1]
        for ip in ips:
            N, dN = host.shape_tables(ct, ip, p2)
            N2, dN2 = oracle.shape_tables(ct, ip, p2)
            assert np.allclose(N, N2, atol=1e-15) and np.allclose(dN, dN2, atol=1e-15)


@pytest.mark.parametrize("ct,ip,qo", [(2, 1, 2), (2, 2, 3), (1, 1, 2), (4, 1, 2), (4, 2, 3), (3, 1, 1), (3, 1, 2)])
def test_facet_values_tables(fg, oracle, ct, ip, qo):
    """The product's FacetValues tables (host.facet_values) equal the oracle-side ones built
    from the reference's facet rules and shape functions."""
    from helpers import facet_tables
    host = __import__("ferrite_gb300.host", fromlist=["host"])
    a = host.facet_values(ct, ip, qo)
    b = facet_tables(oracle, ct, ip, qo)
    assert a[0] == b[0] and a[1] == b[1]
    for x, y in zip(a[2:], b[2:]):
        assert x.shape == y.shape and np.allclose(x, y, rtol=1e-14, atol=1e-15)


def test_buffer_checks(fg, oracle):
    """The Python layer checks element types and lengths before passing bare pointers to the
    C ABI (a float32 buffer where float64 is read, or a short one, would be accessed past its
    end)."""
    import numpy as np
    from helpers import subdomain_specs
    O = oracle
    for ct, nel, ip, nc, want in [(O.HEXAHEDRON, (2, 2, 1), 1, 3, 24), (O.HEXAHEDRON, (1, 1, 1), 2, 3, 81),
                                  (O.QUADRILATERAL, (2, 2), 1, 1, 4), (O.TETRAHEDRON, (1, 1, 1), 1, 3, 12)]:
        prob = O.box_problem(ct, nel, ip_order=ip, ncomp=nc, qr_order=3 if ip == 2 else 2)
        assert fg._max_dofs_per_cell(subdomain_specs(fg, O, prob)) == want
    fg._check(np.zeros(10), "x", "float64", 10)
    with pytest.raises(TypeError):
        fg._check(np.zeros(10, np.float32), "x", "float64", 10)
    with pytest.raises(ValueError):
        fg._check(np.zeros(9), "x", "float64", 10)
    with pytest.raises(TypeError):
        fg._check([0.0] * 10, "x", "float64", 10)
    # extents: row-major [n, m, m], the how-to's column-major, and a per-cell vector
    n, m = 5, 24
    assert fg._extent(n, m, (m * m, m, 1)) == n * m * m
    assert fg._extent(n, m, (1, n, n * m)) == n * m * m
    assert fg._extent(n, m, (1, n)) == n * m
    with pytest.raises(ValueError):
        fg._extent(n, m, (-1, n, n * m))
    torch = pytest.importorskip("torch")
    fg._check(torch.zeros(n * m * m, dtype=torch.float32), "ke", fg._elem_dtype(fg.PREC_MIXED), n * m * m)
    with pytest.raises(TypeError):
        fg._check(torch.zeros(n * m * m, dtype=torch.float32), "ke", fg._elem_dtype(fg.PREC_FP64), n * m * m)


@pytest.mark.parametrize("qo", [1, 2])
def test_wedge_facet_values_integrate_loads(host, oracle, qo):
    """Wedge (RefPrism) facet tables: triangle facets (1, 5) with the triangle rule, quadrilateral
    facets (2-4) with a quarter of the Gauss weights, padded to one length. Through the oracle's
    facet loads they integrate pressure and traction exactly over the box's x, y and z faces,
    so every facet's normal, orientation and dGamma scale is Ferrite's."""
    import numpy as np
    from helpers import boundary_facets
    O = oracle
    tables = host.facet_values(host.WEDGE, 1, qo)
    nf, nq, W, N, dM = tables
    assert nf == 5 and np.allclose(W.sum(axis=1), [0.5, 1.0, 1.0, 1.0, 0.5])
    p = O.box_problem(O.WEDGE, (3, 2, 2), [0.0, 0.0, 0.0], [2.0, 1.0, 3.0], ip_order=1, ncomp=3, qr_order=2,
                      perturb=0.2, seed=9)
    t = np.array([0.5, -0.25, 1.0])
    seen = set()
    for on_face, normal, area, kinds in (
            (lambda X: abs(X[0]) < 1e-12, (-1, 0, 0), 3.0, {2, 3, 4}),
            (lambda X: abs(X[0] - 2.0) < 1e-12, (1, 0, 0), 3.0, {2, 3, 4}),
            (lambda X: abs(X[1]) < 1e-12, (0, -1, 0), 6.0, {2, 3, 4}),
            (lambda X: abs(X[1] - 1.0) < 1e-12, (0, 1, 0), 6.0, {2, 3, 4}),
            (lambda X: abs(X[2]) < 1e-12, (0, 0, -1), 2.0, {1}),
            (lambda X: abs(X[2] - 3.0) < 1e-12, (0, 0, 1), 2.0, {5})):
        cells, facets = boundary_facets(p, O.WEDGE, on_face)
        assert len(cells) > 0 and set(facets.tolist()) <= kinds
        seen |= set(facets.tolist())
        f = p.facet_load(cells, facets, tables, pressure=1.5, traction=tuple(t))
        sums = np.array([f[a::3].sum() for a in range(3)])
        assert np.allclose(sums, 1.5 * area * np.array(normal) + t * area, rtol=1e-13, atol=1e-13), (normal, sums)
    assert seen == {1, 2, 3, 4, 5}
