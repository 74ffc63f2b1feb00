"""The CPU oracle pinned against Ferrite.jl's own known answers and test identities.

These run without a GPU. They check the oracle (a restatement of the reference's assembly
path, oracle/ferrite_oracle.cpp) before anything is compared against it:
  * the two golden values the reference's tutorials assert (tests/golden/known_answers.json);
  * quadrature exactness (test/test_quadrules.jl:22-38);
  * CellValues identities: volume, linear-field reproduction (test/test_cellvalues.jl:51-161);
  * Q2 dof sharing consistency (test/test_dofs.jl:1156-1235, restated as a nodal
    interpolation check);
  * assembler semantics: zero skipping, pattern-miss errors (test/test_assemble.jl:4-214);
  * colored threaded determinism (docs/src/literate-howto/threaded_assembly.jl:397-410).
"""
import itertools
import json
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spla

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def node_to_dofs(prob, ncomp):
    """Map node id (0-based) -> its ncomp dofs (0-based), for vertex-only fields."""
    x = prob.nodes
    out = np.full((len(x), ncomp), -1, np.int64)
    for c in range(prob.n_cells):
        nodes = prob.cells_of(c) - 1
        d = prob.celldofs(c) - 1
        out[nodes] = d[: len(nodes) * ncomp].reshape(len(nodes), ncomp)
    return out


def test_heat_equation_golden(oracle):
    O = oracle
    p = O.box_problem(O.QUADRILATERAL, (20, 20), qr_order=2)
    nz, f = p.assemble(O.HEAT, 1.0, 1.0)
    K = p.to_scipy(nz)
    x = p.nodes
    n2d = node_to_dofs(p, 1)[:, 0]
    bnd = np.where((np.abs(np.abs(x[:, 0]) - 1) < 1e-12) | (np.abs(np.abs(x[:, 1]) - 1) < 1e-12))[0]
    free = np.setdiff1d(np.arange(p.ndofs), n2d[bnd])
    u = np.zeros(p.ndofs)
    u[free] = spla.spsolve(K[free][:, free].tocsc(), f[free])
    g = GOLDEN["heat_equation_norm_u"]
    assert np.linalg.norm(u) == pytest.approx(g["value"], rel=g["rtol"])


def test_heat_equation_golden_with_apply(oracle):
    """The tutorial's own sequence: assemble, apply!(K, f, ch), u = K \\ f (heat_equation.jl:
    215-234), with the oracle's apply! (ConstraintHandler.jl:711-744) on the full system."""
    O = oracle
    p = O.box_problem(O.QUADRILATERAL, (20, 20), qr_order=2)
    nz, f = p.assemble(O.HEAT, 1.0, 1.0)
    x = p.nodes
    n2d = node_to_dofs(p, 1)[:, 0]
    bnd = np.where((np.abs(np.abs(x[:, 0]) - 1) < 1e-12) | (np.abs(np.abs(x[:, 1]) - 1) < 1e-12))[0]
    pd = np.sort(n2d[bnd]) + 1
    p.apply(nz, f, pd, np.zeros(len(pd)))
    K = p.to_scipy(nz)
    # constrained rows and columns are zero apart from the mean diagonal
    m = K.diagonal()[pd[0] - 1]
    assert np.all(K.diagonal()[pd - 1] == m) and m > 0
    assert np.all(f[pd - 1] == 0)
    u = spla.spsolve(K.tocsc(), f)
    g = GOLDEN["heat_equation_norm_u"]
    assert np.linalg.norm(u) == pytest.approx(g["value"], rel=g["rtol"])


def test_apply_inhomogeneous_semantics(oracle):
    """apply! with g != 0 leaves K u = f solved by u = g on the constrained dofs, and the free
    rows see f - K g (the condensed system); apply_zero! sets f[d] = 0."""
    O = oracle
    p = O.box_problem(O.QUADRILATERAL, (6, 5), qr_order=2, perturb=0.2, seed=2)
    nz0, f0 = p.assemble(O.HEAT, 1.0, 1.0)
    rng = np.random.default_rng(3)
    pd = np.sort(rng.choice(p.ndofs, 9, replace=False)) + 1
    g = rng.normal(size=len(pd))
    nz, f = nz0.copy(), f0.copy()
    p.apply(nz, f, pd, g)
    u = spla.spsolve(p.to_scipy(nz).tocsc(), f)
    assert np.allclose(u[pd - 1], g, rtol=1e-12, atol=1e-12)
    free = np.setdiff1d(np.arange(p.ndofs), pd - 1)
    K0 = p.to_scipy(nz0).tocsr()
    r = K0 @ u - f0
    assert np.abs(r[free]).max() < 1e-10 * np.abs(f0).max()
    nz, f = nz0.copy(), f0.copy()
    p.apply(nz, f, pd, g, applyzero=True)
    assert np.all(f[pd - 1] == 0) and np.array_equal(f[free], f0[free])


def test_hyperelasticity_golden(oracle):
    O = oracle
    N, L = 10, 1.0
    p = O.box_problem(O.TETRAHEDRON, (N, N, N), [0, 0, 0], [L, L, L], ip_order=1, ncomp=3, qr_order=1)
    E, nu = 10.0, 0.3
    lam, mu = O.lame(E, nu)
    x = p.nodes
    n2d = node_to_dofs(p, 3)
    right = np.where(np.abs(x[:, 0] - L) < 1e-12)[0]
    left = np.where(np.abs(x[:, 0]) < 1e-12)[0]
    th, t = np.pi / 3, 0.5
    un = np.zeros(p.ndofs)
    for n in left:  # rotation(X, t), hyperelasticity.jl:352-362
        X, Y, Z = x[n]
        un[n2d[n]] = t * np.array([0.0, L / 2 - Y + (Y - L / 2) * np.cos(th) - (Z - L / 2) * np.sin(th),
                                   L / 2 - Z + (Y - L / 2) * np.sin(th) + (Z - L / 2) * np.cos(th)])
    cons = np.concatenate([n2d[right].ravel(), n2d[left].ravel()])
    # dead traction 0.1*n on top/bottom/front/back with a 1-point facet rule
    # (hyperelasticity.jl:262-275): each facet node receives -t * area / 3
    faces = [(0, 2, 1), (0, 1, 3), (1, 2, 3), (0, 3, 2)]
    gt = np.zeros(p.ndofs)
    for c in range(p.n_cells):
        cn = p.cells_of(c) - 1
        for fc in faces:
            nd = cn[list(fc)]
            P = x[nd]
            for ax, val, nrm in [(2, L, (0, 0, 1)), (2, 0, (0, 0, -1)), (1, 0, (0, -1, 0)), (1, L, (0, 1, 0))]:
                if np.all(np.abs(P[:, ax] - val) < 1e-12):
                    area = 0.5 * np.linalg.norm(np.cross(P[1] - P[0], P[2] - P[0]))
                    for n in nd:
                        gt[n2d[n]] -= 0.1 * np.array(nrm) * area / 3
    du = np.zeros(p.ndofs)
    free = np.setdiff1d(np.arange(p.ndofs), cons)
    for _ in range(30):
        u = un + du
        nz, g = p.assemble(O.NEO_HOOKE, mu, lam, body=[0, -0.5, 0], u=u)
        g = g + gt
        g[cons] = 0.0  # apply_zero!
        if np.linalg.norm(g) < 1e-8:
            break
        K = p.to_scipy(nz)
        d = np.zeros(p.ndofs)
        d[free] = spla.spsolve(K[free][:, free].tocsc(), g[free])
        du -= d
    gold = GOLDEN["hyperelasticity_norm_u"]
    assert np.linalg.norm(u) == pytest.approx(gold["value"], rel=gold["rtol"])


@pytest.mark.parametrize("ct,orders,vol", [(2, [1, 2, 3, 4], 4.0), (4, [1, 2, 3, 4], 8.0),
                                           (3, [1, 2, 3], 1 / 6), (5, [1, 2], 0.5), (1, [1, 2], 0.5)])
def test_quadrature_exactness(oracle, ct, orders, vol):
    """Gauss rules on (-1, 1)^d integrate degree 2n-1 per coordinate exactly; the simplex and
    prism rules of order n integrate every monomial of total degree <= n exactly, against the
    closed forms a! b! / (a+b+2)! (triangle), a! b! c! / (a+b+c+3)! (tetrahedron) and
    a! b! / (a+b+2)! / (c+1) (prism = triangle x (0, 1))."""
    from math import factorial
    O = oracle
    for order in orders:
        w, pts = O.quadrature(ct, order)
        assert w.sum() == pytest.approx(vol, abs=1e-14)
        d = pts.shape[1]
        if ct in (O.QUADRILATERAL, O.HEXAHEDRON):
            deg = 2 * order - 1
            for exps in itertools.product(range(deg + 1), repeat=d):
                exact = np.prod([(1 - (-1) ** (e + 1)) / (e + 1) for e in exps])
                num = np.sum(w * np.prod(pts ** np.array(exps), axis=1))
                assert num == pytest.approx(exact, abs=1e-13)
            continue
        for exps in itertools.product(range(order + 1), repeat=d):
            if sum(exps) > order:
                continue
            if ct == O.TRIANGLE:
                a, b = exps
                exact = factorial(a) * factorial(b) / factorial(a + b + 2)
            elif ct == O.TETRAHEDRON:
                a, b, c = exps
                exact = factorial(a) * factorial(b) * factorial(c) / factorial(a + b + c + 3)
            else:
                a, b, c = exps
                exact = factorial(a) * factorial(b) / factorial(a + b + 2) / (c + 1)
            num = np.sum(w * np.prod(pts ** np.array(exps), axis=1))
            assert num == pytest.approx(exact, abs=1e-14), (ct, order, exps)


@pytest.mark.parametrize("ct,nel,ip,nc", [(2, (3, 4), 1, 1), (4, (3, 2, 2), 1, 3), (4, (2, 2, 2), 2, 3),
                                          (3, (2, 2, 2), 1, 3), (5, (2, 2, 3), 1, 3)])
def test_volume_and_linear_field(oracle, ct, nel, ip, nc):
    """sum(detJdV) = |box| on a perturbed grid; the FE gradient of an interpolated linear
    field is exact (test_cellvalues.jl:51-161)."""
    O = oracle
    d = O.ref_dim(ct)
    left, right = -np.ones(d), np.ones(d) * 2
    qo = 2 if ct != O.TETRAHEDRON else 2
    p = O.box_problem(ct, nel, left, right, ip_order=ip, ncomp=nc, qr_order=qo, perturb=0.15, seed=3,
                      pattern=True)
    # volume via heat f with unit source: sum(f) = integral of sum_i N_i = |Omega|
    nz, f = p.assemble(O.HEAT if nc == 1 else O.LINEAR_ELASTIC, 1.0, 1.0 if nc == 1 else 0.3,
                       body=[1.0, 0.0, 0.0])
    total = f.sum()
    assert total == pytest.approx(np.prod(right - left), rel=1e-12)
    # linear field: K * u_lin for heat has zero row sums at interior nodes
    if nc == 1:
        K = p.to_scipy(nz)
        assert np.allclose(K @ np.ones(p.ndofs), 0.0, atol=1e-12)


def test_rigid_body_modes_elastic(oracle):
    """K annihilates rigid translations and infinitesimal rotations."""
    O = oracle
    p = O.box_problem(O.HEXAHEDRON, (3, 3, 2), ip_order=1, ncomp=3, perturb=0.2, seed=7)
    nz, _ = p.assemble(O.LINEAR_ELASTIC, 200e3, 0.3)
    K = p.to_scipy(nz)
    n2d = node_to_dofs(p, 3)
    x = p.nodes
    for mode in range(6):
        u = np.zeros(p.ndofs)
        for n in range(len(x)):
            if mode < 3:
                v = np.eye(3)[mode]
            else:
                w = np.eye(3)[mode - 3]
                v = np.cross(w, x[n])
            u[n2d[n]] = v
        assert np.abs(K @ u).max() < 1e-9 * np.abs(nz).max()


def test_elastic_equals_neo_hooke_tangent_at_rest(oracle):
    """At u = 0 the Neo-Hooke tangent equals the small-strain isotropic stiffness."""
    O = oracle
    p = O.box_problem(O.HEXAHEDRON, (2, 3, 2), ip_order=1, ncomp=3, perturb=0.2, seed=5)
    E, nu = 10.0, 0.3
    lam, mu = O.lame(E, nu)
    k1, _ = p.assemble(O.LINEAR_ELASTIC, E, nu)
    k2, _ = p.assemble(O.NEO_HOOKE, mu, lam, u=np.zeros(p.ndofs))
    assert np.allclose(k1, k2, rtol=1e-12, atol=1e-12 * np.abs(k1).max())


def test_neo_hooke_tangent_matches_fd(oracle):
    O = oracle
    p = O.box_problem(O.WEDGE, (2, 2, 1), ip_order=1, ncomp=3, qr_order=2, perturb=0.1, seed=1)
    rng = np.random.default_rng(0)
    u = 0.05 * rng.uniform(-1, 1, p.ndofs)
    nz, g = p.assemble(O.NEO_HOOKE, 1.0, 10.0, u=u)
    K = p.to_scipy(nz)
    v = rng.standard_normal(p.ndofs)
    h = 1e-6
    _, gp = p.assemble(O.NEO_HOOKE, 1.0, 10.0, u=u + h * v)
    _, gm = p.assemble(O.NEO_HOOKE, 1.0, 10.0, u=u - h * v)
    fd = (gp - gm) / (2 * h)
    assert np.allclose(K @ v, fd, rtol=1e-6, atol=1e-7 * np.abs(fd).max())


def test_q2_dof_sharing_consistent(oracle):
    """Every Q2 hexahedron dof gets one value from the nodal interpolation of a quadratic
    field, and each cell then reproduces the field exactly: shared edge/face dofs are
    shared, not duplicated (restates test_dofs.jl:1156-1235's consistency goal)."""
    O = oracle
    nel = (2, 3, 2)
    p = O.box_problem(O.HEXAHEDRON, nel, [0, 0, 0], [2, 3, 1], ip_order=2, ncomp=1, qr_order=3)
    nv, ne = np.prod(np.array(nel) + 1), 0
    nx, ny, nz = nel
    ne = nx * (ny + 1) * (nz + 1) + ny * (nx + 1) * (nz + 1) + nz * (nx + 1) * (ny + 1)
    nf = nx * ny * (nz + 1) + nx * nz * (ny + 1) + ny * nz * (nx + 1)
    assert p.ndofs == nv + ne + nf + nx * ny * nz
    lattice = np.array(list(itertools.product([-1.0, 0.0, 1.0], repeat=3)))[:, ::-1]
    N27, _ = O.shape_tables(O.HEXAHEDRON, 2, lattice)
    refc = lattice[np.argmax(N27, axis=0)]  # reference coordinate of each base function
    M8, _ = O.shape_tables(O.HEXAHEDRON, 1, refc)
    ufun = lambda X: 1 + X[..., 0] + 2 * X[..., 1] ** 2 + 3 * X[..., 0] * X[..., 2] - X[..., 1] * X[..., 2]
    val = np.full(p.ndofs, np.nan)
    for c in range(p.n_cells):
        xg = p.nodes[p.cells_of(c) - 1]
        pos = M8 @ xg
        d = p.celldofs(c) - 1
        v = ufun(pos)
        seen = ~np.isnan(val[d])
        assert np.allclose(val[d][seen], v[seen], atol=1e-12)
        val[d] = v
    w, qp = O.quadrature(O.HEXAHEDRON, 3)
    Nq, _ = O.shape_tables(O.HEXAHEDRON, 2, qp)
    Mq, _ = O.shape_tables(O.HEXAHEDRON, 1, qp)
    for c in range(p.n_cells):
        xg = p.nodes[p.cells_of(c) - 1]
        assert np.allclose(Nq @ val[p.celldofs(c) - 1], ufun(Mq @ xg), atol=1e-12)


def test_pattern_structure(oracle):
    O = oracle
    p = O.box_problem(O.HEXAHEDRON, (3, 2, 2), ip_order=1, ncomp=3)
    K = p.to_scipy(np.ones(p.nnz))
    assert (abs(K - K.T)).nnz == 0
    assert np.all(K.diagonal() == 1)
    for c in range(p.ndofs):
        rows = p.rowval[p.colptr[c] - 1:p.colptr[c + 1] - 1]
        assert np.all(np.diff(rows) > 0)
    # entries = dof pairs sharing a cell (plus diagonal)
    pairs = set()
    for c in range(p.n_cells):
        d = p.celldofs(c)
        pairs.update((int(a), int(b)) for a in d for b in d)
    assert len(pairs) == p.nnz


def test_zero_skipping_and_pattern_miss(oracle):
    """Exact zeros are never added (entries that only receive zeros stay +0.0), and a
    non-zero value without a pattern entry raises (assembler.jl:413-467)."""
    O = oracle
    p = O.box_problem(O.QUADRILATERAL, (3, 3), qr_order=2)
    nz, f = p.assemble(O.HEAT, 0.0, 1.0)  # k = 0: every Ke entry is exactly 0
    assert np.all(nz == 0) and not np.any(np.signbit(nz))
    # drop one off-diagonal entry from the pattern: assembling must now fail
    col = 5
    a, b = p.colptr[col] - 1, p.colptr[col + 1] - 1
    rows = p.rowval[a:b]
    drop = a + int(np.where(rows != col + 1)[0][0])
    rowval = np.delete(p.rowval, drop)
    colptr = p.colptr.copy()
    colptr[col + 1:] -= 1
    p.rowval, p.colptr = rowval, colptr
    with pytest.raises(O.OracleError) as ei:
        p.assemble(O.HEAT, 1.0, 1.0)
    assert ei.value.name == "PATTERN_MISSING" and ei.value.col == col + 1
    # zero contributions to the missing entry are allowed
    p.assemble(O.HEAT, 0.0, 1.0)


def test_detj_error(oracle):
    O = oracle
    nodes, cells = O.generate_grid(O.QUADRILATERAL, (2, 2))
    cells[3] = cells[3][[1, 0, 3, 2]]  # mirrored cell -> detJ < 0
    p = O.Problem.single(O.QUADRILATERAL, nodes, cells).close().allocate_matrix()
    with pytest.raises(O.OracleError) as ei:
        p.assemble(O.HEAT, 1.0, 1.0)
    assert ei.value.name == "DETJ" and ei.value.cell == 4 and ei.value.detJ < 0


def test_colored_threaded_determinism(oracle):
    """Colored threaded assembly is bitwise identical for 1, 2 and 4 threads and equal to
    the sequential loop up to summation order (threaded_assembly.jl:397-410)."""
    O = oracle
    p = O.box_problem(O.HEXAHEDRON, (10, 5, 5), [0, 0, 0], [10, 5, 5], ip_order=1, ncomp=3)
    runs = [p.assemble(O.LINEAR_ELASTIC, 200e9, 0.3, body=[0, 0, -1], nthreads=t) for t in (1, 2, 4)]
    for nz, f in runs[1:]:
        assert np.array_equal(nz, runs[0][0]) and np.array_equal(f, runs[0][1])
    nz0, f0 = p.assemble(O.LINEAR_ELASTIC, 200e9, 0.3, body=[0, 0, -1])
    assert np.allclose(runs[0][0], nz0, rtol=1e-13, atol=1e-13 * np.abs(nz0).max())
    assert np.allclose(runs[0][1], f0, rtol=1e-13)


@pytest.mark.parametrize("ct,nel", [("QUADRILATERAL", (5, 5)), ("TRIANGLE", (5, 5)), ("TETRAHEDRON", (5, 5, 5)),
                                    ("HEXAHEDRON", (5, 5, 5)), ("HEXAHEDRON", (12, 7, 3))])
def test_colorings_partition_without_conflicts(oracle, ct, nel):
    """Both colorings (WorkStream, Ferrite's default, and Greedy) cover every cell once and
    never give two cells sharing a node the same color (test_grid_dofhandler_vtk.jl:719-740);
    the threaded assembly prepared with either equals the serial loop up to summation order
    and is bitwise the same for 1 and 3 threads (threaded_assembly.jl:397-410)."""
    O = oracle
    ct = getattr(O, ct)
    ncomp = O.ref_dim(ct)
    p = O.box_problem(ct, nel, ip_order=1, ncomp=ncomp, perturb=0.1, seed=4)
    nz0, f0 = p.assemble(O.LINEAR_ELASTIC, 200e3, 0.3, body=[0.0, -1.0, 0.0][:ncomp] + [0.0] * (3 - ncomp))
    for alg in ("workstream", "greedy"):
        runs = []
        for nt in (1, 3):
            T = p.threaded(nt, alg)
            col = T.colors()
            assert col.min() == 1 and col.max() == T.n_colors
            for c in range(p.n_cells):  # no neighbour (shared node) has the cell's color
                nodes = set(p.cells_of(c).tolist())
                for d in range(c + 1, p.n_cells):
                    if col[d] == col[c]:
                        assert not nodes.intersection(p.cells_of(d).tolist()), (alg, c, d)
            runs.append(T.assemble(O.LINEAR_ELASTIC, 200e3, 0.3, body=[0.0, -1.0, 0.0][:ncomp] + [0.0] * (3 - ncomp)))
            T.close()
        assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
        assert np.allclose(runs[0][0], nz0, rtol=1e-13, atol=1e-13 * np.abs(nz0).max())
        assert np.allclose(runs[0][1], f0, rtol=1e-13, atol=1e-15)


def test_index_map_matches_binary_search(oracle):
    O = oracle
    p = O.box_problem(O.HEXAHEDRON, (2, 2, 2), ip_order=2, ncomp=3, qr_order=3)
    for c in (0, 5, 7):
        pos = p.index_map(c)
        d = p.celldofs(c)
        for J in range(len(d)):
            a, b = p.colptr[d[J] - 1] - 1, p.colptr[d[J]] - 1
            expect = a + np.searchsorted(p.rowval[a:b], d) + 1
            assert np.array_equal(pos[:, J], expect)


def test_facet_load_matches_tutorial_traction(oracle):
    """The oracle's facet loads (FacetValues.jl:129-155, 1-point facet rule on tetrahedra)
    reproduce the traction the hyperelasticity golden above is computed with (-tn n area/3 per
    facet node, hyperelasticity.jl:278-290)."""
    from helpers import boundary_facets, facet_tables
    O = oracle
    N, L = 4, 1.0
    p = O.box_problem(O.TETRAHEDRON, (N, N, N), [0, 0, 0], [L, L, L], ip_order=1, ncomp=3, qr_order=1)
    x = p.nodes
    n2d = node_to_dofs(p, 3)
    gt = np.zeros(p.ndofs)
    faces = [(0, 2, 1), (0, 1, 3), (1, 2, 3), (0, 3, 2)]
    sides = [(2, L, (0, 0, 1)), (2, 0, (0, 0, -1)), (1, 0, (0, -1, 0)), (1, L, (0, 1, 0))]
    for c in range(p.n_cells):
        cn = p.cells_of(c) - 1
        for fc in faces:
            nd = cn[list(fc)]
            P = x[nd]
            for ax, val, nrm in sides:
                if np.all(np.abs(P[:, ax] - val) < 1e-12):
                    area = 0.5 * np.linalg.norm(np.cross(P[1] - P[0], P[2] - P[0]))
                    for n in nd:
                        gt[n2d[n]] -= 0.1 * np.array(nrm) * area / 3
    sel = [boundary_facets(p, O.TETRAHEDRON, lambda X, ax=ax, val=val: abs(X[ax] - val) < 1e-12) for ax, val, _ in sides]
    cells = np.concatenate([c for c, _ in sel])
    facets = np.concatenate([f for _, f in sel])
    f = p.facet_load(cells, facets, facet_tables(O, O.TETRAHEDRON, 1, 1), pressure=-0.1)
    assert np.allclose(f, gt, rtol=1e-13, atol=1e-16)


@pytest.mark.parametrize("ct,ip", [(4, 1), (4, 2), (2, 1)])
def test_facet_load_integrates_pressure(oracle, ct, ip):
    """sum of f over a flat face's dofs = pressure * area * n + traction * area (partition of
    unity of the shape functions)."""
    from helpers import boundary_facets, facet_tables
    O = oracle
    d = 3 if ct == O.HEXAHEDRON else 2
    nel = (3, 4, 2) if d == 3 else (5, 4)
    p = O.box_problem(ct, nel, [0.0] * d, [2.0, 1.0, 3.0][:d], ip_order=ip, ncomp=d, qr_order=2, perturb=0.2, seed=9)
    cells, facets = boundary_facets(p, ct, lambda X: abs(X[0] - 2.0) < 1e-12)
    t = (0.5, -0.25, 1.0)[:d]
    f = p.facet_load(cells, facets, facet_tables(O, ct, ip, 2), pressure=1.5, traction=t)
    area = 3.0 if d == 3 else 1.0
    sums = [f[a::d].sum() for a in range(d)]
    expect = [1.5 * area + t[0] * area] + [t[a] * area for a in range(1, d)]
    assert np.allclose(sums, expect, rtol=1e-13, atol=1e-13)


def _element_stack(p, physics, p0, p1, dtype=np.float64):
    """Ke of every cell from the oracle's element routine, as [n_cells, n, n]."""
    return np.stack([p.element(c, physics, p0, p1)[0] for c in range(p.n_cells)]).astype(dtype)


@pytest.mark.parametrize("ct,nel,ip,nc", [("QUADRILATERAL", (5, 4), 1, 1), ("HEXAHEDRON", (3, 2, 2), 1, 3),
                                          ("TETRAHEDRON", (2, 2, 1), 1, 3), ("HEXAHEDRON", (2, 1, 1), 2, 3)])
def test_element_matvec_equals_assembled_product(oracle, ct, nel, ip, nc):
    """sum_c A_c^T Ke_c A_c u with FP64 element matrices equals K u of the assembled K."""
    O = oracle
    ctype = getattr(O, ct)
    phys, p0, p1 = (O.HEAT, 1.0, 1.0) if nc == 1 else (O.LINEAR_ELASTIC, 200e3, 0.3)
    p = O.box_problem(ctype, nel, ip_order=ip, ncomp=nc, qr_order=3 if ip == 2 else 2, perturb=0.15, seed=11)
    nz, _ = p.assemble(phys, p0, p1)
    ke = _element_stack(p, phys, p0, p1)
    u = np.random.default_rng(4).standard_normal(p.ndofs)
    y = p.element_matvec(ke, u)
    ref = p.to_scipy(nz) @ u
    assert np.abs(y - ref).max() <= 1e-13 * np.abs(ke).max() * np.abs(u).max() * 8
    # accumulation: y0 + product
    y0 = np.random.default_rng(5).standard_normal(p.ndofs)
    y2 = p.element_matvec(ke, u, y=y0.copy(), fillzero=False)
    assert np.abs(y2 - (y0 + y)).max() <= 1e-12 * np.abs(y).max()


def test_element_matvec_layouts_and_float_order(oracle):
    """Any strides address the same matrices (the how-to's column-major Kes included), and the
    float form is the fused multiply-add chain of its definition, checked against a numpy loop."""
    O = oracle
    p = O.box_problem(O.HEXAHEDRON, (2, 2, 1), ip_order=1, ncomp=3, perturb=0.1, seed=2)
    ke = _element_stack(p, O.LINEAR_ELASTIC, 200e3, 0.3, np.float32)
    u = np.random.default_rng(6).standard_normal(p.ndofs)
    y_row = p.element_matvec(ke, u)
    y_col = p.element_matvec(np.asfortranarray(ke), u)      # Kes[cell, i, j], column-major
    assert np.array_equal(y_row, y_col)
    # numpy restatement of the fma chain: the float32 product is exact in float64 and so is its
    # sum with a float32 addend of nearby exponent, then one rounding to float32 (a double
    # rounding could only differ for far-apart exponents, which these seeded values do not have)
    y = np.zeros(p.ndofs)
    for c in range(p.n_cells):
        dofs = p.celldofs(c) - 1
        ue = u[dofs].astype(np.float32)
        acc = np.zeros(len(dofs), np.float32)
        for J in range(len(dofs)):
            acc = (ke[c, :, J].astype(np.float64) * np.float64(ue[J]) + acc.astype(np.float64)).astype(np.float32)
        y[dofs] += acc.astype(np.float64)
    assert np.array_equal(y, y_row)


def test_csr_assembly_pins(oracle):
    """CSR assembly (ext/FerriteSparseMatrixCSR.jl): its pattern is the transpose of the CSC
    pattern, which Ferrite's cell-coupling pattern makes the same arrays; K_csr is the
    transpose of K_csc entry by entry (symmetric physics: equal to rounding); a missing entry
    is reported as the CSR (row, col)."""
    O = oracle
    p = O.box_problem(O.HEXAHEDRON, (3, 2, 2), ncomp=3, perturb=0.2, seed=12)
    rowptr, colval = p.csr_pattern()
    assert np.array_equal(rowptr, p.colptr) and np.array_equal(colval, p.rowval)
    for phys, p0, p1 in ((O.LINEAR_ELASTIC, 200e3, 0.3), (O.HEAT, 1.0, 1.0)):
        if phys == O.HEAT:
            p = O.box_problem(O.QUADRILATERAL, (4, 3), perturb=0.2, seed=13)
            rowptr, colval = p.csr_pattern()
        nz_csc, f_csc = p.assemble(phys, p0, p1)
        nz_csr, f_csr = p.assemble_csr(rowptr, colval, phys, p0, p1)
        import scipy.sparse as sp
        Kr = sp.csr_matrix((nz_csr, colval - 1, rowptr - 1), shape=(p.ndofs, p.ndofs))
        Kc = p.to_scipy(nz_csc)
        assert abs(Kr - Kc).max() <= 1e-14 * abs(Kc).max()
        assert np.array_equal(f_csr, f_csc)
    # a pattern without K[r, c] for some coupled pair: the CSR error names row r, column c
    rp, cv = rowptr.copy(), colval.copy()
    r = 0
    lo, hi = rp[r] - 1, rp[r + 1] - 1
    c = int(cv[hi - 1])                     # last column of row 1
    keep = np.ones(len(cv), bool)
    keep[hi - 1] = False
    cv = cv[keep]
    rp[r + 1:] -= 1
    with pytest.raises(O.OracleError) as ei:
        p.assemble_csr(rp, cv, O.HEAT, 1.0, 1.0)
    assert ei.value.row == r + 1 and ei.value.col == c
