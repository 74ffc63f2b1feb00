"""GPU parity: the CUDA engine (through the C ABI) against the CPU oracle.

Tolerances (relative Frobenius norm of nzval and f against the FP64 oracle):
  * FE_PREC_FP64 (the plain FP64 drop-in):      <= 1e-12
  * FE_PREC_MIXED (FP32 element math, compensated sums per entry rounded exactly to FP64): <= 1e-6
Sparsity structure and index maps are bit-exact. Runs are bitwise reproducible.
"""
import numpy as np
import pytest

from helpers import make_handle, rel_fro

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_MIXED = 1e-6


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


def check(fg, O, prob, element_args, oracle_args, precisions=(0, 1), tol=None):
    h = make_handle(fg, O, prob)
    nz_ref, f_ref = prob.assemble(**oracle_args)
    out = {}
    for prec in precisions:
        nz = np.full(prob.nnz, np.nan)
        f = np.full(prob.ndofs, np.nan)
        h.assemble(nz, f, precision=prec, **element_args)
        t = (tol or {}).get(prec, TOL_FP64 if prec == 1 else TOL_MIXED)
        assert rel_fro(nz, nz_ref) <= t, (prec, rel_fro(nz, nz_ref))
        assert rel_fro(f, f_ref) <= t, (prec, rel_fro(f, f_ref))
        out[prec] = (nz, f)
    return h, out


def test_heat_quad_100x100(built, oracle):
    """2D Poisson as in the heat tutorial, 100x100 Q1, 2x2 Gauss (10,201 dofs)."""
    fg, O = built, oracle
    prob = O.box_problem(O.QUADRILATERAL, (100, 100), qr_order=2)
    check(fg, O, prob, dict(physics=fg.HEAT, p0=1.0, p1=1.0), dict(physics=O.HEAT, p0=1.0, p1=1.0))


def test_elastic_hex_q1_perturbed(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (9, 7, 6), [0, 0, 0], [1, 1, 1], ip_order=1, ncomp=3, qr_order=2,
                         perturb=0.2, seed=11)
    E, nu, b = 200e3, 0.3, (0.0, 0.0, -1.0)
    check(fg, O, prob, dict(physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, body=b),
          dict(physics=O.LINEAR_ELASTIC, p0=E, p1=nu, body=b))


def test_elastic_hex_q2_cell_modulus(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (4, 3, 3), [0, 0, 0], [1, 1, 1], ip_order=2, ncomp=3, qr_order=3,
                         perturb=0.2, seed=12)
    rng = np.random.default_rng(5)
    scale = rng.lognormal(0.0, 0.5, prob.n_cells)
    E, nu = 200e3, 0.3
    check(fg, O, prob, dict(physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, cell_scale=scale),
          dict(physics=O.LINEAR_ELASTIC, p0=E, p1=nu, cell_scale=scale))


@pytest.mark.parametrize("ct,qo", [(3, 1), (5, 2), (4, 2)])
def test_neo_hooke_single_type(built, oracle, ct, qo):
    fg, O = built, oracle
    prob = O.box_problem(ct, (4, 3, 3), [0, 0, 0], [1, 1, 1], ip_order=1, ncomp=3, qr_order=qo, perturb=0.15, seed=3)
    rng = np.random.default_rng(1)
    u = 0.05 * rng.uniform(-1, 1, prob.ndofs)
    check(fg, O, prob, dict(physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, u=u, body=(0, -0.5, 0)),
          dict(physics=O.NEO_HOOKE, p0=1.0, p1=10.0, u=u, body=(0, -0.5, 0)), tol={0: 2e-6})


def mixed_problem(O, nel=(6, 3, 3), seed=4, ncomp=3):
    """Three x-slabs over one node grid: hexahedra, then tetrahedra (6 per cube), then
    wedges (2 per cube), one SubDofHandler each, dofs shared through the vertex dict."""
    nodes, hexes = O.generate_grid(O.HEXAHEDRON, nel, [0, 0, 0], [2, 1, 1])
    nodes = O.perturb_interior(nodes, nel, 0.15, seed, [0, 0, 0], [2, 1, 1])
    nx = nel[0]
    i = (np.arange(len(hexes)) % nx)
    third = nx // 3
    T = [[1, 2, 4, 8], [1, 5, 2, 8], [2, 3, 4, 8], [2, 7, 3, 8], [2, 5, 6, 8], [2, 6, 7, 8]]
    W = [[1, 2, 4, 5, 6, 8], [2, 3, 4, 6, 7, 8]]
    cells, types = [], []
    for c in np.where(i < third)[0]:
        cells.append(hexes[c]); types.append(O.HEXAHEDRON)
    for c in np.where((i >= third) & (i < 2 * third))[0]:
        for t in T:
            cells.append(hexes[c][np.array(t) - 1]); types.append(O.TETRAHEDRON)
    for c in np.where(i >= 2 * third)[0]:
        for t in W:
            cells.append(hexes[c][np.array(t) - 1]); types.append(O.WEDGE)
    types = np.array(types, np.int32)
    off = np.zeros(len(cells) + 1, np.int64)
    off[1:] = np.cumsum([len(c) for c in cells])
    flat = np.concatenate(cells).astype(np.int64)
    subs = []
    for ct, qo in [(O.HEXAHEDRON, 2), (O.TETRAHEDRON, 1), (O.WEDGE, 2)]:
        subs.append(O.Subdomain(np.where(types == ct)[0] + 1, 1, ncomp, qo))
    prob = O.Problem(nodes, types, off, flat, subs).close().allocate_matrix()
    return prob


def mixed_problem_2d(O, nel=(8, 5), seed=7, ncomp=2):
    """Two x-halves over one node grid: quadrilaterals, then triangles (2 per square), one
    SubDofHandler each (quadrilaterals 2x2 Gauss, triangles 1 point)."""
    nodes, quads = O.generate_grid(O.QUADRILATERAL, nel, [0, 0], [2, 1])
    nodes = O.perturb_interior(nodes, nel, 0.15, seed, [0, 0], [2, 1])
    i = np.arange(len(quads)) % nel[0]
    cells, types = [], []
    for c in np.where(i < nel[0] // 2)[0]:
        cells.append(quads[c]); types.append(O.QUADRILATERAL)
    for c in np.where(i >= nel[0] // 2)[0]:
        q = quads[c]
        for t in ([0, 1, 2], [0, 2, 3]):
            cells.append(q[np.array(t)]); types.append(O.TRIANGLE)
    types = np.array(types, np.int32)
    off = np.zeros(len(cells) + 1, np.int64)
    off[1:] = np.cumsum([len(c) for c in cells])
    flat = np.concatenate(cells).astype(np.int64)
    subs = [O.Subdomain(np.where(types == ct)[0] + 1, 1, ncomp, qo) for ct, qo in [(O.QUADRILATERAL, 2), (O.TRIANGLE, 1)]]
    return O.Problem(nodes, types, off, flat, subs).close().allocate_matrix()


@pytest.mark.parametrize("dim", [3, 2])
def test_heat_and_elastic_mixed_cells(built, oracle, dim):
    """Heat and linear elasticity over grids with several cell types in one launch: hexahedra /
    tetrahedra / wedges in 3D, quadrilaterals / triangles in 2D (one SubDofHandler per type,
    dofs shared across the type boundary)."""
    fg, O = built, oracle
    make = mixed_problem if dim == 3 else mixed_problem_2d
    heat = make(O, ncomp=1)
    check(fg, O, heat, dict(physics=fg.HEAT, p0=2.0, p1=1.0), dict(physics=O.HEAT, p0=2.0, p1=1.0))
    el = make(O, ncomp=dim)
    b = (0.0, -1.0, 0.0)[:dim] + (0.0,) * (3 - dim)
    rng = np.random.default_rng(8)
    scale = rng.uniform(0.5, 2.0, el.n_cells)
    check(fg, O, el, dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=b, cell_scale=scale),
          dict(physics=O.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=list(b), cell_scale=scale))


def test_neo_hooke_mixed_cells(built, oracle):
    fg, O = built, oracle
    prob = mixed_problem(O)
    rng = np.random.default_rng(2)
    u = 0.05 * rng.uniform(-1, 1, prob.ndofs)
    check(fg, O, prob, dict(physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, u=u),
          dict(physics=O.NEO_HOOKE, p0=1.0, p1=10.0, u=u), tol={0: 2e-6})


def test_index_map_bit_exact(built, oracle):
    fg, O = built, oracle
    for ct, ip, nc, nel in [(4, 1, 3, (3, 3, 2)), (4, 2, 3, (2, 2, 2)), (2, 1, 1, (4, 3)), (3, 1, 3, (2, 2, 1))]:
        prob = O.box_problem(ct, nel, ip_order=ip, ncomp=nc, qr_order=2)
        h = make_handle(fg, O, prob)
        for c in range(prob.n_cells):
            ld = prob.ndofs_per_cell(0)
            assert np.array_equal(h.index_map(c + 1, ld), prob.index_map(c))


def test_bitwise_reproducible_and_device_pointers(built, oracle, torch_cuda):
    fg, O, torch = built, oracle, torch_cuda
    prob = O.box_problem(O.HEXAHEDRON, (8, 8, 8), [0, 0, 0], [1, 1, 1], ip_order=1, ncomp=3, perturb=0.2, seed=9)
    h = make_handle(fg, O, prob)
    args = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0, 0, -1))
    a = [np.zeros(prob.nnz), np.zeros(prob.ndofs)]
    b = [np.zeros(prob.nnz), np.zeros(prob.ndofs)]
    h.assemble(*a, **args)
    h.assemble(*b, **args)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    nz_d = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    f_d = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    h.assemble(nz_d, f_d, stream=torch.cuda.current_stream(), **args)
    torch.cuda.synchronize()
    assert np.array_equal(nz_d.cpu().numpy(), a[0]) and np.array_equal(f_d.cpu().numpy(), a[1])


def test_fillzero_false_accumulates(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.QUADRILATERAL, (7, 5), qr_order=2)
    h = make_handle(fg, O, prob)
    nz1, f1 = np.zeros(prob.nnz), np.zeros(prob.ndofs)
    h.assemble(nz1, f1, physics=fg.HEAT, p0=1.0, p1=1.0, precision=fg.PREC_FP64)
    nz2, f2 = nz1.copy(), f1.copy()
    h.assemble(nz2, f2, physics=fg.HEAT, p0=1.0, p1=1.0, precision=fg.PREC_FP64, fillzero=False)
    assert np.allclose(nz2, 2 * nz1, rtol=1e-14, atol=0) and np.allclose(f2, 2 * f1, rtol=1e-14)


def test_detj_error(built, oracle):
    fg, O = built, oracle
    nodes, cells = O.generate_grid(O.QUADRILATERAL, (3, 3))
    cells[4] = cells[4][[1, 0, 3, 2]]
    prob = O.Problem.single(O.QUADRILATERAL, nodes, cells).close().allocate_matrix()
    h = make_handle(fg, O, prob)
    for form in ("fused", "two_phase"):
        for prec in (0, 1):
            with pytest.raises(fg.FEError) as ei:
                h.assemble(np.zeros(prob.nnz), np.zeros(prob.ndofs), physics=fg.HEAT, p0=1.0, p1=1.0, precision=prec,
                           form=form)
            assert ei.value.name == "DETJ" and ei.value.cell == 5 and ei.value.detJ < 0


def test_async_chain_matches_sync_and_keeps_errors(built, oracle, torch_cuda):
    """FE_ASYNC assemblies on one stream with device outputs run back to back without host
    waits; their statuses accumulate, so an error of any of them is reported at fe_sync."""
    torch = torch_cuda
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (6, 5, 4), ncomp=3, perturb=0.2, seed=6)
    h = make_handle(fg, O, prob)
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=1.0, p1=0.3, body=(0.0, 0.0, -1.0))
    nz0 = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    f0 = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    h.assemble(nz0, f0, **kw)
    nz = torch.zeros_like(nz0)
    f = torch.zeros_like(f0)
    s = torch.cuda.Stream()
    for _ in range(4):
        h.assemble(nz, f, stream=s, sync=False, **kw)
    h.sync()
    assert torch.equal(nz, nz0) and torch.equal(f, f0)
    # an inverted cell in a chain: reported once the chain is synchronised
    nodes, cells = O.generate_grid(O.QUADRILATERAL, (3, 3))
    cells[4] = cells[4][[1, 0, 3, 2]]
    bad = O.Problem.single(O.QUADRILATERAL, nodes, cells).close().allocate_matrix()
    hb = make_handle(fg, O, bad)
    nzb = torch.zeros(bad.nnz, dtype=torch.float64, device="cuda")
    fb = torch.zeros(bad.ndofs, dtype=torch.float64, device="cuda")
    for _ in range(3):
        hb.assemble(nzb, fb, physics=fg.HEAT, p0=1.0, p1=1.0, stream=s, sync=False)
    with pytest.raises(fg.FEError) as ei:
        hb.sync()
    assert ei.value.name == "DETJ" and ei.value.cell == 5


def test_pattern_missing_error(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.QUADRILATERAL, (3, 3), qr_order=2)
    col = 5
    a, b = prob.colptr[col] - 1, prob.colptr[col + 1] - 1
    rows = prob.rowval[a:b]
    drop = a + int(np.where(rows != col + 1)[0][0])
    dropped_row = int(prob.rowval[drop])
    prob.rowval = np.delete(prob.rowval, drop)
    prob.colptr = prob.colptr.copy()
    prob.colptr[col + 1:] -= 1
    h = make_handle(fg, O, prob)
    for form in ("fused", "two_phase"):
        with pytest.raises(fg.FEError) as ei:
            h.assemble(np.zeros(prob.nnz), np.zeros(prob.ndofs), physics=fg.HEAT, p0=1.0, p1=1.0, form=form)
        assert ei.value.name == "PATTERN_MISSING"
        assert (ei.value.row, ei.value.col) in [(dropped_row, col + 1)]
        # zero contributions to the missing entry are fine (k = 0)
        h.assemble(np.zeros(prob.nnz), np.zeros(prob.ndofs), physics=fg.HEAT, p0=0.0, p1=1.0, form=form)


def test_distorted_cells_use_fp64_jacobians(built, oracle):
    """A layer of thin cells (aspect ratio ~2500, detJ > 0, Jacobian condition number far
    above the threshold) is recomputed with FP64 Jacobians; the mixed result stays within
    tolerance."""
    fg, O = built, oracle
    nel = (4, 4, 4)
    nodes, cells = O.generate_grid(O.HEXAHEDRON, nel, [0, 0, 0], [1, 1, 1])
    nodes = nodes.copy()
    nodes[np.abs(nodes[:, 2] - 0.25) < 1e-12, 2] = 1e-4
    prob = O.Problem.single(O.HEXAHEDRON, nodes, cells, 1, 3, 2).close().allocate_matrix()
    h = make_handle(fg, O, prob)
    nz_ref, f_ref = prob.assemble(O.LINEAR_ELASTIC, 200e3, 0.3, body=[0, 0, -1])
    nz, f = np.zeros(prob.nnz), np.zeros(prob.ndofs)
    h.assemble(nz, f, physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0, 0, -1), cond_threshold=16.0)
    # 16 thin cells; a cell is evaluated once per owner tile it touches, each evaluation counts
    assert h.info()["flagged_cells"] >= 16
    assert rel_fro(nz, nz_ref) <= TOL_MIXED and rel_fro(f, f_ref) <= TOL_MIXED


def test_unaligned_device_output(built, oracle, torch_cuda):
    """nzval views that are only 8-byte aligned take the scalar store path, same bits."""
    fg, O, torch = built, oracle, torch_cuda
    prob = O.box_problem(O.HEXAHEDRON, (5, 4, 3), [0, 0, 0], [1, 1, 1], ip_order=1, ncomp=3, perturb=0.2, seed=4)
    h = make_handle(fg, O, prob)
    args = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0, 0, -1), stream=torch.cuda.current_stream())
    a = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    buf = torch.zeros(prob.nnz + 1, dtype=torch.float64, device="cuda")
    b = buf[1:]
    f = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    h.assemble(a, f, **args)
    h.assemble(b, f, **args)
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def _forms_bitwise(fg, O, prob, element_args):
    """Element matrices first (two-phase, CUDA cores) and in-tile (fused) give the same bits,
    with fill-zero and accumulating: the same FP32 element math feeds the same per-entry sums
    in cell order."""
    h = make_handle(fg, O, prob)
    out = {}
    forms = ("fused", "two_phase_cuda_cores")
    for form in forms:
        for prec in (0, 1):
            nz = np.full(prob.nnz, np.nan)
            f = np.full(prob.ndofs, np.nan)
            h.assemble(nz, f, precision=prec, form=form, **element_args)
            out[form, prec] = (nz, f)
            # accumulation without fill-zero follows the same sums
            h.assemble(nz, f, precision=prec, form=form, fillzero=False, **element_args)
            out[form, prec, "acc"] = (nz.copy(), f.copy())
    for prec in (0, 1):
        for form in forms[1:]:
            for key in ((prec,), (prec, "acc")):
                a, b = out[("fused",) + key], out[(form,) + key]
                assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (form, key)
    return h


@pytest.mark.parametrize("case", ["hex_q1_elastic", "hex_q2_elastic", "hex_q2_heat", "quad_q2_heat", "tet_elastic"])
def test_two_phase_matches_fused_bitwise(built, oracle, case):
    fg, O = built, oracle
    E, nu, b = 200e3, 0.3, (0.0, 0.0, -1.0)
    el = dict(physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, body=b)
    ht = dict(physics=fg.HEAT, p0=1.0, p1=1.0)
    if case == "hex_q1_elastic":
        prob = O.box_problem(O.HEXAHEDRON, (7, 6, 5), ip_order=1, ncomp=3, qr_order=2, perturb=0.2, seed=21)
        args = el
    elif case == "hex_q2_elastic":
        prob = O.box_problem(O.HEXAHEDRON, (4, 3, 3), ip_order=2, ncomp=3, qr_order=3, perturb=0.2, seed=22)
        args = dict(el, cell_scale=np.random.default_rng(3).lognormal(0.0, 0.5, prob.n_cells))
    elif case == "hex_q2_heat":
        prob = O.box_problem(O.HEXAHEDRON, (4, 4, 3), ip_order=2, ncomp=1, qr_order=3, perturb=0.2, seed=23)
        args = ht
    elif case == "quad_q2_heat":
        prob = O.box_problem(O.QUADRILATERAL, (12, 9), ip_order=2, ncomp=1, qr_order=3, perturb=0.2, seed=24)
        args = ht
    else:
        prob = O.box_problem(O.TETRAHEDRON, (4, 3, 3), ip_order=1, ncomp=3, qr_order=1, perturb=0.15, seed=25)
        args = el
    _forms_bitwise(fg, O, prob, args)


def test_two_phase_neo_hooke_mixed_cells(built, oracle):
    fg, O = built, oracle
    prob = mixed_problem(O)
    u = 0.05 * np.random.default_rng(7).uniform(-1, 1, prob.ndofs)
    _forms_bitwise(fg, O, prob, dict(physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, u=u))


def test_two_phase_q2_against_oracle(built, oracle):
    """The default form of quadratic elements (two-phase) against the oracle."""
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (3, 3, 2), ip_order=2, ncomp=3, qr_order=3, perturb=0.2, seed=26)
    E, nu = 200e3, 0.3
    check(fg, O, prob, dict(physics=fg.LINEAR_ELASTIC, p0=E, p1=nu), dict(physics=O.LINEAR_ELASTIC, p0=E, p1=nu))


def test_pinned_host_outputs_written_directly(built, oracle, torch_cuda):
    """Page-locked host nzval/f are written by the kernels through their mapping (no staging
    copy): the same bits as device outputs, including accumulation without fill-zero."""
    torch = torch_cuda
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (6, 5, 4), ncomp=3, perturb=0.2, seed=51)
    h = make_handle(fg, O, prob)
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0))
    nz_d = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    f_d = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    h.assemble(nz_d, f_d, **kw)
    nz_p = torch.full((prob.nnz,), float("nan"), dtype=torch.float64).pin_memory()
    f_p = torch.full((prob.ndofs,), float("nan"), dtype=torch.float64).pin_memory()
    h.assemble(nz_p, f_p, **kw)
    assert torch.equal(nz_p, nz_d.cpu()) and torch.equal(f_p, f_d.cpu())
    h.assemble(nz_p, f_p, fillzero=False, **kw)
    h.assemble(nz_d, f_d, fillzero=False, **kw)
    assert torch.equal(nz_p, nz_d.cpu()) and torch.equal(f_p, f_d.cpu())
    s = torch.cuda.Stream()
    nz_p.fill_(float("nan"))
    h.assemble(nz_p, f_p, stream=s, sync=False, **kw)
    h.sync()
    h.assemble(nz_d, f_d, **kw)
    assert torch.equal(nz_p, nz_d.cpu())


@pytest.mark.parametrize("nel,scale", [((3, 3, 2), False), ((4, 3, 3), True), ((5, 4, 4), True)])
def test_q2_tensor_core_elements(built, oracle, nel, scale):
    """Q2 hexahedron elasticity with the element matrices on the tensor cores (tcgen05,
    split-TF32 Gram products, FP32 accumulation; the default for this element) against the
    FP64 oracle (1e-6) and against the CUDA-core element matrices (FP32-rounding apart)."""
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, nel, ip_order=2, ncomp=3, qr_order=3, perturb=0.2, seed=61 + nel[0])
    E, nu, b = 200e3, 0.3, (0.0, -1.0, 0.5)
    sc = np.random.default_rng(6).lognormal(0.0, 0.5, prob.n_cells) if scale else None
    h, out = check(fg, O, prob, dict(physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, body=b, cell_scale=sc),
                   dict(physics=O.LINEAR_ELASTIC, p0=E, p1=nu, body=b, cell_scale=sc), precisions=(0,))
    nz_tc, f_tc = out[0]
    nz_cc, f_cc = np.zeros(prob.nnz), np.zeros(prob.ndofs)
    h.assemble(nz_cc, f_cc, physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, body=b, cell_scale=sc, form="two_phase_cuda_cores")
    assert rel_fro(nz_tc, nz_cc) <= 1e-6
    assert np.array_equal(f_tc, f_cc)  # the loads are computed the same way on both paths
    # no K / no f
    nz1 = np.full(prob.nnz, 7.0)
    f1 = np.zeros(prob.ndofs)
    h.assemble(None, f1, physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, body=b, cell_scale=sc)
    assert np.array_equal(f1, f_tc)
    h.assemble(nz1, None, physics=fg.LINEAR_ELASTIC, p0=E, p1=nu, body=b, cell_scale=sc)
    assert np.array_equal(nz1, nz_tc)


def test_q2_tensor_core_detj_error(built, oracle):
    fg, O = built, oracle
    nodes, cells = O.generate_grid(O.HEXAHEDRON, (2, 2, 2))
    cells[3] = cells[3][[1, 0, 3, 2, 5, 4, 7, 6]]
    prob = O.Problem.single(O.HEXAHEDRON, nodes, cells, ip_order=2, ncomp=3, qr_order=3).close().allocate_matrix()
    h = make_handle(fg, O, prob)
    with pytest.raises(fg.FEError) as ei:
        h.assemble(np.zeros(prob.nnz), np.zeros(prob.ndofs), physics=fg.LINEAR_ELASTIC, p0=1.0, p1=0.3)
    assert ei.value.name == "DETJ" and ei.value.cell == 4
