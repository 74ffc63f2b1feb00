"""Matrix-free product with element matrices (fe_element_matvec): y (+)= sum_c A_c^T Ke_c A_c u,
the consumer of the element-assembly output of the GPU how-to (gpu_assembly.jl:265-303).

Parity: bitwise against the oracle's or_element_matvec (the same fused multiply-add chain per
cell in the element precision, FP64 sums in ascending cell order) on the same Ke and u, for
float and double element matrices, row-major and the how-to's column-major layout, with and
without fill-zero. Against the assembled matrix: |y - K u| <= 1e-12 relative (FP64)."""
import numpy as np
import pytest

from helpers import make_handle
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


CASES = {
    # name: (cell type, nel, ip order, components) -- dofs per cell in the comment
    "tri_heat": ("TRIANGLE", (4, 3), 1, 1),           # 3
    "tri_elastic": ("TRIANGLE", (3, 3), 1, 2),        # 6
    "quad_heat": ("QUADRILATERAL", (5, 4), 1, 1),     # 4
    "quad_elastic": ("QUADRILATERAL", (4, 3), 1, 2),  # 8
    "quad9_heat": ("QUADRILATERAL", (3, 3), 2, 1),    # 9
    "quad9_elastic": ("QUADRILATERAL", (3, 2), 2, 2), # 18
    "tet_elastic": ("TETRAHEDRON", (2, 2, 2), 1, 3),  # 12
    "wedge_heat": ("WEDGE", (2, 2, 2), 1, 1),         # 6
    "hex_heat": ("HEXAHEDRON", (3, 3, 2), 1, 1),      # 8
    "hex_elastic": ("HEXAHEDRON", (4, 3, 3), 1, 3),   # 24
    "hex27_heat": ("HEXAHEDRON", (2, 2, 2), 2, 1),    # 27
    "hex27_elastic": ("HEXAHEDRON", (2, 2, 1), 2, 3), # 81
}


def problem(O, case):
    if case == "mixed":
        return mixed_problem(O)
    ct, nel, ip, nc = CASES[case]
    return O.box_problem(getattr(O, ct), nel, ip_order=ip, ncomp=nc, qr_order=3 if ip == 2 else 2,
                         perturb=0.1, seed=21)


@pytest.mark.parametrize("case", sorted(CASES) + ["mixed"])
def test_element_matvec_bitwise(built, oracle, torch_cuda, case):
    torch, fg, O = torch_cuda, built, oracle
    prob = problem(O, case)
    h = make_handle(fg, O, prob)
    n = prob.n_cells
    m = max(prob.ndofs_per_cell(s) for s in range(len(prob.subdomains)))
    rng = np.random.default_rng(7)
    u = torch.as_tensor(rng.standard_normal(prob.ndofs), device="cuda")
    y0 = rng.standard_normal(prob.ndofs)
    for prec, npdt, tdt in ((fg.PREC_MIXED, np.float32, torch.float32), (fg.PREC_FP64, np.float64, torch.float64)):
        ke_np = rng.standard_normal((n, m, m)).astype(npdt)
        # row-major [cell, I, J]
        ke = torch.as_tensor(ke_np, device="cuda")
        op = h.element_operator(ke.stride(), prec)
        y = torch.full((prob.ndofs,), float("nan"), dtype=torch.float64, device="cuda")
        op.matvec(ke, u, y)
        ref = prob.element_matvec(ke_np, u.cpu().numpy())
        assert np.array_equal(y.cpu().numpy(), ref), (case, prec)
        # accumulate into an existing y
        ya = torch.as_tensor(y0.copy(), device="cuda")
        op.matvec(ke, u, ya, fillzero=False)
        refa = prob.element_matvec(ke_np, u.cpu().numpy(), y=y0.copy(), fillzero=False)
        assert np.array_equal(ya.cpu().numpy(), refa), (case, prec)
        op.close()
        # the how-to's Kes[ncells, nbf, nbf] (column-major: cell fastest)
        kj = ke.permute(2, 1, 0).contiguous()
        opj = h.element_operator((1, n, n * m), prec)
        yj = torch.full((prob.ndofs,), float("nan"), dtype=torch.float64, device="cuda")
        opj.matvec(kj, u, yj)
        assert torch.equal(yj, y), (case, prec)
        opj.close()


def test_element_matvec_of_assembled_elements(built, oracle, torch_cuda):
    """With the FP64 element matrices of fe_assemble_elements, the product equals K u of
    fe_assemble's FP64 K; with the mixed (float) ones it agrees to FP32 rounding."""
    torch, fg, O = torch_cuda, built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (6, 5, 4), ncomp=3, perturb=0.2, seed=23)
    h = make_handle(fg, O, prob)
    n, nbf = prob.n_cells, prob.ndofs_per_cell(0)
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0))
    nz = np.zeros(prob.nnz)
    f = np.zeros(prob.ndofs)
    h.assemble(nz, f, precision=fg.PREC_FP64, **kw)
    u_np = np.random.default_rng(8).standard_normal(prob.ndofs)
    Ku = prob.to_scipy(nz) @ u_np
    u = torch.as_tensor(u_np, device="cuda")
    for prec, dt, tol in ((fg.PREC_FP64, torch.float64, 1e-12), (fg.PREC_MIXED, torch.float32, 1e-6)):
        ke = torch.zeros((n, nbf, nbf), dtype=dt, device="cuda")
        h.assemble_elements(ke, None, fe_stride=(0, 0), precision=prec, **kw)
        op = h.element_operator(ke.stride(), prec)
        y = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
        op.matvec(ke, u, y)
        err = np.linalg.norm(y.cpu().numpy() - Ku) / np.linalg.norm(Ku)
        assert err <= tol, (prec, err)
        op.close()


def test_element_matvec_arguments(built, oracle, torch_cuda):
    torch, fg, O = torch_cuda, built, oracle
    prob = O.box_problem(O.QUADRILATERAL, (3, 3))
    h = make_handle(fg, O, prob)
    ke = torch.zeros((9, 4, 4), dtype=torch.float32, device="cuda")
    op = h.element_operator(ke.stride())
    u = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    with pytest.raises(fg.FEError) as ei:
        op.matvec(ke, u, np.zeros(prob.ndofs))  # host y
    assert ei.value.name == "ARG"
    with pytest.raises(fg.FEError):
        h.element_operator(ke.stride(), 7)  # unknown precision
    op.close()
