"""CUDA-graph re-assembly (fe_graph_capture / fe_graph_replay): a Newton-style sequence of
Neo-Hooke assemblies with different u, captured once and replayed, against direct assemblies.
Replays read the buffers' current contents, so u updated in place is re-assembled."""
import numpy as np
import pytest

from helpers import make_handle, rel_fro

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


def test_graph_replay_matches_direct_assembly(built, oracle, torch_cuda):
    torch = torch_cuda
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (5, 4, 4), ncomp=3, perturb=0.2, seed=3)
    h = make_handle(fg, O, prob)
    rng = np.random.default_rng(1)
    us = [torch.as_tensor(0.05 * rng.uniform(-1, 1, prob.ndofs), device="cuda") for _ in range(3)]
    nz = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    f = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    kw = dict(physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, body=(0.0, 0.0, -0.5))
    stream = torch.cuda.Stream()
    gid = h.graph_capture([dict(u=u, **kw) for u in us], [nz] * 3, [f] * 3, stream)
    nz.zero_()
    f.zero_()
    h.graph_replay(gid, stream)
    # the last step writes last: compare with a direct assembly of us[-1]
    nz_ref = torch.zeros_like(nz)
    f_ref = torch.zeros_like(f)
    h.assemble(nz_ref, f_ref, u=us[-1], **kw)
    assert torch.equal(nz, nz_ref) and torch.equal(f, f_ref)
    # against the oracle
    nz_o, f_o = prob.assemble(O.NEO_HOOKE, 1.0, 10.0, body=(0.0, 0.0, -0.5), u=us[-1].cpu().numpy())
    assert rel_fro(nz.cpu().numpy(), nz_o) <= 2e-6 and rel_fro(f.cpu().numpy(), f_o) <= 2e-6
    # update u in place and replay
    us[-1].copy_(torch.as_tensor(0.03 * rng.uniform(-1, 1, prob.ndofs), device="cuda"))
    h.graph_replay(gid, stream)
    h.assemble(nz_ref, f_ref, u=us[-1], **kw)
    assert torch.equal(nz, nz_ref) and torch.equal(f, f_ref)
    # profiled, asynchronous replays
    for _ in range(3):
        h.graph_replay(gid, stream, sync=False, profile=True)
    h.sync()
    ms, n = h.kernel_time()
    assert n == 3 and ms > 0
    h.graph_destroy(gid)


def test_graph_capture_rejects_host_buffers(built, oracle):
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (2, 2, 2), ncomp=3)
    h = make_handle(fg, O, prob)
    import torch
    stream = torch.cuda.Stream()
    with pytest.raises(fg.FEError) as e:
        h.graph_capture([dict(physics=fg.LINEAR_ELASTIC, p0=1.0, p1=0.3)], [np.zeros(prob.nnz)], [np.zeros(prob.ndofs)],
                        stream)
    assert e.value.code == 1


def test_autotune_keeps_fastest_plan_and_results(built, oracle, torch_cuda):
    """fe_autotune re-plans with each staging capacity; every candidate assembles the same
    matrix (the plan does not change values), and the handle keeps the fastest plan."""
    torch = torch_cuda
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (10, 9, 8), ncomp=3, perturb=0.2, seed=5)
    h = make_handle(fg, O, prob)
    nz = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    f = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0))
    h.assemble(nz, f, **kw)
    nz0, f0 = nz.clone(), f.clone()
    res = h.autotune(nz, f, stage_caps=[4096, 8192, 12288], reps=2, **kw)
    assert res["best_stage_cap"] in (4096, 8192, 12288)
    assert all(c[1] > 0 for c in res["candidates"])
    assert res["best_form_mask"] in (0, 1)  # one subdomain: fused or two-phase
    assert res["candidates"][0][2] > res["candidates"][2][2]  # smaller tiles, more of them
    nz.zero_()
    f.zero_()
    h.assemble(nz, f, **kw)
    # summation order is cell order whatever the tiles: bitwise the same
    assert torch.equal(nz, nz0) and torch.equal(f, f0)


def test_graph_replay_two_phase_tensor_core(built, oracle, torch_cuda):
    """Q2 hexahedra (two-phase form, element matrices on the tensor cores) captured as a
    graph: the element kernel, the gather-only tile kernel and the scratch they share."""
    torch = torch_cuda
    fg, O = built, oracle
    prob = O.box_problem(O.HEXAHEDRON, (3, 3, 2), ip_order=2, ncomp=3, qr_order=3, perturb=0.2, seed=8)
    h = make_handle(fg, O, prob)
    rng = np.random.default_rng(2)
    scales = [torch.as_tensor(rng.lognormal(0.0, 0.5, prob.n_cells), device="cuda") for _ in range(2)]
    nz = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    f = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=200e3, p1=0.3, body=(0.0, 0.0, -1.0))
    stream = torch.cuda.Stream()
    nz2 = torch.zeros_like(nz)
    gid = h.graph_capture([dict(cell_scale=scales[0], **kw), dict(cell_scale=scales[1], **kw)], [nz, nz2], [f, f], stream)
    nz.zero_()
    nz2.zero_()
    h.graph_replay(gid, stream)
    ref1 = torch.zeros_like(nz)
    ref2 = torch.zeros_like(nz)
    fr = torch.zeros_like(f)
    h.assemble(ref1, fr, cell_scale=scales[0], **kw)
    h.assemble(ref2, fr, cell_scale=scales[1], **kw)
    assert torch.equal(nz, ref1) and torch.equal(nz2, ref2) and torch.equal(f, fr)
    h.graph_destroy(gid)


def test_autotune_chooses_a_form_per_cell_type(built, oracle, torch_cuda):
    """On a hexahedron / tetrahedron / wedge grid (three SubDofHandlers) the tuner times every
    assignment of the cell types to the fused or two-phase form; all of them give the same bits
    (the element math is the same on the CUDA cores), and later calls without a form use the
    chosen one."""
    from test_gpu_parity import mixed_problem
    torch = torch_cuda
    fg, O = built, oracle
    prob = mixed_problem(O, nel=(9, 4, 4), seed=6)
    h = make_handle(fg, O, prob)
    rng = np.random.default_rng(3)
    u = torch.as_tensor(0.02 * rng.uniform(-1, 1, prob.ndofs), device="cuda")
    nz = torch.zeros(prob.nnz, dtype=torch.float64, device="cuda")
    f = torch.zeros(prob.ndofs, dtype=torch.float64, device="cuda")
    kw = dict(physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, u=u)
    h.assemble(nz, f, form="fused", **kw)
    ref = (nz.clone(), f.clone())
    res = h.autotune(nz, f, stage_caps=[8192, 12288], reps=1, **kw)  # all 8 form masks per capacity
    assert 0 <= res["best_form_mask"] < 8
    assert res["best_form_mask"] in [c[4] for c in res["candidates"]]
    assert torch.equal(nz, ref[0]) and torch.equal(f, ref[1])  # the tuner's last assembly
    nz.zero_()
    f.zero_()
    h.assemble(nz, f, **kw)  # the tuned form
    assert torch.equal(nz, ref[0]) and torch.equal(f, ref[1])
    for form in ("fused", "two_phase"):
        nz.zero_()
        f.zero_()
        h.assemble(nz, f, form=form, **kw)
        assert torch.equal(nz, ref[0]) and torch.equal(f, ref[1]), form
