"""Host-side set-up on the CPU (no GPU): input validation, the index map and the owner-tile
plan with its bounds check, through fe_plan_dry_run."""
import numpy as np
import pytest

from helpers import subdomain_specs


def dry(fg, O, prob):
    return fg.plan_dry_run(prob.nodes, subdomain_specs(fg, O, prob), prob.cell_dofs, prob.cell_dofs_offset,
                           prob.ndofs, prob.colptr, prob.rowval, prob.n_cells)


@pytest.mark.parametrize("ct,nel,ip,nc,qo", [(2, (13, 9), 1, 1, 2), (2, (6, 5), 1, 2, 2), (4, (7, 6, 5), 1, 3, 2),
                                             (4, (4, 3, 3), 2, 3, 3), (3, (4, 4, 3), 1, 3, 1), (5, (4, 3, 3), 1, 3, 2),
                                             (1, (5, 4), 1, 1, 1), (1, (6, 5), 1, 2, 1), (2, (4, 3), 2, 2, 3),
                                             (5, (4, 3, 3), 1, 1, 2)])
def test_dry_run_plans(fg, oracle, ct, nel, ip, nc, qo):
    fg.build()
    O = oracle
    prob = O.box_problem(ct, nel, ip_order=ip, ncomp=nc, qr_order=qo, perturb=0.1, seed=1)
    info = dry(fg, O, prob)
    assert info["ndofs"] == prob.ndofs and info["nnz"] == prob.nnz
    assert info["n_items"] == prob.n_cells * O.nbase(ct, ip)
    assert info["n_cell_visits"] >= prob.n_cells and info["n_tiles"] >= 1


def test_dry_run_mixed(fg, oracle):
    from test_gpu_parity import mixed_problem
    fg.build()
    prob = mixed_problem(oracle)
    info = dry(fg, oracle, prob)
    assert info["n_cells"] == prob.n_cells


def test_rejects_bad_input(fg, oracle):
    fg.build()
    O = oracle
    prob = O.box_problem(O.HEXAHEDRON, (2, 2, 2), ip_order=1, ncomp=3)
    cells = prob.cell_nodes.copy()
    prob.cell_nodes = cells
    bad = prob.cell_nodes.copy()
    bad[5] = prob.nodes.shape[0] + 7
    prob.cell_nodes = bad
    with pytest.raises(fg.FEError) as ei:
        dry(fg, O, prob)
    assert ei.value.name == "BOUNDS"
    prob.cell_nodes = cells
    # a pattern that does not couple all components of an entity is not supported
    rowval = prob.rowval.copy()
    colptr = prob.colptr.copy()
    drop = int(colptr[0] - 1) + 1  # second row entry of column 1 (same entity, component 2)
    prob.rowval = np.delete(rowval, drop)
    prob.colptr = colptr.copy()
    prob.colptr[1:] -= 1
    with pytest.raises(fg.FEError) as ei:
        dry(fg, O, prob)
    assert ei.value.name == "UNSUPPORTED"


_DIGEST_SCRIPT = r"""
import sys
sys.path[:0] = [{tests!r}, {oracle!r}]
import conftest
fg = conftest.load_package()
import oracle as O
from helpers import subdomain_specs
for ct, nel, ip, nc in [(4, (40, 40, 42), 1, 1), (4, (12, 10, 9), 1, 3), (4, (5, 4, 4), 2, 3), (4, (200, 200, 2), 1, 1)]:
    p = O.box_problem(ct, nel, ip_order=ip, ncomp=nc, qr_order=3 if ip == 2 else 2, perturb=0.1, seed=2)
    info = fg.plan_dry_run(p.nodes, subdomain_specs(fg, O, p), p.cell_dofs, p.cell_dofs_offset, p.ndofs, p.colptr,
                           p.rowval, p.n_cells)
    print(info["n_tiles"], info["plan_checksum"])
"""


def test_plan_independent_of_thread_count(fg, oracle):
    """The planner splits large bisection parts as OpenMP tasks and builds records in parallel;
    the plan (its record digest) is the same with 1 and 4 host threads, including a problem
    large enough (70k entities) for the parallel bisection and a thin slab (121k nodes, most of
    them on its faces) whose uneven entity loads cut every part by its own summed load."""
    import os
    import subprocess
    import sys
    fg.build()
    here = os.path.dirname(os.path.abspath(__file__))
    script = _DIGEST_SCRIPT.format(tests=here, oracle=os.path.join(os.path.dirname(here), "oracle"))
    outs = []
    for threads in ("1", "4"):
        env = dict(os.environ, OMP_NUM_THREADS=threads)
        r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(r.stdout.split())
    assert outs[0] == outs[1] and len(outs[0]) == 8
    assert all(int(x) != 0 for x in outs[0][1::2])
