"""Benchmark: K+f assembly throughput of 3D Q1 hexahedral small-strain elasticity at 128^3.

Workload (one "step" = one full K+f assembly, start_assemble + the whole cell loop):
generate_grid(Hexahedron, (128,128,128)) on the unit cube, interior nodes perturbed by
seeded uniform noise of +-0.2h, Lagrange{RefHexahedron,1}^3 (6,440,067 dofs), 2x2x2 Gauss,
E = 200e3, nu = 0.3, body force (0,0,-1); nnz(K) = 513,599,625. Synthetic inputs (the
reference publishes no dataset for this path). nzval (4.1 GB) is larger than L2, and the
per-step inputs (coordinates, connectivity, tile plan: ~0.35 GB) are too, so no L2 flush is
needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Arms:
  ours       mixed precision engine (FP32 element math, FP64-class accumulation), device
             resident inputs -> `value`; the same through the C ABI with pinned HOST buffers
             (device->host copy of nzval and f inside the timed region) -> `e2e`; the plain
             FP64 GPU form of the same engine -> `fp64_gpu`; the CPU oracle (a restatement of
             Ferrite's colored threaded assembly) on a slab of the grid -> `cpu_baseline`.
  reference  the CPU restatement of Ferrite's threaded colored assembly on all host cores,
             per step a slab of the same grid (Ferrite itself needs Julia, absent here).
"""
import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
NEL = (128, 128, 128)
SEED = 20261203
E_MOD, NU, BODY = 200e3, 0.3, (0.0, 0.0, -1.0)
METRIC = "K+f assembly Melem/s (3D Q1 hex elasticity, mixed FP32/FP64-accumulate)"
WORKLOAD = "hex128_q1_elasticity"
PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "tile_kernel_hex8_q1_elastic.md")


def _package():
    if "ferrite_gb300" in sys.modules:
        return sys.modules["ferrite_gb300"]
    path = os.path.join(ROOT, "ferrite.jl_gb300", "__init__.py")
    spec = importlib.util.spec_from_file_location("ferrite_gb300", path,
                                                  submodule_search_locations=[os.path.dirname(path)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["ferrite_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def _oracle():
    """The CPU restatement of Ferrite's assembly (CPU baseline only)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    return oracle


def algorithmic_bytes(nnz, ndofs, n_nodes, n_cells):
    """Compulsory traffic of one assembly: nzval and f written once (FP64), node coordinates
    read once (3 x FP64), 8 node ids per cell read once (int32)."""
    return 8 * nnz + 8 * ndofs + 24 * n_nodes + 4 * 8 * n_cells


class ClockSampler:
    """nvidia-smi SM clock / throttle-reason samples while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.samples = []
        self.dev = str(device_index)
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", self.dev, f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([v.strip() for v in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.05)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "n_samples": 0}
        sm = [float(s[0]) for s in self.samples if s[0] not in ("", "[N/A]")]
        mx = [float(s[1]) for s in self.samples if s[1] not in ("", "[N/A]")]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 3 + k and "Active" in s[3 + k]
                          and "Not" not in s[3 + k]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "n_samples": len(self.samples)}


def read_profile_traffic():
    """DRAM bytes per launch of the tile kernel from the committed ncu summary, if any."""
    try:
        for line in open(PROFILE_SUMMARY):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1].split()[0])
    except OSError:
        pass
    return None


def setup_problem(fg, nel=NEL):
    host = __import__("ferrite_gb300.host", fromlist=["host"])
    t0 = time.perf_counter()
    g = host.generate_grid(host.HEXAHEDRON, nel, (0, 0, 0), (1, 1, 1))
    g = host.perturb_interior(g, nel, 0.2, SEED, (0, 0, 0), (1, 1, 1))
    dh = host.DofHandler.from_grid(g, ip_order=1, n_components=3).close()
    colptr, rowval = dh.allocate_matrix()
    cv = host.CellValues(host.HEXAHEDRON, ip_order=1, qr_order=2)
    t1 = time.perf_counter()
    h = dh.handle([cv], colptr, rowval)
    t2 = time.perf_counter()
    return dict(grid=g, dh=dh, colptr=colptr, rowval=rowval, handle=h, setup_s=t1 - t0, create_s=t2 - t1)


def cpu_rate(O, nslab, nthreads, repeats=1):
    """Melem/s of the oracle's colored threaded assembly on a 128x128xnslab slab."""
    prob = O.box_problem(O.HEXAHEDRON, (NEL[0], NEL[1], nslab), [0, 0, 0], [1, 1, nslab / NEL[2]], ip_order=1,
                         ncomp=3, qr_order=2, perturb=0.2, seed=SEED)
    nz = np.zeros(prob.nnz)
    f = np.zeros(prob.ndofs)
    times = []
    for _ in range(repeats):
        t = time.perf_counter()
        prob.assemble(O.LINEAR_ELASTIC, E_MOD, NU, body=list(BODY), nthreads=nthreads, nzval=nz, f=f)
        times.append(time.perf_counter() - t)
    return prob.n_cells, times


def run_reference(args):
    """--impl reference: the CPU restatement of Ferrite's threaded colored assembly."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    O = _oracle()
    cores = os.cpu_count() or 1
    # size the per-step slab so warmup + steps take about a minute
    n0, t0 = cpu_rate(O, 2, cores)
    rate = n0 / t0[0]
    per_step = 60.0 / max(1, args.steps + args.warmup)
    nslab = int(max(1, min(NEL[2], round(per_step * rate / (NEL[0] * NEL[1])))))
    prob = O.box_problem(O.HEXAHEDRON, (NEL[0], NEL[1], nslab), [0, 0, 0], [1, 1, nslab / NEL[2]], ip_order=1,
                         ncomp=3, qr_order=2, perturb=0.2, seed=SEED)
    nz, f = np.zeros(prob.nnz), np.zeros(prob.ndofs)
    for _ in range(args.warmup):
        prob.assemble(O.LINEAR_ELASTIC, E_MOD, NU, body=list(BODY), nthreads=cores, nzval=nz, f=f)
    t = time.perf_counter()
    for _ in range(args.steps):
        prob.assemble(O.LINEAR_ELASTIC, E_MOD, NU, body=list(BODY), nthreads=cores, nzval=nz, f=f)
    dt = time.perf_counter() - t
    value = prob.n_cells * args.steps / dt / 1e6
    sample = f"128x128x{nslab} slab of the 128^3 grid ({prob.n_cells} cells) per step"
    line = {"metric": METRIC, "value": value, "unit": "Melem/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": 2097152, "ndofs": 6440067, "nnz": 513599625,
                       "sample_cells_per_step": prob.n_cells},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "Melem/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "Melem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "C++ FP64 restatement of Ferrite's colored threaded CPU assembly (Julia is not installed)"}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    fg = _package()
    fg.build()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    P = setup_problem(fg, NEL)
    h, dh = P["handle"], P["dh"]
    info = h.info()
    n_cells, ndofs, nnz = dh.n_cells, dh.ndofs, h.nnz
    n_nodes = P["grid"].nodes.shape[0]
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    nz = torch.empty(nnz, dtype=torch.float64, device=dev)
    f = torch.empty(ndofs, dtype=torch.float64, device=dev)
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=E_MOD, p1=NU, body=BODY, stream=stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- warmup + timed loop (device-resident inputs, mixed precision) ----
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            h.assemble(nz, f, sync=False, **kw)
        h.sync()
        h.kernel_time()
        barrier()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            time.sleep(0.3)
            start.record(stream)
            for _ in range(args.steps):
                h.assemble(nz, f, sync=False, profile=True, **kw)
            end.record(stream)
            h.sync()
            barrier()
        total_ms = start.elapsed_time(end)
        kern_ms, kern_n = h.kernel_time()
    ms = total_ms / args.steps
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n_cells / (ms * 1e-3) / 1e6
    kernel_ms = kern_ms / max(kern_n, 1)

    # ---- correctness at full size: rigid-body modes annihilated, body force integrates to -1 ----
    checks = {}
    if rank == 0:
        import scipy.sparse as sp
        nzh = nz.cpu().numpy()
        fh = f.cpu().numpy()
        K = sp.csc_matrix((nzh, P["rowval"] - 1, P["colptr"] - 1), shape=(ndofs, ndofs))
        x = P["grid"].nodes
        ent = (dh.cell_dofs.reshape(-1, 8, 3)[:, :, 0] - 1) // 3
        node_of_ent = np.empty(ndofs // 3, np.int64)
        node_of_ent[ent.reshape(-1)] = P["grid"].cells.reshape(-1) - 1
        worst = 0.0
        for mode in range(6):
            u = np.zeros((ndofs // 3, 3))
            if mode < 3:
                u[:, mode] = 1.0
            else:
                u[:] = np.cross(np.eye(3)[mode - 3], x[node_of_ent])
            r = K @ u.reshape(-1)
            worst = max(worst, float(np.abs(r).max() / (np.abs(nzh).max() * np.abs(u).max())))
        checks = {"rigid_body_residual_rel": worst, "sum_f_z": float(fh[2::3].sum()),
                  "finite": bool(np.isfinite(nzh).all() and np.isfinite(fh).all())}
        del K, nzh, fh

    # ---- plain FP64 GPU form of the same engine ----
    fp64 = None
    if rank == 0 and not args.skip_fp64:
        k64 = max(1, min(args.steps, 10))
        with torch.cuda.stream(stream):
            h.assemble(nz, f, precision=fg.PREC_FP64, **kw)
            h.kernel_time()
            torch.cuda.synchronize()
            s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s2.record(stream)
            for _ in range(k64):
                h.assemble(nz, f, precision=fg.PREC_FP64, sync=False, profile=True, **kw)
            e2.record(stream)
            h.sync()
            torch.cuda.synchronize()
        ms64 = s2.elapsed_time(e2) / k64
        fp64 = {"value": n_cells / (ms64 * 1e-3) / 1e6, "unit": "Melem/s", "ms_per_step": ms64, "steps": k64,
                "speedup_mixed_over_fp64": ms64 / ms}
        h.kernel_time()

    # ---- e2e: public API with pinned host buffers (D2H of nzval and f each step) ----
    e2e = None
    if rank == 0 and not args.skip_e2e:
        nz_h = torch.empty(nnz, dtype=torch.float64, pin_memory=True).numpy()
        f_h = torch.empty(ndofs, dtype=torch.float64, pin_memory=True).numpy()
        ke = max(3, min(args.steps, 10))
        h.assemble(nz_h, f_h, physics=fg.LINEAR_ELASTIC, p0=E_MOD, p1=NU, body=BODY, stream=stream)
        t = time.perf_counter()
        for _ in range(ke):
            h.assemble(nz_h, f_h, physics=fg.LINEAR_ELASTIC, p0=E_MOD, p1=NU, body=BODY, stream=stream)
        dt = (time.perf_counter() - t) / ke
        e2e = {"value": n_cells / dt / 1e6, "unit": "Melem/s", "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": 8 * nnz + 8 * ndofs, "ms_per_step": dt * 1e3, "steps": ke,
               "note": "fe_assemble with pinned host nzval/f; per-step inputs are scalars (grid, dofs and "
                       "pattern stay resident from fe_create)"}

    # ---- CPU baseline: the oracle's colored threaded assembly on a slab ----
    cpu = None
    if rank == 0 and not args.skip_cpu:
        O = _oracle()
        cores = os.cpu_count() or 1
        ncell, times = cpu_rate(O, 16, cores, repeats=3)
        cpu = {"value": ncell / statistics.median(times) / 1e6, "unit": "Melem/s", "cores": cores, "kind": "port",
               "sample": f"128x128x16 slab ({ncell} cells) of the 128^3 grid, median of 3, colored OpenMP"}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    balg = algorithmic_bytes(nnz, ndofs, n_nodes, n_cells)
    achieved = balg / (kernel_ms * 1e-3) / 1e9
    traffic = read_profile_traffic()
    line = {"metric": METRIC, "value": value, "unit": "Melem/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64acc", "data": "synthetic",
            "config": {"workload": WORKLOAD, "nel": list(NEL), "cells": n_cells, "ndofs": ndofs, "nnz": nnz, "seed": SEED,
                       "perturbation": "interior nodes +-0.2h uniform", "E": E_MOD, "nu": NU, "body": BODY,
                       "l2": "inputs (~0.35 GB) and outputs (4.1 GB) larger than L2; no flush",
                       "parallelism": "replicas" if world > 1 else "single-gpu",
                       "tiles": info["n_tiles"], "cell_visits_per_cell": info["n_cell_visits"] / n_cells},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "algorithmic_bytes": balg, "kernel_ms": kernel_ms,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy)" if peaks else "fallback"},
            "clocks": clk.summary(), "gpu_launches": args.steps, "e2e": e2e, "fp64_gpu": fp64,
            "cpu_baseline": cpu, "checks": checks,
            "setup_s": {"host_setup": P["setup_s"], "fe_create": P["create_s"]}}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--nel", type=int, default=128, help="cells per axis (128 = the benchmark workload)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    global NEL, WORKLOAD
    NEL = (args.nel,) * 3
    if args.nel != 128:
        WORKLOAD = f"hex{args.nel}_q1_elasticity"
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
