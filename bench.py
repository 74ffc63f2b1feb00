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
# accumulation of the timed mixed-precision form: "compensated" (TwoSum FP32 pairs per entry,
# FP64-class, rounded exactly to FP64) or "plain_fp32" (one FP32 sum per entry)
DEFAULT_ACCUMULATION = "compensated"
DTYPE = {"compensated": "f32 element math, FP64-class accumulation (compensated FP32 pairs, exact FP64 rounding)",
         "plain_fp32": "f32 element math, FP32 sums per entry (exact FP64 rounding)"}
PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "tile_kernel_hex8_q1_elastic.md")
Q2_PROFILE = os.path.join(ROOT, "profiles", "q2_two_phase_hex64.md")


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


def read_profile_value(path, key):
    """A `key: value` line of a committed ncu summary (None when absent)."""
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":")[1].split()[0])
    except (OSError, ValueError):
        pass
    return None


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


def oracle_view(O, dh, colptr, rowval, qr_orders):
    """The oracle's Problem over the product's own host arrays (grid, cell_dofs, colptr /
    rowval), which the CPU tests check bit for bit against the oracle's set-up; qr_orders per
    SubDofHandler."""
    n = dh.n_cells
    types = np.zeros(n, np.int32)
    npc = np.zeros(n, np.int64)
    for s in dh.subs:
        types[s["cellset"] - 1] = s["cell_type"]
        npc[s["cellset"] - 1] = s["cell_nodes"].shape[1]
    off = np.zeros(n + 1, np.int64)
    off[1:] = np.cumsum(npc)
    cn = np.zeros(int(off[-1]), np.int64)
    for s in dh.subs:
        k = s["cell_nodes"].shape[1]
        cn[(off[s["cellset"] - 1][:, None] + np.arange(k)[None, :]).ravel()] = s["cell_nodes"].ravel()
    subs = [O.Subdomain(s["cellset"], s["ip_order"], s["n_components"], q) for s, q in zip(dh.subs, qr_orders)]
    prob = O.Problem(dh.nodes, types, off, cn, subs)
    prob.cell_dofs, prob.cell_dofs_offset, prob.ndofs = dh.cell_dofs, dh.cell_dofs_offset, dh.ndofs
    prob.colptr, prob.rowval = colptr, rowval
    return prob


def rel_fro_np(a, b, chunk=1 << 26):
    """|a - b| / |b| over host vectors, in chunks (no full-size temporaries)."""
    num = den = 0.0
    for k in range(0, len(b), chunk):
        d = a[k:k + chunk] - b[k:k + chunk]
        num += float(np.dot(d, d))
        den += float(np.dot(b[k:k + chunk], b[k:k + chunk]))
    return (num ** 0.5) / (den ** 0.5 if den > 0 else 1.0)


def oracle_parity(O, prob, dev_nz, dev_f, nthreads, **phys):
    """Relative Frobenius error of the engine's K and f (device tensors) against the oracle's
    FP64 threaded assembly of the same problem (outside every timed region)."""
    t = time.perf_counter()
    T = prob.threaded(nthreads)
    nz_o, f_o = T.assemble(**phys)
    T.close()
    cpu_s = time.perf_counter() - t
    out = {"K": rel_fro_np(dev_nz.cpu().numpy(), nz_o), "f": rel_fro_np(dev_f.cpu().numpy(), f_o),
           "oracle_s": cpu_s, "oracle_threads": nthreads,
           "oracle": "FP64 C++ restatement of Ferrite's threaded colored assembly (WorkStream coloring)"}
    del nz_o, f_o
    return out


def slab_problem(O, nslab):
    return O.box_problem(O.HEXAHEDRON, (NEL[0], NEL[1], nslab), [0, 0, 0], [1, 1, nslab / NEL[2]], ip_order=1,
                         ncomp=3, qr_order=2, perturb=0.2, seed=SEED)


def cpu_rate(O, nslab, nthreads, repeats=1):
    """Melem/s of the oracle's threaded colored assembly on a 128x128xnslab slab: the
    CellValues and the WorkStream coloring are built once (threaded_assembly.jl:134-141); each
    timed call is one assemble_global! (start_assemble + the colored loop, 232-265)."""
    prob = slab_problem(O, nslab)
    T = prob.threaded(nthreads)
    nz = np.zeros(prob.nnz)
    f = np.zeros(prob.ndofs)
    times = []
    for _ in range(repeats):
        t = time.perf_counter()
        T.assemble(O.LINEAR_ELASTIC, E_MOD, NU, body=list(BODY), nzval=nz, f=f)
        times.append(time.perf_counter() - t)
    info = {"n_colors": T.n_colors, "coloring_setup_s": T.setup_s}
    T.close()
    return prob.n_cells, times, info


def run_reference(args):
    """--impl reference: the CPU restatement of Ferrite's threaded colored assembly."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    O = _oracle()
    cores = os.cpu_count() or 1
    # size the per-step slab so warmup + steps take about a minute
    n0, t0, _ = cpu_rate(O, 2, cores)
    rate = n0 / t0[0]
    per_step = 60.0 / max(1, args.steps + args.warmup)
    nslab = int(max(1, min(NEL[2], round(per_step * rate / (NEL[0] * NEL[1])))))
    prob = slab_problem(O, nslab)
    T = prob.threaded(cores)
    nz, f = np.zeros(prob.nnz), np.zeros(prob.ndofs)
    for _ in range(args.warmup):
        T.assemble(O.LINEAR_ELASTIC, E_MOD, NU, body=list(BODY), nzval=nz, f=f)
    t = time.perf_counter()
    for _ in range(args.steps):
        T.assemble(O.LINEAR_ELASTIC, E_MOD, NU, body=list(BODY), nzval=nz, f=f)
    dt = time.perf_counter() - t
    value = prob.n_cells * args.steps / dt / 1e6
    sample = (f"128x128x{nslab} slab of the 128^3 grid ({prob.n_cells} cells) per step; WorkStream coloring "
              f"({T.n_colors} colors) and CellValues built once at set-up, not timed; each step = start_assemble + "
              f"the colored loop on {cores} threads")
    T.close()
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


def dist_setup(world: int):
    """Replicas only: one process per GPU, NCCL between them (gloo when CUDA is absent, e.g.
    the CPU tests of this logic); nothing but the timing crosses ranks."""
    if world > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")


def max_over_ranks(ms: float, world: int, device=None) -> float:
    """The step time of the slowest rank (all ranks receive it)."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(world: int, cells_per_rank: int, ms: float) -> float:
    """Whole-job throughput in Melem/s: every rank assembles its own copy of the workload."""
    return world * cells_per_rank / (ms * 1e-3) / 1e6


def run_ours(args):
    import torch

    fg = _package()
    fg.build()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist_setup(world)
    P = setup_problem(fg, NEL)
    h, dh = P["handle"], P["dh"]
    info = h.info()
    n_cells, ndofs, nnz = dh.n_cells, dh.ndofs, h.nnz
    n_nodes = P["grid"].nodes.shape[0]
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    nz = torch.empty(nnz, dtype=torch.float64, device=dev)
    f = torch.empty(ndofs, dtype=torch.float64, device=dev)
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=E_MOD, p1=NU, body=BODY, stream=stream,
              compensated=DEFAULT_ACCUMULATION == "compensated")

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
    ms = max_over_ranks(total_ms / args.steps, world, dev)
    value = replica_value(world, n_cells, ms)
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

    # ---- parity at full size: the oracle's FP64 threaded assembly of the same 128^3 problem,
    # against the default (timed) result and the plain-FP32-sum form ----
    parity = None
    accumulation = None
    if rank == 0 and not args.skip_oracle:
        O = _oracle()
        prob_o = oracle_view(O, dh, P["colptr"], P["rowval"], [2])
        t0 = time.perf_counter()
        T = prob_o.threaded(os.cpu_count() or 1)
        nz_o, f_o = T.assemble(O.LINEAR_ELASTIC, E_MOD, NU, body=list(BODY))
        T.close()
        oracle_s = time.perf_counter() - t0
        parity = {"oracle_rel_frobenius": {"K": rel_fro_np(nz.cpu().numpy(), nz_o), "f": rel_fro_np(f.cpu().numpy(), f_o)},
                  "oracle_s": oracle_s, "oracle_threads": os.cpu_count(),
                  "oracle": "FP64 C++ restatement of Ferrite's threaded colored assembly, full 128^3 grid",
                  "accumulation": DEFAULT_ACCUMULATION}
        # the other accumulation: its time and its error against the same oracle result
        other = "plain_fp32" if DEFAULT_ACCUMULATION == "compensated" else "compensated"
        with torch.cuda.stream(stream):
            kw_other = dict(kw, compensated=(other == "compensated"))
            ms_other = _timed(stream, lambda: h.assemble(nz, f, sync=False, **kw_other), max(3, min(args.steps, 10)))
            h.sync()
        accumulation = {"default": DEFAULT_ACCUMULATION, "default_ms": ms, other + "_ms": ms_other,
                        other + "_oracle_rel_frobenius": {"K": rel_fro_np(nz.cpu().numpy(), nz_o),
                                                          "f": rel_fro_np(f.cpu().numpy(), f_o)},
                        "what": "compensated = TwoSum pairs of FP32 per nzval/f entry (FP64-class), rounded exactly "
                                "to FP64; plain_fp32 = one FP32 sum per entry, rounded exactly to FP64"}
        del nz_o, f_o, T
        h.assemble(nz, f, **kw)  # the default result again (the legs below reuse nz / f)

    # ---- plain FP64 GPU form of the same engine ----
    fp64 = None
    if rank == 0 and not args.skip_fp64:
        k64 = max(1, min(args.steps, 10))
        with torch.cuda.stream(stream):
            h.assemble(nz, f, **kw)  # the mixed result, against the FP64 one below
            nz_mixed, f_mixed = nz.clone(), f.clone()
            h.assemble(nz, f, precision=fg.PREC_FP64, **kw)
            err = {"K": rel_fro_t(nz_mixed, nz), "f": rel_fro_t(f_mixed, f)}
            del nz_mixed, f_mixed
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
                "speedup_mixed_over_fp64": ms64 / ms, "mixed_vs_fp64_rel_frobenius": err,
                "note": "the FP64 form equals the CPU oracle (FP64 restatement of Ferrite's assembly) to 1e-12 "
                        "in the parity tests, so this is the mixed form's error against it"}
        h.kernel_time()

    # ---- e2e: public API with pinned host buffers (D2H of nzval and f each step) ----
    e2e = None
    if rank == 0 and not args.skip_e2e:
        nz_h = torch.empty(nnz, dtype=torch.float64, pin_memory=True).numpy()
        f_h = torch.empty(ndofs, dtype=torch.float64, pin_memory=True).numpy()
        ke = max(3, min(args.steps, 10))

        def host_rate(staged):
            akw = dict(physics=fg.LINEAR_ELASTIC, p0=E_MOD, p1=NU, body=BODY, stream=stream, staged_output=staged)
            h.assemble(nz_h, f_h, **akw)
            t = time.perf_counter()
            for _ in range(ke):
                h.assemble(nz_h, f_h, **akw)
            return (time.perf_counter() - t) / ke

        paths = {"mapped": host_rate(False)}
        try:  # the copy-engine path for the same page-locked buffers
            paths["staged"] = host_rate(True)
        except Exception as exc:
            paths["staged_error"] = f"{type(exc).__name__}: {exc}"
        best = min((k for k in ("mapped", "staged") if k in paths), key=lambda k: paths[k])
        dt = paths[best]
        # the host link's own ceiling: one plain device -> pinned host copy of the same bytes
        d2h_bytes = 8 * nnz + 8 * ndofs
        src = torch.empty(d2h_bytes // 8, dtype=torch.float64, device="cuda")
        dst = torch.empty(d2h_bytes // 8, dtype=torch.float64, pin_memory=True)
        link = []
        for _ in range(3):
            torch.cuda.synchronize()
            t = time.perf_counter()
            dst.copy_(src, non_blocking=True)
            torch.cuda.synchronize()
            link.append(time.perf_counter() - t)
        link_gbs = d2h_bytes / min(link) / 1e9
        del src, dst
        e2e = {"value": n_cells / dt / 1e6, "unit": "Melem/s", "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": d2h_bytes, "ms_per_step": dt * 1e3, "steps": ke, "path": best,
               "ms_per_step_by_path": {k: v * 1e3 if isinstance(v, float) else v for k, v in paths.items()},
               "achieved_link_GBs": d2h_bytes / dt / 1e9, "link_copy_peak_GBs": link_gbs,
               "link_frac": d2h_bytes / dt / 1e9 / link_gbs,
               "note": "fe_assemble with pinned host nzval/f, host wall time per call including the device->host "
                       "transfer; paths: 'mapped' = the kernels store through the host mapping, 'staged' = "
                       "FE_STAGED_OUTPUT (device buffer, then the copy engine); per-step inputs are scalars "
                       "(grid, dofs and pattern stay resident from fe_create); link_copy_peak_GBs = one plain "
                       "device-to-pinned-host copy of the same bytes (the host link's ceiling for this transfer)"}

    # ---- the other configurations: heat 100^2, Q2 hex 64^3, SIMP adjoint, mixed-cell Neo-Hooke graph ----
    configs = None
    if rank == 0 and not args.skip_configs:
        configs = {}
        try:
            configs["apply"] = config_apply(fg, stream, P, nz, f, kw)
        except Exception as exc:
            configs["apply"] = {"error": f"{type(exc).__name__}: {exc}"}
        for name, fn in (("heat", config_heat), ("q2", config_q2), ("adjoint", config_adjoint),
                         ("mixed_graph", config_mixed_graph), ("elements", config_elements),
                         ("pattern", config_pattern)):
            try:
                configs[name] = fn(fg, stream)
            except Exception as exc:  # reported, not fatal: the headline line still prints
                configs[name] = {"error": f"{type(exc).__name__}: {exc}"}
            torch.cuda.empty_cache()

    # ---- CPU baseline: the oracle's colored threaded assembly on a slab ----
    cpu = None
    if rank == 0 and not args.skip_cpu:
        O = _oracle()
        cores = os.cpu_count() or 1
        ncell, times, cinfo = cpu_rate(O, 16, cores, repeats=5)
        cpu = {"value": ncell / statistics.median(times) / 1e6, "unit": "Melem/s", "cores": cores, "kind": "port",
               "sample": f"128x128x16 slab ({ncell} cells) of the 128^3 grid, median of 5; WorkStream coloring "
                         f"({cinfo['n_colors']} colors) and CellValues built once at set-up (not timed); each call = "
                         f"start_assemble + the colored loop on {cores} OpenMP threads"}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = hbm_peak_gbs()
    balg = algorithmic_bytes(nnz, ndofs, n_nodes, n_cells)
    achieved = balg / (kernel_ms * 1e-3) / 1e9
    traffic = read_profile_traffic()
    line = {"metric": METRIC, "value": value, "unit": "Melem/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPE[DEFAULT_ACCUMULATION], "data": "synthetic",
            "config": {"workload": WORKLOAD, "nel": list(NEL), "cells": n_cells, "ndofs": ndofs, "nnz": nnz, "seed": SEED,
                       "perturbation": "interior nodes +-0.2h uniform", "E": E_MOD, "nu": NU, "body": BODY,
                       "l2": f"outputs ({8 * (nnz + ndofs) / 1e9:.2f} GB) and inputs larger than the 129 MB L2; no flush",
                       "parallelism": "replicas" if world > 1 else "single-gpu",
                       "tiles": info["n_tiles"], "cell_visits_per_cell": info["n_cell_visits"] / n_cells},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "frac_of_nominal": achieved / NOMINAL_HBM_GBS, "nominal_peak": NOMINAL_HBM_GBS,
                         "traffic": traffic, "algorithmic_bytes": balg, "kernel_ms": kernel_ms,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy)" if peaks else "fallback"},
            "clocks": clk.summary(), "gpu_launches": args.steps, "e2e": e2e, "fp64_gpu": fp64,
            "cpu_baseline": cpu, "checks": checks, "parity": parity, "accumulation": accumulation, "configs": configs,
            "setup_s": {"host_setup": P["setup_s"], "fe_create": P["create_s"]}}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def rel_fro_t(a, b) -> float:
    """relative Frobenius norm |a - b| / |b| of two device vectors"""
    import torch
    nb = float(torch.linalg.vector_norm(b))
    return float(torch.linalg.vector_norm(a - b)) / (nb if nb > 0 else 1.0)


NOMINAL_HBM_GBS = 7900.0  # GB300 HBM3e, nominal (the roofline's denominator is the measured copy rate)


def hbm_peak_gbs():
    """Measured copy bandwidth of this GPU model (MEASURED_PEAKS.json), else 6800 GB/s."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(path)).get("hbm_gbs", 6800.0) if os.path.exists(path) else 6800.0


def _timed(stream, fn, reps, warmup=2):
    """CUDA-event time of fn() per call on `stream` (fn enqueues asynchronously)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def config_apply(fg, stream, P, nz, f, kw, reps=20):
    """Dirichlet apply! on the assembled 128^3 system: x = 0 face clamped (all components),
    u_z = -0.01 on the z = 1 face; device fe_apply after a fresh assembly, against the oracle's
    apply! (the reference's serial algorithm) on the host copy of the same K and f."""
    import torch
    O = _oracle()
    h, dh, g = P["handle"], P["dh"], P["grid"]
    x = g.nodes
    nodes = np.arange(x.shape[0])
    # vertex dofs of node n: the first visit numbering of a Q1 field is not node order, so
    # read them from the cells (cell k, local node a -> dofs 3 a .. 3 a + 2)
    cn = g.cells - 1
    cd = dh.cell_dofs.reshape(-1, 24) - 1
    n2d = np.full((x.shape[0], 3), -1, np.int64)
    n2d[cn.ravel()] = cd.reshape(-1, 8, 3).reshape(-1, 3)
    clamp = nodes[np.abs(x[:, 0]) < 1e-12]
    top = nodes[np.abs(x[:, 2] - 1) < 1e-12]
    gmap = dict(zip(n2d[top][:, 2].tolist(), [-0.01] * len(top)))
    gmap.update(dict.fromkeys(n2d[clamp].ravel().tolist(), 0.0))  # the clamp wins on the shared edge
    pd = np.array(sorted(gmap), np.int64)
    gv = np.array([gmap[d] for d in pd.tolist()])
    pd1 = pd + 1
    t0 = time.perf_counter()
    ch = h.dirichlet(P["rowval"], pd1)
    create_s = time.perf_counter() - t0
    gd = torch.as_tensor(gv, device="cuda")
    h.assemble(nz, f, **kw)
    torch.cuda.synchronize()
    nz_h, f_h = nz.cpu().numpy(), f.cpu().numpy()
    ms = _timed(stream, lambda: ch.apply(nz, f, gd, stream=stream, sync=False), reps)
    # one clean application on a fresh assembly for the comparison
    h.assemble(nz, f, **kw)
    ch.apply(nz, f, gd, stream=stream)
    prob = O.Problem.__new__(O.Problem)
    prob.colptr, prob.rowval, prob.ndofs = P["colptr"], P["rowval"], dh.ndofs
    t0 = time.perf_counter()
    prob.apply(nz_h, f_h, pd1, gv)
    cpu_s = time.perf_counter() - t0
    d_nz, d_f = nz.cpu().numpy(), f.cpu().numpy()
    out = {"workload": "hex128_q1_elasticity_dirichlet", "prescribed": int(len(pd1)), "apply_ms": ms,
           "create_s": create_s, "cpu_reference_apply_s": cpu_s, "cpu_threads": 1,
           "max_abs_diff_vs_cpu": {"nzval": float(np.abs(d_nz - nz_h).max()), "f": float(np.abs(d_f - f_h).max())},
           "note": "fe_apply touches the prescribed columns, rows and diagonals only; the CPU reference "
                   "(oracle restatement of ConstraintHandler.jl apply!) also scans every rowval entry"}
    ch.close()
    # facet loads on the same system: pressure on the x = 1 face (local facet 3 of the cells
    # with i = n-1), a traction on the z = 1 face (facet 6 of the cells with k = n-1)
    n = NEL[0]
    ids = np.arange(n ** 3, dtype=np.int64)
    i, k = ids % n, ids // (n * n)
    cells = np.concatenate([ids[i == n - 1], ids[k == n - 1]]) + 1
    facets = np.concatenate([np.full(n * n, 3, np.int32), np.full(n * n, 6, np.int32)])
    fs = h.facet_set(cells, facets, host_module().facet_values(host_module().HEXAHEDRON, 1, 2))
    f.zero_()
    fs.load(f, pressure=-1.0, traction=(0.0, 0.0, -0.5), stream=stream)
    t0 = time.perf_counter()
    for _ in range(reps):
        fs.load(f, pressure=-1.0, traction=(0.0, 0.0, -0.5), stream=stream)
    out["facet_load"] = {"facets": int(len(cells)), "ms": (time.perf_counter() - t0) * 1e3 / reps,
                         "note": "fe_assemble_facet_load, synchronous (host wall time per call)"}
    fs.close()
    return out


def host_module():
    return __import__("ferrite_gb300.host", fromlist=["host"])


def config_heat(fg, stream):
    """2D Poisson as in the heat tutorial: Quadrilateral 100x100 on [-1,1]^2, k = 1, source 1."""
    import torch
    host = __import__("ferrite_gb300.host", fromlist=["host"])
    g = host.generate_grid(host.QUADRILATERAL, (100, 100), (-1, -1), (1, 1))
    dh = host.DofHandler.from_grid(g, ip_order=1, n_components=1).close()
    colptr, rowval = dh.allocate_matrix()
    h = dh.handle([host.CellValues(host.QUADRILATERAL, 1, 2)], colptr, rowval)
    nz = torch.empty(h.nnz, dtype=torch.float64, device="cuda")
    f = torch.empty(dh.ndofs, dtype=torch.float64, device="cuda")
    out = {"workload": "heat_quad100x100", "cells": dh.n_cells, "ndofs": dh.ndofs, "nnz": h.nnz}
    res = {}
    for name, prec in (("mixed", fg.PREC_MIXED), ("fp64", fg.PREC_FP64)):
        ms = _timed(stream, lambda: h.assemble(nz, f, physics=fg.HEAT, p0=1.0, p1=1.0, precision=prec, stream=stream,
                                               sync=False), 200)
        h.sync()
        out[name] = {"us_per_assembly": ms * 1e3, "Melem_s": dh.n_cells / (ms * 1e-3) / 1e6}
        res[name] = (nz.clone(), f.clone())
    out["mixed_vs_fp64_rel_frobenius"] = {"K": rel_fro_t(res["mixed"][0], res["fp64"][0]),
                                          "f": rel_fro_t(res["mixed"][1], res["fp64"][1])}
    out["note"] = "launch-bound (10,000 cells); one kernel launch per assembly"
    h.close()
    return out


# FLOPs of the adjoint per Q1 hexahedron, counted from the formula per quadrature point (8
# points): Jacobian (7 node offsets x 9 FMA = 126 flops), adjugate and determinant (~45),
# gradient table dN/dx (8 x 9 FMA = 144), grad u and grad lambda (2 x 8 x 9 FMA = 288), the
# two stresses (2 x ~15), psi (18), Sigma (2 x 27 FMA = 108) and dPhi/dx_k (8 x 9 FMA = 144),
# plus the load density (~30): ~935 per point
ADJ_FLOPS_PER_CELL = 8 * 935


def ADJ_BYTES(n_cells, n_nodes, ndofs):
    """compulsory bytes of one adjoint: coordinates, connectivity, rho, u, lambda read; d_rho,
    d_X written (FP64, int32 ids)"""
    return 24 * n_nodes + 32 * n_cells + 8 * n_cells + 16 * ndofs + 8 * n_cells + 24 * n_nodes


def adjoint_fd_check(dh, colptr, rowval, rho, u, lam, adj, h=1e-6, ndir=3):
    """Central finite differences (step h) of Phi = lambda^T (K(X, rho^3) u - f(X)) from the
    oracle's FP64 threaded assembly, along `ndir` seeded random directions in rho and in X,
    against the engine's adjoint (mixed and FP64) projected on the same directions. The
    difference Phi(+) - Phi(-) is taken entry-wise (K+ - K-, f+ - f-) before the products, so
    cancellation stays at the entry level."""
    import scipy.sparse as sp
    O = _oracle()
    prob = oracle_view(O, dh, colptr, rowval, [2])
    prob.nodes = dh.nodes.copy()
    X0 = prob.nodes.copy()
    T = prob.threaded(os.cpu_count() or 1)
    rng = np.random.default_rng(SEED + 11)
    t0 = time.perf_counter()

    def dphi(s_plus, s_minus):
        kp, fp = T.assemble(O.LINEAR_ELASTIC, 1.0, NU, body=list(BODY), cell_scale=s_plus)
        km, fm = T.assemble(O.LINEAR_ELASTIC, 1.0, NU, body=list(BODY), cell_scale=s_minus)
        dK = sp.csc_matrix((kp - km, rowval - 1, colptr - 1), shape=(dh.ndofs, dh.ndofs))
        return float(lam @ (dK @ u) - lam @ (fp - fm)) / (2 * h)

    out = {"h": h, "directions": ndir, "rho": [], "X": []}
    for _ in range(ndir):
        v = rng.standard_normal(dh.n_cells)
        fd = dphi((rho + h * v) ** 3, (rho - h * v) ** 3)
        out["rho"].append({"fd": fd, **{k: float(a[0] @ v) for k, a in adj.items()}})
    s = rho ** 3
    for _ in range(ndir):
        w = rng.standard_normal(X0.shape)
        prob.nodes[:] = X0 + h * w
        kp, fp = T.assemble(O.LINEAR_ELASTIC, 1.0, NU, body=list(BODY), cell_scale=s)
        prob.nodes[:] = X0 - h * w
        km, fm = T.assemble(O.LINEAR_ELASTIC, 1.0, NU, body=list(BODY), cell_scale=s)
        dK = sp.csc_matrix((kp - km, rowval - 1, colptr - 1), shape=(dh.ndofs, dh.ndofs))
        fd = float(lam @ (dK @ u) - lam @ (fp - fm)) / (2 * h)
        out["X"].append({"fd": fd, **{k: float(a[1] @ w.reshape(-1)) for k, a in adj.items()}})
    prob.nodes[:] = X0
    T.close()
    for key in ("rho", "X"):
        for name in adj:
            out[f"max_rel_err_{key}_{name}"] = max(abs(d[name] - d["fd"]) / abs(d["fd"]) for d in out[key])
    out["oracle_s"] = time.perf_counter() - t0
    out["what"] = ("directional derivatives d/dt Phi(rho + t v) and d/dt Phi(X + t w): FD of the oracle's FP64 "
                   "assembly vs the engine's adjoint (d_rho . v, d_X . w); mixed and fp64 = the engine's precisions")
    return out


def config_adjoint(fg, stream, oracle=True):
    """SIMP cantilever (96,48,48) on [0,2]x[0,1]^2: rho ~ U(0.01,1), E = rho^3, nu = 0.3, u and
    lambda ~ N(0, 1e-3^2); adjoint (d/d rho, d/dX) against the forward K+f assembly."""
    import torch
    host = __import__("ferrite_gb300.host", fromlist=["host"])
    nel = (96, 48, 48)
    g = host.generate_grid(host.HEXAHEDRON, nel, (0, 0, 0), (2, 1, 1))
    dh = host.DofHandler.from_grid(g, ip_order=1, n_components=3).close()
    colptr, rowval = dh.allocate_matrix()
    h = dh.handle([host.CellValues(host.HEXAHEDRON, 1, 2)], colptr, rowval)
    rng = np.random.default_rng(SEED + 4)
    rho = rng.uniform(0.01, 1.0, dh.n_cells)
    d = lambda a: torch.as_tensor(a, device="cuda")
    scale, dscale = d(rho ** 3), d(3 * rho ** 2)
    u, lam = d(rng.normal(0, 1e-3, dh.ndofs)), d(rng.normal(0, 1e-3, dh.ndofs))
    nz = torch.empty(h.nnz, dtype=torch.float64, device="cuda")
    f = torch.empty(dh.ndofs, dtype=torch.float64, device="cuda")
    d_rho = torch.empty(dh.n_cells, dtype=torch.float64, device="cuda")
    d_X = torch.empty(g.nodes.shape[0] * 3, dtype=torch.float64, device="cuda")
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=1.0, p1=NU, body=BODY, cell_scale=scale, stream=stream)
    fwd = _timed(stream, lambda: h.assemble(nz, f, sync=False, **kw), 20)
    h.sync()
    out = {"workload": "simp_cantilever_hex96x48x48", "cells": dh.n_cells, "ndofs": dh.ndofs, "forward_ms": fwd}
    res = {}
    for name, prec in (("mixed", fg.PREC_MIXED), ("fp64", fg.PREC_FP64)):
        ms = _timed(stream, lambda: h.adjoint(u, lam, d_rho, d_X, fg.LINEAR_ELASTIC, 1.0, NU, body=BODY, cell_scale=scale,
                                              dscale=dscale, precision=prec, stream=stream, sync=False), 20)
        h.sync()
        res[name] = (d_rho.clone(), d_X.clone())
        out[f"adjoint_{name}_ms"] = ms
    out["adjoint_over_forward"] = out["adjoint_mixed_ms"] / fwd
    rel = lambda a, b: float((a - b).abs().max() / b.abs().max())
    out["mixed_vs_fp64_rel_max"] = {"d_rho": rel(res["mixed"][0], res["fp64"][0]), "d_X": rel(res["mixed"][1], res["fp64"][1])}
    # work of one adjoint: FLOPs counted from the formula per quadrature point (8 per cell)
    out["roofline"] = {"bound": "fp32 issue (compute)", "flops_per_cell": ADJ_FLOPS_PER_CELL,
                       "achieved_tflops": dh.n_cells * ADJ_FLOPS_PER_CELL / (out["adjoint_mixed_ms"] * 1e-3) / 1e12,
                       "algorithmic_bytes": ADJ_BYTES(dh.n_cells, g.nodes.shape[0], dh.ndofs),
                       "achieved_GBs": ADJ_BYTES(dh.n_cells, g.nodes.shape[0], dh.ndofs) / (out["adjoint_mixed_ms"] * 1e-3) / 1e9,
                       "bar": "adjoint <= 2x one forward assembly of the same grid"}
    if oracle:
        out["fd_check"] = adjoint_fd_check(dh, colptr, rowval, rho, u.cpu().numpy(), lam.cpu().numpy(),
                                           {k: (v[0].cpu().numpy(), v[1].cpu().numpy()) for k, v in res.items()})
    out["note"] = ("forward = mixed K+f assembly with E_e = rho^3; adjoint recomputes the geometry; "
                   "finite-difference checks of the formulas are in the tests")
    h.close()
    return out


def config_q2(fg, stream, nel=64, reps=5, oracle=True):
    """Q2 hexahedra (27 nodes, 81 dofs per cell) on the perturbed unit cube, 3x3x3 Gauss,
    linear elasticity with a per-cell modulus E_e ~ lognormal(log 200e3, 0.5) (seeded), nu 0.3,
    b = (0, 0, -1). Mixed and FP64 forms timed; the mixed result against the FP64 one."""
    import torch
    host = __import__("ferrite_gb300.host", fromlist=["host"])
    n3 = (nel, nel, nel)
    t0 = time.perf_counter()
    g = host.generate_grid(host.HEXAHEDRON, n3, (0, 0, 0), (1, 1, 1))
    g = host.perturb_interior(g, n3, 0.2, SEED + 3, (0, 0, 0), (1, 1, 1))
    dh = host.DofHandler.from_grid(g, ip_order=2, n_components=3).close()
    colptr, rowval = dh.allocate_matrix()
    t1 = time.perf_counter()
    h = dh.handle([host.CellValues(host.HEXAHEDRON, 2, 3)], colptr, rowval)
    t2 = time.perf_counter()
    E = np.random.default_rng(SEED + 7).lognormal(np.log(E_MOD), 0.5, dh.n_cells)
    scale = torch.as_tensor(E / E_MOD, device="cuda")
    nz = torch.empty(h.nnz, dtype=torch.float64, device="cuda")
    f = torch.empty(dh.ndofs, dtype=torch.float64, device="cuda")
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=E_MOD, p1=NU, body=BODY, cell_scale=scale, stream=stream)
    mixed = _timed(stream, lambda: h.assemble(nz, f, sync=False, **kw), reps)
    h.sync()
    nz_m, f_m = nz.clone(), f.clone()
    fp64 = _timed(stream, lambda: h.assemble(nz, f, sync=False, precision=fg.PREC_FP64, **kw), 1, warmup=1)
    h.sync()
    rel_k = float(torch.linalg.vector_norm(nz_m - nz) / torch.linalg.vector_norm(nz))
    rel_f = float(torch.linalg.vector_norm(f_m - f) / torch.linalg.vector_norm(f))
    parity = None
    if oracle:
        O = _oracle()
        prob_o = oracle_view(O, dh, colptr, rowval, [3])
        parity = oracle_parity(O, prob_o, nz_m, f_m, os.cpu_count() or 1, physics=O.LINEAR_ELASTIC, p0=E_MOD, p1=NU,
                               body=list(BODY), cell_scale=E / E_MOD)
        del prob_o
    del nz_m, f_m, rowval
    info = h.info()
    n_nodes = g.nodes.shape[0]
    balg = 8 * h.nnz + 8 * dh.ndofs + 24 * n_nodes + 4 * 27 * dh.n_cells + 8 * dh.n_cells
    out = {"workload": f"hex{nel}_q2_elasticity", "cells": dh.n_cells, "ndofs": dh.ndofs, "nnz": h.nnz,
           "mixed": {"ms_per_assembly": mixed, "Melem_s": dh.n_cells / (mixed * 1e-3) / 1e6,
                     "achieved_GBs": balg / (mixed * 1e-3) / 1e9, "algorithmic_bytes": balg},
           "fp64": {"ms_per_assembly": fp64, "Melem_s": dh.n_cells / (fp64 * 1e-3) / 1e6},
           "speedup_mixed_over_fp64": fp64 / mixed,
           "mixed_vs_fp64_rel_frobenius": {"K": rel_k, "f": rel_f}, "oracle_parity": parity,
           "roofline": {"bound": "hbm", "achieved": balg / (mixed * 1e-3) / 1e9, "peak": hbm_peak_gbs(), "unit": "GB/s",
                        "frac": balg / (mixed * 1e-3) / 1e9 / hbm_peak_gbs(), "algorithmic_bytes": balg,
                        "tensor_pipe": read_profile_value(Q2_PROFILE, "tensor_pipe_active_pct"),
                        "tensor_pipe_source": os.path.relpath(Q2_PROFILE, ROOT)},
           "tiles": info["n_tiles"], "cell_visits_per_cell": info["n_cell_visits"] / dh.n_cells,
           "setup_s": {"host": t1 - t0, "fe_create": t2 - t1},
           "path": "two-phase: element matrices once per cell on the tensor cores (tcgen05 kind::tf32, split-TF32 "
                   "Gram products), then the gather-only owner-tile reduce"}
    h.close()
    return out


def config_elements(fg, stream, nel=64, reps=10):
    """Element assembly (fe_assemble_elements, the GPU how-to's Kes/fes) of Q1 hex elasticity
    on the perturbed unit cube: FP32 Ke per cell, per-cell contiguous (Kes[c, I, J] row-major)
    and the how-to's cell-fastest layout (Julia Kes[ncells, nbf, nbf])."""
    import torch
    host = __import__("ferrite_gb300.host", fromlist=["host"])
    n3 = (nel, nel, nel)
    g = host.generate_grid(host.HEXAHEDRON, n3, (0, 0, 0), (1, 1, 1))
    g = host.perturb_interior(g, n3, 0.2, SEED, (0, 0, 0), (1, 1, 1))
    dh = host.DofHandler.from_grid(g, ip_order=1, n_components=3).close()
    colptr, rowval = dh.allocate_matrix()
    h = dh.handle([host.CellValues(host.HEXAHEDRON, 1, 2)], colptr, rowval)
    n, nbf = dh.n_cells, 24
    ke = torch.empty((n, nbf, nbf), dtype=torch.float32, device="cuda")
    fe = torch.empty((n, nbf), dtype=torch.float32, device="cuda")
    kw = dict(physics=fg.LINEAR_ELASTIC, p0=E_MOD, p1=NU, body=BODY, stream=stream, sync=False)
    out = {"workload": f"hex{nel}_q1_elasticity_elements", "cells": n, "bytes_out": (ke.numel() + fe.numel()) * 4}
    for name, ks, fs in (("cell_major", None, None), ("cell_fastest", (1, n, n * nbf), (1, n))):
        ms = _timed(stream, lambda: h.assemble_elements(ke, fe, ke_stride=ks, fe_stride=fs, **kw), reps)
        h.sync()
        out[name] = {"ms": ms, "Melem_s": n / (ms * 1e-3) / 1e6, "write_GBs": out["bytes_out"] / (ms * 1e-3) / 1e9}
    h.assemble_elements(ke, fe, **kw)
    h.sync()
    ke64 = torch.empty((n, nbf, nbf), dtype=torch.float64, device="cuda")
    fe64 = torch.empty((n, nbf), dtype=torch.float64, device="cuda")
    h.assemble_elements(ke64, fe64, precision=fg.PREC_FP64, **kw)
    h.sync()
    out["fp32_vs_fp64_rel_frobenius"] = {"Ke": rel_fro_t(ke.double(), ke64), "fe": rel_fro_t(fe.double(), fe64)}
    out["matvec"] = matvec_leg(fg, h, stream, dh, colptr, rowval, ke, ke64, kw, reps)
    del ke64, fe64
    h.close()
    return out


def matvec_leg(fg, h, stream, dh, colptr, rowval, ke, ke64, kw, reps):
    """Matrix-free product y = sum_c A_c^T Ke_c A_c u (fe_element_matvec) with the element
    matrices just assembled (row-major Kes[c, I, J]), float and double, against y = K u of the
    assembled FP64 K as a CSR product (torch.sparse, a library SpMV; K is symmetric, so its CSC
    arrays are its CSR arrays)."""
    import torch
    n, nbf = ke.shape[0], ke.shape[1]
    rng = np.random.default_rng(SEED + 9)
    u = torch.as_tensor(rng.standard_normal(dh.ndofs), device="cuda")
    y = torch.empty(dh.ndofs, dtype=torch.float64, device="cuda")
    res = {"what": "y = sum_c A_c^T Ke_c A_c u, two kernels (per-cell products, per-dof gather in cell order); "
                   "cell_major = Kes[c, I, J] row-major (a warp per cell), cell_fastest = the how-to's "
                   "Kes[ncells, nbf, nbf] column-major (a thread per cell)"}
    ys = {}
    for name, kk, prec in (("float", ke, fg.PREC_MIXED), ("double", ke64, fg.PREC_FP64)):
        res[name] = {}
        alg = kk.numel() * kk.element_size() + 4 * 8 * n + 16 * dh.ndofs
        for layout in ("cell_major", "cell_fastest"):
            kl = kk if layout == "cell_major" else kk.permute(2, 1, 0).contiguous()
            ks = kk.stride() if layout == "cell_major" else (1, n, n * nbf)
            op = h.element_operator(ks, prec)
            ms = _timed(stream, lambda: op.matvec(kl, u, y, stream=stream, sync=False), reps)
            torch.cuda.synchronize()
            if layout == "cell_major":
                ys[name] = y.clone()
            else:
                res[name]["layouts_bitwise_equal"] = bool(torch.equal(y, ys[name]))
            res[name][layout] = {"ms": ms, "GBs": alg / (ms * 1e-3) / 1e9,
                                 "frac_of_measured_hbm": alg / (ms * 1e-3) / 1e9 / hbm_peak_gbs()}
            op.close()
            del kl
        res[name]["algorithmic_bytes"] = alg
    nz = torch.empty(h.nnz, dtype=torch.float64, device="cuda")
    f = torch.empty(dh.ndofs, dtype=torch.float64, device="cuda")
    h.assemble(nz, f, **dict(kw, precision=fg.PREC_FP64, sync=True))
    try:
        K = torch.sparse_csr_tensor(torch.as_tensor(colptr - 1, device="cuda"), torch.as_tensor(rowval - 1, device="cuda"),
                                    nz, size=(dh.ndofs, dh.ndofs))
        uc = u.unsqueeze(1)
        with torch.cuda.stream(stream):
            ms = _timed(stream, lambda: torch.sparse.mm(K, uc), reps)
            Ku = torch.sparse.mm(K, uc).squeeze(1)
        torch.cuda.synchronize()
        res["csr_spmv_fp64"] = {"ms": ms, "nnz": h.nnz}
        res["rel_error_vs_Ku"] = {k: rel_fro_t(v, Ku) for k, v in ys.items()}
        del K, Ku
    except Exception as e:  # the library SpMV is a comparison only
        res["csr_spmv_fp64"] = {"error": str(e)[:200]}
    del nz, f
    return res


def config_pattern(fg, stream, nel=128):
    """allocate_matrix(dh) for 128^3 Q1 hex elasticity (6.4M dofs, nnz 513.6M): the host
    fe_sparsity_pattern (threaded, all host cores) against fe_sparsity_pattern_device (GPU
    kernels, outputs in device memory, inputs uploaded inside the timing); identical arrays."""
    import torch
    host = __import__("ferrite_gb300.host", fromlist=["host"])
    n3 = (nel, nel, nel)
    g = host.generate_grid(host.HEXAHEDRON, n3, (0, 0, 0), (1, 1, 1))
    dh = host.DofHandler.from_grid(g, ip_order=1, n_components=3).close()
    t0 = time.perf_counter()
    cp_h, rv_h = dh.allocate_matrix()
    host_s = time.perf_counter() - t0
    dh.allocate_matrix(device=True)  # warm-up (module load, first allocations)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cp_d, rv_d = dh.allocate_matrix(device=True)
    torch.cuda.synchronize()
    dev_s = time.perf_counter() - t0
    same = bool(np.array_equal(cp_d.cpu().numpy(), cp_h) and np.array_equal(rv_d.cpu().numpy(), rv_h))
    # fe_create on either pattern: the host one reads rowval on the host; the device one keeps
    # it on the device (pattern check and rank tables by kernels); the plans must be the same
    cvs = [host.CellValues(host.HEXAHEDRON, ip_order=1, qr_order=2)]
    create = {}
    digests = []
    for name, (cp, rv) in (("host_pattern", (cp_h, rv_h)), ("device_pattern", (cp_d, rv_d))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h = dh.handle(cvs, cp, rv)
        torch.cuda.synchronize()
        create[name] = time.perf_counter() - t0
        digests.append(h.info()["plan_checksum"])
        h.close()
    out = {"workload": f"hex{nel}_q1_vector_pattern", "ndofs": dh.ndofs, "nnz": int(len(rv_h)), "host_s": host_s,
           "host_threads": os.cpu_count(), "device_s": dev_s, "identical": same,
           "fe_create_s": create, "plan_digests_equal": digests[0] == digests[1],
           "note": "device time includes the host pass over cell_dofs, the uploads and both passes "
                   "(count, then fill); the two-call protocol of fe_sparsity_pattern. fe_create_s: the handle "
                   "(validation, index map, owner-tile plan, uploads) from each pattern"}
    del rv_d, cp_d
    torch.cuda.empty_cache()
    return out


def config_mixed_graph(fg, stream, steps=20, oracle=True, ny=100, tune=True):
    """~2M cells over three x-slabs sharing vertex nodes (Hex Q1 50%, Tet P1 25% as 6 per cube,
    Wedge P1 25% as 2 per cube), compressible Neo-Hooke (mu 1, lambda 10), displacement
    amplitude 0.05 of the cell size h = 0.01 (u = 0.05 h U(-1,1), seeded per step: an absolute
    0.05 is five cells wide and inverts most cells, a state no Newton iteration of the tutorial
    visits); the tile plan autotuned, then `steps` re-assemblies with updated u captured as one
    CUDA graph and replayed."""
    import torch
    host = __import__("ferrite_gb300.host", fromlist=["host"])
    nh, nt, nw, nzc = 100, 8, 25, ny
    nx = nh + nt + nw
    box = (nx / 100.0, ny / 100.0, nzc / 100.0)  # cubes of side 0.01 (the unit-depth box at ny = 100)
    g = host.generate_grid(host.HEXAHEDRON, (nx, ny, nzc), (0, 0, 0), box)
    g = host.perturb_interior(g, (nx, ny, nzc), 0.15, SEED + 5, (0, 0, 0), box)
    cubes = g.cells  # [n, 8], 1-based, x fastest
    ix = np.arange(cubes.shape[0]) % nx
    T = np.array([[1, 2, 4, 8], [1, 5, 2, 8], [2, 3, 4, 8], [2, 7, 3, 8], [2, 5, 6, 8], [2, 6, 7, 8]]) - 1
    W = np.array([[1, 2, 4, 5, 6, 8], [2, 3, 4, 6, 7, 8]]) - 1
    hexes = cubes[ix < nh]
    tets = cubes[(ix >= nh) & (ix < nh + nt)][:, T].reshape(-1, 4)
    wedges = cubes[ix >= nh + nt][:, W].reshape(-1, 6)
    n_cells = len(hexes) + len(tets) + len(wedges)
    dh = host.DofHandler(g.nodes, n_cells)
    o = 0
    for ct, cn in ((host.HEXAHEDRON, hexes), (host.TETRAHEDRON, tets), (host.WEDGE, wedges)):
        dh.add(ct, np.ascontiguousarray(cn, np.int64), np.arange(o + 1, o + len(cn) + 1, dtype=np.int64), 1, 3)
        o += len(cn)
    dh.close()
    colptr, rowval = dh.allocate_matrix()
    cvs = [host.CellValues(host.HEXAHEDRON, 1, 2), host.CellValues(host.TETRAHEDRON, 1, 1), host.CellValues(host.WEDGE, 1, 2)]
    h = dh.handle(cvs, colptr, rowval)
    rng = np.random.default_rng(SEED + 6)
    cell_h = 0.01
    us = [torch.as_tensor(0.05 * cell_h * rng.uniform(-1, 1, dh.ndofs), device="cuda") for _ in range(steps)]
    nz = torch.empty(h.nnz, dtype=torch.float64, device="cuda")
    f = torch.empty(dh.ndofs, dtype=torch.float64, device="cuda")
    kw = dict(physics=fg.NEO_HOOKE, p0=1.0, p1=10.0, body=(0.0, 0.0, 0.0))
    if tune:
        tune = h.autotune(nz, f, stage_caps=[6144, 7168, 8192, 9216, 10240, 12288], reps=2, stream=stream, u=us[0], **kw)
    else:  # the form and tile size the tuner picks at full size (profiling runs)
        tune = h.autotune(nz, f, stage_caps=[9216], reps=1, stream=stream, u=us[0], form="two_phase", **kw)
    single = _timed(stream, lambda: h.assemble(nz, f, u=us[0], stream=stream, sync=False, **kw), 5)
    h.sync()
    gid = h.graph_capture([dict(u=u, **kw) for u in us], [nz] * steps, [f] * steps, stream)
    replay = _timed(stream, lambda: h.graph_replay(gid, stream, sync=False), 3, warmup=1)
    h.sync()
    # e2e: a Newton step as a host caller makes it, through fe_assemble with page-locked host
    # buffers -- u uploaded, K and f read back, every step
    e2e = None
    if not os.environ.get("FE_BENCH_SKIP_E2E"):
        u_h = torch.empty(dh.ndofs, dtype=torch.float64, pin_memory=True)
        nz_h = torch.empty(h.nnz, dtype=torch.float64, pin_memory=True).numpy()
        f_h = torch.empty(dh.ndofs, dtype=torch.float64, pin_memory=True).numpy()
        u_h.copy_(us[0].cpu())
        u_hn = u_h.numpy()
        h.assemble(nz_h, f_h, u=u_hn, stream=stream, **kw)
        ke = 5
        t = time.perf_counter()
        for k in range(ke):
            h.assemble(nz_h, f_h, u=u_hn, stream=stream, **kw)
        dt = (time.perf_counter() - t) / ke
        e2e = {"ms_per_step": dt * 1e3, "Melem_s": n_cells / dt / 1e6, "h2d_bytes_per_step": 8 * dh.ndofs,
               "d2h_bytes_per_step": 8 * h.nnz + 8 * dh.ndofs, "steps": ke,
               "what": "fe_assemble with u, nzval and f in page-locked host memory (host wall time per call)"}
        del nz_h, f_h, u_h
    h.assemble(nz, f, u=us[-1], stream=stream, **kw)
    nz_m, f_m = nz.clone(), f.clone()
    h.assemble(nz, f, u=us[-1], stream=stream, precision=fg.PREC_FP64, **kw)
    err = {"K": rel_fro_t(nz_m, nz), "f": rel_fro_t(f_m, f)}
    parity = None
    if oracle:
        O = _oracle()
        prob_o = oracle_view(O, dh, colptr, rowval, [2, 1, 2])
        parity = oracle_parity(O, prob_o, nz_m, f_m, os.cpu_count() or 1, physics=O.NEO_HOOKE, p0=1.0, p1=10.0,
                               body=[0.0, 0.0, 0.0], u=us[-1].cpu().numpy())
        del prob_o
    del nz_m, f_m
    info = h.info()
    n_nodes = g.nodes.shape[0]
    balg = 8 * h.nnz + 16 * dh.ndofs + 24 * n_nodes + 4 * (8 * len(hexes) + 4 * len(tets) + 6 * len(wedges))
    out = {"workload": "mixed_hex_tet_wedge_neo_hooke_2M", "cells": n_cells, "hex": len(hexes), "tet": len(tets),
           "wedge": len(wedges), "ndofs": dh.ndofs, "nnz": h.nnz, "steps_per_graph": steps,
           "graph_replay_ms": replay, "ms_per_assembly_in_graph": replay / steps,
           "Melem_s_in_graph": n_cells * steps / (replay * 1e-3) / 1e6, "ms_single_assembly": single,
           "autotune": {"best_stage_cap": tune["best_stage_cap"], "best_form_mask": tune["best_form_mask"],
                        "form_mask_bits": "bit 0 hex, bit 1 tet, bit 2 wedge subdomain in the two-phase form",
                        "candidates": [{"stage_cap": c, "ms": ms, "tiles": t, "form_mask": m}
                                       for c, ms, t, _, m in tune["candidates"]]},
           "tiles": info["n_tiles"], "cell_visits_per_cell": info["n_cell_visits"] / n_cells,
           "mixed_vs_fp64_rel_frobenius": err, "oracle_parity": parity, "e2e": e2e,
           "roofline": {"bound": "hbm", "achieved": balg / (replay / steps * 1e-3) / 1e9, "peak": hbm_peak_gbs(),
                        "unit": "GB/s", "frac": balg / (replay / steps * 1e-3) / 1e9 / hbm_peak_gbs(),
                        "algorithmic_bytes": balg,
                        "formula": "8 nnz + 8 ndofs (f written) + 8 ndofs (u read) + 24 n_nodes (coordinates) + "
                                   "4 bytes per node id per cell (8 hex, 4 tet, 6 wedge)"},
           "u": "0.05 * 0.01 * U(-1,1) per dof (amplitude 0.05 of the cell size)",
           "quadrature": "hex 2x2x2 Gauss, tet 1 point, wedge 5-point order-2 rule"}
    h.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-configs", action="store_true", help="skip the heat / Q2 / adjoint / mixed-graph configurations")
    ap.add_argument("--skip-oracle", action="store_true", help="skip the full-size FP64 oracle parity legs")
    ap.add_argument("--nel", type=int, default=128, help="cells per axis (128 = the benchmark workload)")
    ap.add_argument("--config", choices=["heat", "q2", "adjoint", "mixed_graph", "elements", "pattern"],
                    help="run only this configuration and print its JSON (profiling runs)")
    ap.add_argument("--q2-nel", type=int, default=64, help="cells per axis of the Q2 configuration")
    ap.add_argument("--mixed-ny", type=int, default=100,
                    help="cells along y and z of the mixed-cell configuration (100 = the 1.98M-cell workload)")
    ap.add_argument("--no-tune", action="store_true",
                    help="mixed-cell configuration: skip the autotuner, use its full-size choice (profiling runs)")
    args = ap.parse_args()
    if args.config:
        import torch
        fg = _package()
        fg.build()
        stream = torch.cuda.Stream()
        fn = {"heat": config_heat, "q2": lambda g, s: config_q2(g, s, nel=args.q2_nel), "adjoint": config_adjoint,
              "mixed_graph": lambda g, s: config_mixed_graph(g, s, ny=args.mixed_ny, tune=not args.no_tune),
              "elements": config_elements, "pattern": config_pattern}[args.config]
        print(json.dumps({"config": args.config, "result": fn(fg, stream)}))
        return
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
