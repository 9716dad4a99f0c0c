#!/usr/bin/env python
"""Throughput of the explicit finite-volume step on one GB300, FP64.

Workload (the large plain configuration): 1448 x 1448 periodic square split
into 4,193,408 triangles, interior nodes jittered by U(-0.2h, 0.2h) from seed
20261203, isentropic vortex (strength 5 at (5,5), freestream rho=u=v=p=1),
second order with least-squares gradients (the reference's determinant guard)
and the Barth limiter, Roe flux (--flux llf for local Lax-Friedrichs), SSP-RK3,
CFL 0.8.  Synthetic data of the configuration's shape; no public dataset.

A "step" is one SSP-RK3 step (3 stages) of the whole mesh; the metric is
cell-stage updates per second = cells x 3 x steps / time.  Every array of the
step is larger than the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--flux roe|llf]
                    [--workload vortex_large|cylinder_ns|batch|adjoint|output]

Multi-GPU: the path is single-GPU; with N > 1 every rank runs an independent
replica of the workload (weak scaling, no collective on the data path) and the
time is the maximum over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SIDE = 1448
JSON_METRIC = "cell-stage updates/s (1 GB300, FP64, matched ref)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--flux", choices=["roe", "llf"], default="roe")
    ap.add_argument("--n", type=int, default=N_SIDE, help="cells per side of the square (default 1448)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", choices=["vortex_large", "cylinder_ns", "batch", "adjoint", "output"],
                    default="vortex_large",
                    help="cylinder_ns: the laminar cylinder O-grid (512 x 256 quads, Navier-Stokes, Kutta RK3) "
                         "through the plain path; batch: many cylinder instances in one persistent launch per stage vs the same "
                         "instances stepped one after another through the plain path; adjoint: the discrete "
                         "adjoint through K SSP-RK3 steps on the 256x256 jittered vortex")
    ap.add_argument("--batch-n", type=int, default=256)
    ap.add_argument("--adjoint-k", type=int, default=500)
    ap.add_argument("--fd-directions", type=int, default=64)
    ap.add_argument("--oracle-directions", type=int, default=0)
    return ap.parse_args()


def run_adjoint(args):
    """Discrete adjoint through K SSP-RK3 steps (256x256 jittered vortex with smooth waves on
    every variable, 131,072 cells, LSQ + Barth, Roe): time ratio to the primal, and central finite differences (step 1e-6) on random directions."""
    import torch
    torch.cuda.set_device(0)
    import cfd_solver_2d_gpu_gb300 as fv
    from cfd_solver_2d_gpu_gb300 import adjoint_backward, adjoint_forward, cases
    K = args.adjoint_k
    with tempfile.TemporaryDirectory() as d:
        su2 = cases.square_mesh(256, jitter=0.2, directory=d)
        tp = os.path.join(d, "adj.toml")
        with open(tp, "w") as f:
            f.write(cases.toml_text(flux=2002, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.8))
        p = fv.Params.from_toml(tp)
        mesh = fv.Mesh.read_su2(su2, p)
        s = fv.GPUSolver2(mesh, p)
        U0 = cases.wavy(mesh, s.get_state())
        rng = np.random.default_rng(20261203)
        r = rng.uniform(-1, 1, 3)
        pt = fv.Params.from_toml(tp)
        pt.vortex[0], pt.vortex[1], pt.vortex[2] = 5 + 0.1 * r[1], 5 + 0.1 * r[2], 5 * (1 + 0.02 * r[0])
        Ut0 = cases.wavy(mesh, fv.initial_field(mesh, pt))

        def fwd(U):
            s.set_state(U)
            s.set_time(0.0)
            s.step_timed(p.T_end, K)
            return s.get_state()

        rho_t = fwd(Ut0)[0]
        s.set_state(U0)
        s.set_time(0.0)
        s.step_timed(p.T_end, 3)  # warm-up
        s.set_state(U0)
        s.set_time(0.0)
        ms_primal = s.step_timed(p.T_end, K)
        nck = max(1, int(round(np.sqrt(K))))
        adjoint_forward(s, U0, K, nck)  # warm-up of the adjoint path
        t0 = time.perf_counter()
        UK, ms_f = adjoint_forward(s, U0, K, nck)
        dd = UK[0] - rho_t
        seed = np.zeros_like(UK)
        seed[0] = dd
        g, ms_b = adjoint_backward(s, seed)
        wall = time.perf_counter() - t0
        L0 = 0.5 * float(dd @ dd)

        def loss(U):
            x = fwd(U)[0] - rho_t
            return 0.5 * float(x @ x)

        h = 1e-6
        errs = []
        drng = np.random.default_rng(64)
        dirs = []
        for _ in range(args.fd_directions):
            v = drng.standard_normal(U0.shape)
            v /= np.linalg.norm(v)
            dirs.append(v)
            fd = (loss(U0 + h * v) - loss(U0 - h * v)) / (2 * h)
            errs.append(abs(fd - float(np.sum(g * v))) / max(abs(fd), 1e-300))
        ref_errs = []
        if args.oracle_directions > 0:
            from oracle import pyoracle
            pyoracle.set_threads(os.cpu_count() or 1)
            o = pyoracle.Oracle(tp, su2)
            rho_to = o.run(Ut0, K)[0][0]

            def oloss(U):
                x = o.run(U, K)[0][0] - rho_to
                return 0.5 * float(x @ x)
            for v in dirs[: args.oracle_directions]:
                fd = (oloss(U0 + h * v) - oloss(U0 - h * v)) / (2 * h)
                ref_errs.append(abs(fd - float(np.sum(g * v))) / max(abs(fd), 1e-300))
    errs = np.array(errs)
    # the forward sweep is the primal run itself (it produces U_K, which the loss needs) plus the
    # checkpoint copies; the adjoint's own cost is that overhead plus the reverse sweep (which
    # includes the recomputation of every segment but the last)
    line = {"metric": "adjoint-to-primal time ratio (1 GB300, FP64)",
            "value": (ms_f - ms_primal + ms_b) / ms_primal,
            "definition": "(forward sweep with checkpoints - plain primal + reverse sweep) / plain primal, "
                          "K steps each",
            "total_ratio": (ms_f + ms_b) / ms_primal,
            "unit": "x", "higher_is_better": False, "n_gpus": 1, "steps": K, "dtype": "f64",
            "data": "synthetic (generated mesh and initial field of the configuration's shape)",
            "config": {"workload": f"discrete adjoint through {K} SSP-RK3 steps, 256x256 jittered vortex + waves "
                                   f"({mesh.N} cells), LSQ + Barth, Roe, CFL 0.8, {nck} checkpoints",
                       "loss": "1/2 ||rho_K - rho_target||^2, target from a perturbed vortex"},
            "primal_ms": ms_primal, "adjoint_forward_ms": ms_f, "adjoint_backward_ms": ms_b,
            "ratio_backward_to_primal": ms_b / ms_primal, "wall_s": wall, "loss": L0,
            "fd": {"step": h, "directions": len(errs),
                   "median_rel_err": float(np.median(errs)) if len(errs) else None,
                   "max_rel_err": float(errs.max()) if len(errs) else None,
                   "frac_below_1e-6": float(np.mean(errs < 1e-6)) if len(errs) else None},
            "reference_gradient": {"directions": len(ref_errs),
                                   "max_rel_err": float(max(ref_errs)) if ref_errs else None,
                                   "source": "central differences of the oracle's forward map"}}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """Batched cylinder instances (cells log-uniform in [5k, 200k], Mach in [0.1, 0.6], Euler, Roe,
    LSQ + Barth, Kutta RK3): one persistent launch per stage in a graph, against the same instances
    stepped one after another through the plain path."""
    import torch
    torch.cuda.set_device(0)
    import cfd_solver_2d_gpu_gb300 as fv
    from cfd_solver_2d_gpu_gb300 import cases
    with tempfile.TemporaryDirectory() as d:
        insts = cases.cylinder_batch(d, n=args.batch_n)
        meshes, params = [], []
        for tp, sp, _ in insts:
            p = fv.Params.from_toml(tp)
            meshes.append(fv.Mesh.read_su2(sp, p))
            params.append(p)
    cells = sum(m.N for m in meshes)
    b = fv.Batch(meshes, params)
    report = b.tune(2)
    b.step_timed(args.warmup)
    with ClockSampler(0) as clk:
        ms_batch = b.step_timed(args.steps)
    info = b.info()
    clocks = clk.summary()
    # the same instances, one after another through the plain path
    ms_seq = 0.0
    launches_seq = 0
    for m, p in zip(meshes, params):
        s = fv.GPUSolver2(m, p)
        s.step_timed(p.T_end, 1)
        l0 = s.kernel_launches()
        ms_seq += s.step_timed(p.T_end, args.steps)
        launches_seq += s.kernel_launches() - l0
        s.close()
    value = 3.0 * cells * args.steps / (ms_batch / 1e3)
    seq = 3.0 * cells * args.steps / (ms_seq / 1e3)
    line = {"metric": JSON_METRIC + " [batched form]", "value": value, "unit": "cell-stage updates/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_batch / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (generated O-grids)",
            "config": {"workload": f"{len(meshes)} cylinder O-grid instances, {cells} cells in total "
                                   f"(log-uniform 5k-200k each, n_theta = 2 n_r), Mach U[0.1, 0.6], Euler, Roe, "
                                   f"LSQ + Barth, Kutta RK3, CFL 0.5"},
            "clocks": clocks, "gpu_launches": 3 * args.steps,
            "batch": {"persistent_launches_per_step": 3, "graph": bool(info["graph"]), "grid": info["grid"],
                      "block": info["block"], "tile": abs(info["tile"]),
                      "schedule": "queue" if info["tile"] < 0 else "static", "autotuner": report.strip().split("\n")},
            "sequential_plain": {"value": seq, "ms_per_step": ms_seq / args.steps,
                                 "kernel_launches_per_step": launches_seq / args.steps},
            "speedup_vs_sequential": ms_seq / ms_batch}
    print(json.dumps(line), flush=True)


def run_output(args):
    """Field output on the 1448x1448 mesh: the node-value kernel (FieldWriter::update_nodeField)
    and the colouring kernel (the GUI's cell -> node -> colour), device-timed, against HBM."""
    import torch
    torch.cuda.set_device(0)
    import cfd_solver_2d_gpu_gb300 as fv
    with tempfile.TemporaryDirectory() as d:
        tp, su2, _ = workload(args, d)
        p = fv.Params.from_toml(tp)
        mesh = fv.Mesh.read_su2(su2, p)
        s = fv.GPUSolver2(mesh, p)
        s.step(0.0, p.T_end, 2)
        N, V = mesh.N, mesh.V
        s.output_timed(args.warmup)
        reps = max(args.steps, 10)
        with ClockSampler(0) as clk:
            ms_nf, ms_col = s.output_timed(reps)
        t0 = time.perf_counter()
        path = os.path.join(d, "vol.dat")
        s.write_tecplot_volume(path, 1.0)
        t_write = time.perf_counter() - t0
        size = os.path.getsize(path)
    peak, peak_kind = measured_peaks()
    # compulsory bytes: node values = the cells' primitives (read U 32 N, write 32 N) + the node
    # gather (lists 4 (V + 1) + 12 N, primitives 32 N, outputs 48 V); colouring reads U once
    nf_bytes = 64 * N + 4 * (V + 1) + 12 * N + 32 * N + 48 * V
    col_bytes = 4 * (V + 1) + 12 * N + 32 * N + 16 * V
    nf_ms, col_ms = ms_nf / reps, ms_col / reps
    line = {"metric": "node values/s (field output, 1 GB300)", "value": V / (nf_ms / 1e3), "unit": "nodes/s",
            "n_gpus": 1, "steps": reps, "warmup": args.warmup, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic (generated mesh and initial field of the configuration's shape)",
            "config": {"workload": f"node values and colouring of the 1448x1448 jittered vortex ({N} cells, {V} nodes)"},
            "clocks": clk.summary(), "gpu_launches": 3 * reps,
            "roofline": {"bound": "hbm", "kernel": "k_cell_ruvp + k_node_field", "achieved": nf_bytes / (nf_ms / 1e3) / 1e9,
                         "peak": peak, "unit": "GB/s", "frac": nf_bytes / (nf_ms / 1e3) / 1e9 / peak,
                         "algorithmic_bytes_per_launch": nf_bytes, "avg_launch_ms": nf_ms, "peak_source": peak_kind},
            "colouring": {"value": V / (col_ms / 1e3), "unit": "nodes/s", "avg_launch_ms": col_ms,
                          "achieved_gbs": col_bytes / (col_ms / 1e3) / 1e9,
                          "frac": col_bytes / (col_ms / 1e3) / 1e9 / peak},
            "tecplot_volume_write": {"seconds": t_write, "bytes": size, "MB_per_s": size / t_write / 1e6}}
    print(json.dumps(line), flush=True)


def max_over_ranks(x, world):
    """The largest x over the ranks: a replicated job takes as long as its slowest rank."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(cells, stages, steps, world, seconds):
    """Whole-job cell-stage updates/s of world replicas, each advancing cells x stages x steps."""
    return stages * cells * steps * world / seconds


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def workload(args, directory):
    from cfd_solver_2d_gpu_gb300 import cases
    flux = 2002 if args.flux == "roe" else 2001
    if args.workload == "cylinder_ns":  # the laminar cylinder O-grid, 512 x 256 quads
        tp, su2 = cases.cylinder_ns(directory, flux=flux)
    else:
        tp, su2 = cases.vortex_large(directory, n=args.n, flux=flux)
    return tp, su2, flux


def config(args, N, E, V):
    if args.workload == "cylinder_ns":
        return {"workload": f"laminar cylinder O-grid 512x256 quads -> {N} triangles, Navier-Stokes, Ma 0.2, Re 100, "
                            f"second order (LSQ + Barth), {args.flux.upper()} flux, Kutta RK3, CFL 0.5",
                "cells": N, "edges": E, "nodes": V, "stages_per_step": 3,
                "gradient": "least squares (reference determinant guard) + Barth", "flux": args.flux,
                "integrator": "Kutta RK3", "l2_flush": "none: the per-step arrays (about 0.2 GB) exceed the L2 only "
                                                       "together",
                "parallelism": "replicas" if args.gpus > 1 else "single GPU"}
    return {"workload": f"jittered periodic vortex {args.n}x{args.n} quads -> {N} triangles, second order "
                        f"(LSQ + Barth), {args.flux.upper()} flux, SSP-RK3, CFL 0.8",
            "cells": N, "edges": E, "nodes": V, "stages_per_step": 3,
            "gradient": "least squares (reference determinant guard) + Barth", "flux": args.flux,
            "integrator": "SSP-RK3", "l2_flush": "none needed: every per-step array exceeds the 129 MB L2",
            "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def algorithmic_bytes(N, E, V):
    """Bytes each kernel group must move per launch under the convention 'every
    array element touched once, neighbour re-reads free' (FP64 8 B, int32 4 B)."""
    return {
        # U 32, 3 neighbour ids 12, count 4, least-squares weights 48, vertex offsets 48; grad write 64
        "gradient": 208 * N,
        # per edge: L,R 8, geometry 64, flux write 32; per cell: U + gradients read once 96
        "flux": 104 * E + 96 * N,
        # per cell: edge refs 12, -1/vol 8, U read+write 64, U0 32; per edge: flux read once 32
        "update": 116 * N + 32 * E,
        # prim: U 32 + prim 32 (+U0 copy 32); alpha: ids 8 + geometry 32 + prim 32/cell + alpha 8;
        # dt cell: CSR ids + alpha + vol
        "dt": 96 * N + 48 * E + 32 * N + 8 * N + 4 * (N + 2 * E),
        "restrict": 8,
    }


def stage_bytes(N, E, V):
    """Per-stage algorithmic bytes of the second-order step, 332 N + 48 E + 16 V."""
    return 332 * N + 48 * E + 16 * V


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_figures(flux, cells):
    """Per-launch DRAM traffic and FP64 flop / instruction counts from the committed ncu summary,
    scaled from the mesh they are quoted on to this run's by the cell count."""
    path = os.path.join(ROOT, "profiles", "ncu_step_kernels.json")
    try:
        with open(path) as f:
            figs = json.load(f).get(flux, {})
    except Exception:
        return {}
    out = {}
    for group, f in figs.items():
        scale = cells / f["scaled_to_cells"] if f.get("scaled_to_cells") else 1.0
        g = dict(f)
        for k in ("dram_bytes_per_launch", "fp64_flop_per_launch", "fp64_inst_per_launch"):
            if g.get(k) is not None:
                g[k] = g[k] * scale
        out[group] = g
    return out


def cpu_baseline(tp, su2, N, threads, max_steps, budget_s=30.0):
    """The oracle's restatement of the reference step on the host, same workload, bounded sample."""
    from oracle import pyoracle
    used = pyoracle.set_threads(threads)
    o = pyoracle.Oracle(tp, su2)
    U = o.init_field()
    t = 0.0
    done, elapsed = 0, 0.0
    while done < max_steps and (done == 0 or elapsed < budget_s):
        t0 = time.perf_counter()
        U, t, _, _ = o.run(U, 1, t)
        elapsed += time.perf_counter() - t0
        done += 1
    return {"value": 3.0 * N * done / elapsed, "unit": "cell-stage updates/s", "cores": used, "kind": "port",
            "sample": f"{done} SSP-RK3 step(s) of the full {N}-cell mesh in {elapsed:.1f} s, {used} thread(s)"}


def run_reference(args, rank, world):
    """The reference arm: the reference step's CPU restatement (oracle/fvm_oracle.c) with all host threads."""
    if rank != 0:
        return
    ncores = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as d:
        tp, su2, flux = workload(args, d)
        from oracle import pyoracle
        pyoracle.set_threads(ncores)
        o = pyoracle.Oracle(tp, su2)
        N, E, V = o.N, o.E, o.V
        U = o.init_field()
        t = 0.0
        for _ in range(min(args.warmup, 1)):
            U, t, _, _ = o.run(U, 1, t)
        steps = max(1, min(args.steps, 10))
        t0 = time.perf_counter()
        U, t, _, _ = o.run(U, steps, t)
        el = time.perf_counter() - t0
    value = 3.0 * N * steps / el
    line = {"impl": "reference", "metric": JSON_METRIC, "value": value, "unit": "cell-stage updates/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": min(args.warmup, 1), "ms_per_step": 1e3 * el / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(args, N, E, V),
            "cpu_baseline": {"value": value, "unit": "cell-stage updates/s", "cores": ncores, "kind": "port",
                             "sample": f"{steps} SSP-RK3 steps of the full {N}-cell mesh, {ncores} threads "
                                       f"(the reference has no GPU path for this configuration)"},
            "e2e": {"value": value, "unit": "cell-stage updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.workload == "batch" and args.impl == "ours":
        if rank == 0:
            run_batch(args)
        return
    if args.workload == "adjoint" and args.impl == "ours":
        if rank == 0:
            run_adjoint(args)
        return
    if args.workload == "output" and args.impl == "ours":
        if rank == 0:
            run_output(args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import cfd_solver_2d_gpu_gb300 as fv

    with tempfile.TemporaryDirectory() as d:
        tp, su2, flux = workload(args, d)
        p = fv.Params.from_toml(tp)
        p.device = local
        mesh = fv.Mesh.read_su2(su2, p)
        N, E, V = mesh.N, mesh.E, mesh.V
        s = fv.GPUSolver2(mesh, p)
        U0 = s.get_state()
        T = p.T_end
        s.set_time(0.0)
        # warm-up
        s.step_timed(T, args.warmup)

        def barrier():
            if world > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
            s.synchronize()

        barrier()
        l0 = s.kernel_launches()
        with ClockSampler(local) as clk:
            ms = s.step_timed(T, args.steps)
        barrier()
        launches = s.kernel_launches() - l0
        ms = max_over_ranks(ms, world)
        clocks = clk.summary()
        value = job_throughput(N, 3, args.steps, world, ms / 1e3)

        # per-kernel-group device times (same steps, launched one by one with events)
        prof = s.profile_steps(T, max(3, min(args.steps, 20)))
        algo = algorithmic_bytes(N, E, V)
        dom = max((k for k in prof if prof[k][1] > 0 and k != "restrict"), key=lambda k: prof[k][0])
        avg_ms = prof[dom][0] / prof[dom][1]
        peak, peak_kind = measured_peaks()
        achieved = algo[dom] / (avg_ms / 1e3) / 1e9
        # the committed per-launch ncu figures are of the vortex workload's kernels
        ncu = ncu_figures(args.flux, N) if args.workload == "vortex_large" else {}
        traffic = ncu.get(dom, {}).get("dram_bytes_per_launch")
        stage_ms = (prof["gradient"][0] + prof["flux"][0] + prof["update"][0]) / max(prof["update"][1], 1)
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": algo[dom], "avg_launch_ms": avg_ms,
                "share_of_step": prof[dom][0] / sum(v[0] for v in prof.values())}
        fp64_peak = fv.fp64_peak(local)  # GFLOP/s, register FMA chains on every SM, measured now
        fp64 = None
        if ncu.get(dom, {}).get("fp64_flop_per_launch"):
            a64 = ncu[dom]["fp64_flop_per_launch"] / (avg_ms / 1e3) / 1e9
            fp64 = {"achieved_gflops": a64, "peak_gflops": fp64_peak, "frac": a64 / fp64_peak,
                    "kernel": dom, "peak_source": "fvgb_fp64_peak (FMA chains, measured in this run)",
                    "source": "fp64 flop per launch from ncu x live launch time"}
            if ncu[dom].get("fp64_inst_per_launch") and clocks.get("sm_mhz"):
                # the FP64 pipe issues 2 thread-instructions per SM per cycle (dadd, dmul and dfma alike)
                sms = torch.cuda.get_device_properties(local).multi_processor_count
                peak_inst = 2 * sms * clocks["sm_mhz"] * 1e6
                ach_inst = ncu[dom]["fp64_inst_per_launch"] / (avg_ms / 1e3)
                fp64["issue_frac"] = ach_inst / peak_inst
                fp64["issue_note"] = ("FP64 instructions per second over 2 x SMs x the sampled SM clock: the "
                                      "pipe-issue bound, which counts dadd and dmul as full slots")
        stage_roof = {"achieved": stage_bytes(N, E, V) / (stage_ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                      "frac": stage_bytes(N, E, V) / (stage_ms / 1e3) / 1e9 / peak,
                      "bytes_per_stage": stage_bytes(N, E, V), "formula": "332N + 48E + 16V"}

        # end to end through the C ABI with host buffers: H2D of the state, one step, D2H of the state
        e2e = None
        if not args.no_e2e:
            host = torch.empty((4, N), dtype=torch.float64, pin_memory=True)
            host.copy_(torch.from_numpy(U0))
            k_e2e = max(3, min(args.steps, 20))
            t = 0.0
            s.set_state_ptr(host.data_ptr())
            t = s.step(t, T, 1)
            s.get_state_ptr(host.data_ptr())
            barrier()
            t0 = time.perf_counter()
            for _ in range(k_e2e):
                s.set_state_ptr(host.data_ptr())
                t = s.step(t, T, 1)
                s.get_state_ptr(host.data_ptr())
            barrier()
            el = max_over_ranks(time.perf_counter() - t0, world)
            e2e = {"value": job_throughput(N, 3, k_e2e, world, el), "unit": "cell-stage updates/s",
                   "h2d_bytes_per_step": 32 * N, "d2h_bytes_per_step": 32 * N, "steps": k_e2e,
                   "api": "fvgb_set_state + fvgb_step + fvgb_get_state (pinned host buffers)"}

        cpu = None
        if rank == 0 and not args.no_cpu_baseline:
            cpu = cpu_baseline(tp, su2, N, threads=1, max_steps=3)

    if rank == 0:
        line = {"metric": JSON_METRIC, "value": value, "unit": "cell-stage updates/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (generated mesh and initial field of the configuration's shape)",
                "config": config(args, N, E, V), "clocks": clocks, "gpu_launches": launches,
                "roofline": roof, "roofline_stage": stage_roof, "fp64": fp64, "kernel_ms": prof,
                "e2e": e2e, "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
