#!/usr/bin/env python
"""Throughput of the explicit finite-volume step on one GB300, FP64.

Headline workload (the large plain configuration): 1448 x 1448 periodic square
split into 4,193,408 triangles, interior nodes jittered by U(-0.2h, 0.2h) from
seed 20261203, isentropic vortex (strength 5 at (5,5), freestream
rho=u=v=p=1), second order with least-squares gradients (the reference's
determinant guard) and the Barth limiter, Roe flux (--flux llf for local
Lax-Friedrichs), SSP-RK3, CFL 0.8.  Synthetic data of the configuration's
shape; no public dataset.

A "step" is one SSP-RK3 step (3 stages) of the whole mesh; the metric is
cell-stage updates per second = cells x 3 x steps / time.  Every array of the
step is larger than the 129 MB L2, so no flush is needed between steps.

At one GPU the same JSON line also carries the other configurations' records:
  edge_colour  the same workload with the edge-coloured scatter in place of the gather;
  cylinder_ns  the laminar cylinder O-grid (512 x 256 quads, Navier-Stokes, Kutta RK3);
  batch        256 cylinder O-grids in one persistent launch per stage against the same
               instances stepped one after another through the plain path;
  adjoint      the discrete adjoint through 500 SSP-RK3 steps of the 256 x 256 jittered
               vortex: time ratio to the primal, central finite differences on 64
               directions (with a sweep of the difference step on the worst ones) and
               the reference gradient (finite differences of the oracle's forward map).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--flux roe|llf]
                    [--workload vortex_large|cylinder_ns|batch|adjoint|output] [--no-extras]

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
    ap.add_argument("--no-extras", action="store_true",
                    help="leave the cylinder_ns, batch and adjoint records out of the headline line")
    ap.add_argument("--workload", choices=["vortex_large", "cylinder_ns", "batch", "adjoint", "output"],
                    default="vortex_large",
                    help="cylinder_ns: the laminar cylinder O-grid (512 x 256 quads, Navier-Stokes, Kutta RK3) "
                         "through the plain path; batch: many cylinder instances in one persistent launch per stage vs the same "
                         "instances stepped one after another through the plain path; adjoint: the discrete "
                         "adjoint through K SSP-RK3 steps on the 256x256 jittered vortex")
    ap.add_argument("--batch-n", type=int, default=256)
    ap.add_argument("--adjoint-k", type=int, default=500)
    ap.add_argument("--fd-directions", type=int, default=64)
    ap.add_argument("--oracle-directions", type=int, default=8)
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms during the timed region.
    Entering waits (up to 5 s) for the first sample, so that sampling covers the region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index, interval_ms=50):
        self.index = index
        self.interval_ms = interval_ms
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return self
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.01)
        self.skip = self._rows_now()  # samples taken before the region starts are left out
        return self

    def _rows_now(self):
        self.f.flush()
        with open(self.f.name) as fh:
            return sum(1 for line in fh if line.count(",") >= 8)

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(self.interval_ms / 1e3)  # one more sample at the end of the region
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
        rows = rows[getattr(self, "skip", 0):] or rows[-1:]  # the samples taken during the region
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        num = lambda x: x.replace(".", "", 1).isdigit()
        sm = [float(r[1]) for r in rows if num(r[1])]
        mx = [float(r[2]) for r in rows if num(r[2])]
        pw = [float(r[3]) for r in rows if num(r[3])]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "sm_mhz_min": min(sm) if sm else None, "power_w_max": max(pw) if pw else None,
                "reasons": sorted(reasons), "samples": len(rows), "interval_ms": self.interval_ms}


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


# ---- workloads ------------------------------------------------------------------

def workload(args, directory):
    from cfd_solver_2d_gpu_gb300 import cases
    flux = 2002 if args.flux == "roe" else 2001
    if args.workload == "cylinder_ns":  # the laminar cylinder O-grid, 512 x 256 quads
        tp, su2 = cases.cylinder_ns(directory, flux=flux)
    else:
        tp, su2 = cases.vortex_large(directory, n=args.n, flux=flux)
    return tp, su2, flux


def config(args, N, E, V, workload=None):
    workload = workload or args.workload
    if workload == "cylinder_ns":
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


def kernel_roofline(s, T, N, E, V, steps, flux, with_ncu, device):
    """Per-kernel-group device times of `steps` steps (launched one by one with CUDA events on
    the solver's stream), the dominant group's HBM roofline and, where the committed ncu figures
    cover the workload, its FP64-pipe roofline."""
    prof = s.profile_steps(T, steps)
    algo = algorithmic_bytes(N, E, V)
    dom = max((k for k in prof if prof[k][1] > 0 and k != "restrict"), key=lambda k: prof[k][0])
    avg_ms = prof[dom][0] / prof[dom][1]
    peak, peak_kind = measured_peaks()
    achieved = algo[dom] / (avg_ms / 1e3) / 1e9
    ncu = ncu_figures(flux, N) if with_ncu else {}
    traffic = ncu.get(dom, {}).get("dram_bytes_per_launch")
    stage_ms = (prof["gradient"][0] + prof["flux"][0] + prof["update"][0]) / max(prof["update"][1], 1)
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": algo[dom], "avg_launch_ms": avg_ms,
            "share_of_step": prof[dom][0] / sum(v[0] for v in prof.values())}
    stage_roof = {"achieved": stage_bytes(N, E, V) / (stage_ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                  "frac": stage_bytes(N, E, V) / (stage_ms / 1e3) / 1e9 / peak,
                  "bytes_per_stage": stage_bytes(N, E, V), "formula": "332N + 48E + 16V"}
    return prof, dom, avg_ms, ncu, roof, stage_roof


def run_cylinder(args, quiet=False):
    """C3: the laminar Navier-Stokes cylinder (512 x 256 O-grid, 262,144 cells, Ma 0.2, Re 100,
    LSQ + Barth, Kutta RK3) through the plain path."""
    import torch
    torch.cuda.set_device(0)
    import cfd_solver_2d_gpu_gb300 as fv
    from cfd_solver_2d_gpu_gb300 import cases
    flux = 2002 if args.flux == "roe" else 2001
    with tempfile.TemporaryDirectory() as d:
        tp, su2 = cases.cylinder_ns(d, flux=flux)
        p = fv.Params.from_toml(tp)
        mesh = fv.Mesh.read_su2(su2, p)
    N, E, V = mesh.N, mesh.E, mesh.V
    s = fv.GPUSolver2(mesh, p)
    s.set_time(0.0)
    s.step_timed(p.T_end, args.warmup)
    steps = max(args.steps, 50)  # a step is under 1 ms: at least 50 for the clock record
    l0 = s.kernel_launches()
    with ClockSampler(0) as clk:
        ms = s.step_timed(p.T_end, steps)
    launches = s.kernel_launches() - l0
    prof, dom, avg_ms, _, roof, stage_roof = kernel_roofline(s, p.T_end, N, E, V, max(3, min(steps, 20)),
                                                             args.flux, False, 0)
    res = s.update_residual_vector(0)
    s.close()
    line = {"metric": JSON_METRIC + " [laminar cylinder]", "value": 3.0 * N * steps / (ms / 1e3),
            "unit": "cell-stage updates/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup,
            "ms_per_step": ms / steps, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic (generated O-grid, uniform freestream)",
            "config": config(args, N, E, V, "cylinder_ns"), "clocks": clk.summary(), "gpu_launches": launches,
            "roofline": roof, "roofline_stage": stage_roof, "kernel_ms": prof,
            "residual_linf": [float(x) for x in res]}
    if not quiet:
        print(json.dumps(line), flush=True)
    return line


def run_colour(args, quiet=False):
    """The headline workload with the edge-coloured scatter ([gpu] edge_colour = 1: each
    colour's edges add their fluxes into the cells' sums) in place of the slot-order gather:
    the side-by-side measurement of the two residual forms on the same mesh."""
    import torch
    torch.cuda.set_device(0)
    import cfd_solver_2d_gpu_gb300 as fv
    with tempfile.TemporaryDirectory() as d:
        tp, su2, flux = workload(args, d)
        p = fv.Params.from_toml(tp)
        p.edge_colour = 1
        mesh = fv.Mesh.read_su2(su2, p)
    N, E, V = mesh.N, mesh.E, mesh.V
    s = fv.GPUSolver2(mesh, p)
    _, ncol = s.edge_colours()
    s.set_time(0.0)
    s.step_timed(p.T_end, args.warmup)
    l0 = s.kernel_launches()
    with ClockSampler(0) as clk:
        ms = s.step_timed(p.T_end, args.steps)
    launches = s.kernel_launches() - l0
    prof = s.profile_steps(p.T_end, max(3, min(args.steps, 20)))
    s.close()
    line = {"metric": JSON_METRIC + " [edge-coloured scatter]", "value": 3.0 * N * args.steps / (ms / 1e3),
            "unit": "cell-stage updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "dtype": "f64",
            "config": dict(config(args, N, E, V), residual="edge-coloured scatter", colours=ncol),
            "clocks": clk.summary(), "gpu_launches": launches, "kernel_ms": prof}
    if not quiet:
        print(json.dumps(line), flush=True)
    return line


def run_batch(args, quiet=False):
    """C4: batched cylinder instances (cells log-uniform in [5k, 200k], Mach in [0.1, 0.6], Euler,
    Roe, LSQ + Barth, Kutta RK3): one persistent launch per stage in a graph, against the same
    instances stepped one after another through the plain path."""
    import torch
    torch.cuda.set_device(0)
    import cfd_solver_2d_gpu_gb300 as fv
    from cfd_solver_2d_gpu_gb300 import cases
    t_setup = time.perf_counter()
    with tempfile.TemporaryDirectory() as d:
        insts = cases.cylinder_batch(d, n=args.batch_n)
        meshes, params = [], []
        for tp, sp, _ in insts:
            p = fv.Params.from_toml(tp)
            meshes.append(fv.Mesh.read_su2(sp, p))
            params.append(p)
    cells = sum(m.N for m in meshes)
    b = fv.Batch(meshes, params)
    setup_s = time.perf_counter() - t_setup
    report = b.tune(2)
    steps = max(args.steps, 20)
    b.step_timed(args.warmup)
    l0 = b.info()["launches"]
    with ClockSampler(0) as clk:
        ms_batch = b.step_timed(steps)
    launches = b.info()["launches"] - l0
    info = b.info()
    clocks = clk.summary()
    b.close()
    # the same instances, one after another through the plain path, each warmed up first
    ms_seq = 0.0
    launches_seq = 0
    with ClockSampler(0) as clk_seq:
        for m, p in zip(meshes, params):
            s = fv.GPUSolver2(m, p)
            s.step_timed(p.T_end, 1)
            l1 = s.kernel_launches()
            ms_seq += s.step_timed(p.T_end, steps)
            launches_seq += s.kernel_launches() - l1
            s.close()
    value = 3.0 * cells * steps / (ms_batch / 1e3)
    seq = 3.0 * cells * steps / (ms_seq / 1e3)
    line = {"metric": JSON_METRIC + " [batched form]", "value": value, "unit": "cell-stage updates/s", "n_gpus": 1,
            "steps": steps, "warmup": args.warmup, "ms_per_step": ms_batch / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (generated O-grids)",
            "config": {"workload": f"{len(meshes)} cylinder O-grid instances, {cells} cells in total "
                                   f"(log-uniform 5k-200k each, n_theta = 2 n_r), Mach U[0.1, 0.6], Euler, Roe, "
                                   f"LSQ + Barth, Kutta RK3, CFL 0.5", "instances": len(meshes), "cells": cells},
            "clocks": clocks, "gpu_launches": launches,
            "batch": {"persistent_launches_per_step": launches / steps, "graph": bool(info["graph"]),
                      "grid": info["grid"], "block": info["block"], "tile": abs(info["tile"]),
                      "schedule": "queue" if info["tile"] < 0 else "static",
                      "autotuner": report.strip().split("\n"), "setup_s": setup_s},
            "sequential_plain": {"value": seq, "ms_per_step": ms_seq / steps,
                                 "kernel_launches_per_step": launches_seq / steps, "clocks": clk_seq.summary()},
            "speedup_vs_sequential": ms_seq / ms_batch}
    if not quiet:
        print(json.dumps(line), flush=True)
    return line


def run_adjoint(args, quiet=False):
    """C5: the discrete adjoint through K SSP-RK3 steps (256x256 jittered vortex with smooth waves on
    every variable, 131,072 cells, LSQ + Barth, Roe, sqrt(K) checkpoints): time ratio to the primal;
    central finite differences (step 1e-6) on random unit directions, and on the directions whose
    error exceeds 1e-6 a sweep of the difference step (1e-4 .. 1e-8), which separates truncation
    and round-off from branch switches of the limiter and the time-step minimum; the reference
    gradient: central differences of the oracle's forward map on the first directions."""
    import torch
    torch.cuda.set_device(0)
    import cfd_solver_2d_gpu_gb300 as fv
    from cfd_solver_2d_gpu_gb300 import adjoint_backward, adjoint_forward, adjoint_overlap, cases
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
        nck = max(1, int(round(np.sqrt(K))))
        with ClockSampler(0) as clk:
            s.set_state(U0)
            s.set_time(0.0)
            ms_primal = s.step_timed(p.T_end, K)
            # warm-up of the adjoint path: lays out the workspace and captures the backward
            # sweep's graphs, which the timed pair reuses (as the primal reuses its step graphs)
            UK, ms_f_first = adjoint_forward(s, U0, K, nck)
            dd = UK[0] - rho_t
            seed = np.zeros_like(UK)
            seed[0] = dd
            _, ms_b_first = adjoint_backward(s, seed)
            t0 = time.perf_counter()
            UK, ms_f = adjoint_forward(s, U0, K, nck)
            g, ms_b = adjoint_backward(s, seed)
            wall = time.perf_counter() - t0
            overlapped = adjoint_overlap(s)
            # the same sweeps with recomputation and reverse one after the other (one set of records)
            adjoint_overlap(s, 0)
            adjoint_forward(s, U0, K, nck)
            adjoint_backward(s, seed)
            UK_seq, ms_f_seq = adjoint_forward(s, U0, K, nck)
            g_seq, ms_b_seq = adjoint_backward(s, seed)
            adjoint_overlap(s, 1)
        L0 = 0.5 * float(dd @ dd)

        def loss(U):
            x = fwd(U)[0] - rho_t
            return 0.5 * float(x @ x)

        def fd(lossf, v, h):
            return (lossf(U0 + h * v) - lossf(U0 - h * v)) / (2 * h)

        def err(a, b):
            return abs(a - b) / max(abs(a), 1e-300)

        h = 1e-6
        drng = np.random.default_rng(64)
        dirs, errs, fds = [], [], []
        for _ in range(args.fd_directions):
            v = drng.standard_normal(U0.shape)
            v /= np.linalg.norm(v)
            dirs.append(v)
            fds.append(fd(loss, v, h))
            errs.append(err(fds[-1], float(np.sum(g * v))))
        errs = np.array(errs)
        # difference-step sweep on the directions above 1e-6
        sweep_steps = [1e-4, 1e-5, 1e-6, 1e-7, 1e-8]
        worst = [i for i in range(len(dirs)) if errs[i] > 1e-6]
        sweep = {f"{hh:g}": [] for hh in sweep_steps}
        best = []
        for i in worst:
            e_i = []
            for hh in sweep_steps:
                e = errs[i] if hh == h else err(fd(loss, dirs[i], hh), float(np.sum(g * dirs[i])))
                sweep[f"{hh:g}"].append(e)
                e_i.append(e)
            best.append(min(e_i))
        sweep_summary = {k: {"median": float(np.median(v)), "max": float(np.max(v))} for k, v in sweep.items() if v}
        # the reference gradient: central differences of the oracle's forward map (FP64 C restatement
        # of the reference step, all host threads), on the first directions
        ref_errs, ref_vs_gpu_fd = [], []
        oracle_s = 0.0
        if args.oracle_directions > 0:
            from oracle import pyoracle
            pyoracle.set_threads(os.cpu_count() or 1)
            t_o = time.perf_counter()
            o = pyoracle.Oracle(tp, su2)
            rho_to = o.run(Ut0, K)[0][0]

            def oloss(U):
                x = o.run(U, K)[0][0] - rho_to
                return 0.5 * float(x @ x)
            for i, v in enumerate(dirs[: args.oracle_directions]):
                fo = fd(oloss, v, h)
                ref_errs.append(err(fo, float(np.sum(g * v))))
                ref_vs_gpu_fd.append(err(fo, fds[i]))
            oracle_s = time.perf_counter() - t_o
        s.close()
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
            "clocks": clk.summary(),
            "primal_ms": ms_primal, "adjoint_forward_ms": ms_f, "adjoint_backward_ms": ms_b,
            "ratio_backward_to_primal": ms_b / ms_primal, "wall_s": wall, "loss": L0,
            "overlap": {"used": overlapped,
                        "note": "each segment's recomputation on the solver's stream beside the reverse of the "
                                "next segment on a second stream (two sets of records); sequential: one set, "
                                "recomputation then reverse, same run",
                        "sequential_forward_ms": ms_f_seq, "sequential_backward_ms": ms_b_seq,
                        "sequential_value": (ms_f_seq - ms_primal + ms_b_seq) / ms_primal,
                        "bitwise_equal": bool(np.array_equal(g_seq, g) and np.array_equal(UK_seq, UK))},
            "first_call": {"adjoint_forward_ms": ms_f_first, "adjoint_backward_ms": ms_b_first,
                           "value": (ms_f_first - ms_primal + ms_b_first) / ms_primal,
                           "note": "the warm-up pair: a fresh workspace, the backward sweep capturing its graphs"},
            "fd": {"step": h, "directions": len(errs),
                   "median_rel_err": float(np.median(errs)) if len(errs) else None,
                   "max_rel_err": float(errs.max()) if len(errs) else None,
                   "frac_below_1e-6": float(np.mean(errs < 1e-6)) if len(errs) else None,
                   "frac_below_1e-5": float(np.mean(errs < 1e-5)) if len(errs) else None},
            "fd_step_sweep": {"directions": len(worst), "per_step": sweep_summary,
                              "best_step_max_rel_err": float(max(best)) if best else None,
                              "best_step_median_rel_err": float(np.median(best)) if best else None,
                              "note": "directions whose error at step 1e-6 exceeds 1e-6; per difference step the "
                                      "median and max relative error against the adjoint"},
            "reference_gradient": {"directions": len(ref_errs),
                                   "median_rel_err": float(np.median(ref_errs)) if ref_errs else None,
                                   "max_rel_err": float(max(ref_errs)) if ref_errs else None,
                                   "oracle_fd_vs_gpu_fd_max_rel": float(max(ref_vs_gpu_fd)) if ref_vs_gpu_fd else None,
                                   "step": h, "seconds": oracle_s,
                                   "source": "central differences of the oracle's forward map (FP64 C restatement "
                                             "of the reference step), all host threads"}}
    if not quiet:
        print(json.dumps(line), flush=True)
    return line


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
    """The reference arm: the reference's CPU step path for the headline workload, timed on the
    host cores with every thread.  The reference compiled from its own sources (oracle/_ref) is
    built only where its sources are mounted and is x86; everywhere else this is the oracle's C
    restatement of it (oracle/fvm_oracle.c, bit for bit equal to the reference on every golden
    case), OpenMP across the host cores.  The mesh comes from oracle/meshgen.py and the input.toml
    text from cases.toml_text, both pure Python: this process loads none of the product's native
    code.  W untimed and K timed steps, as given."""
    if rank != 0:
        return
    if args.workload != "vortex_large":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the headline workload "
                                                             "(vortex_large) only"}), flush=True)
        return
    from cfd_solver_2d_gpu_gb300 import cases  # input.toml text only (pure Python)
    from oracle import meshgen, pyoracle
    ncores = os.cpu_count() or 1
    flux = 2002 if args.flux == "roe" else 2001
    with tempfile.TemporaryDirectory() as d:
        su2 = meshgen.write_periodic_square(os.path.join(d, "vortex.su2"), args.n, 10.0, 0.2, cases.JITTER_SEED)
        tp = os.path.join(d, "vortex.toml")
        with open(tp, "w") as f:
            f.write(cases.toml_text(flux=flux, reconstruct=3002, gradient=1, limiter=1, time_advance=3104, CFL=0.8))
        used = pyoracle.set_threads(ncores)
        o = pyoracle.Oracle(tp, su2)
        N, E, V = o.N, o.E, o.V
        U = o.init_field()
        t = 0.0
        if args.warmup > 0:
            U, t, _, _ = o.run(U, args.warmup, t)
        steps = max(1, args.steps)
        t0 = time.perf_counter()
        U, t, _, _ = o.run(U, steps, t)
        el = time.perf_counter() - t0
    value = 3.0 * N * steps / el
    line = {"impl": "reference", "metric": JSON_METRIC, "value": value, "unit": "cell-stage updates/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(args, N, E, V),
            "cpu_baseline": {"value": value, "unit": "cell-stage updates/s", "cores": used, "kind": "port",
                             "sample": f"{steps} SSP-RK3 steps of the full {N}-cell mesh after {args.warmup} "
                                       f"untimed, {used} threads (the reference has no GPU path for this "
                                       f"configuration: its GPU step supports Green-Gauss and forward Euler only)"},
            "e2e": {"value": value, "unit": "cell-stage updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _gpu_numa_node(torch, local):
    """The host NUMA node the GPU is attached to, and that node's CPUs, as the host reports them
    (sysfs); (-1, []) where it reports none."""
    try:
        pr = torch.cuda.get_device_properties(local)
        bus = f"{pr.pci_domain_id:04x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0"
        with open(f"/sys/bus/pci/devices/{bus}/numa_node") as f:
            node = int(f.read().strip())
    except Exception:
        return -1, []
    cpus = []
    try:
        with open(f"/sys/devices/system/node/node{node}/cpulist") as f:
            for part in f.read().strip().split(","):
                if "-" in part:
                    a, b = part.split("-")
                    cpus += list(range(int(a), int(b) + 1))
                elif part:
                    cpus.append(int(part))
    except Exception:
        pass
    return node, cpus


def _pages_per_node(addr):
    """Pages of the mapping that holds addr, per NUMA node (/proc/self/numa_maps)."""
    try:
        start = None
        with open("/proc/self/maps") as f:
            for line in f:
                a, b = (int(x, 16) for x in line.split()[0].split("-"))
                if a <= addr < b:
                    start = a
                    break
        with open("/proc/self/numa_maps") as f:
            for line in f:
                parts = line.split()
                if start is not None and int(parts[0], 16) == start:
                    return {p.split("=")[0]: int(p.split("=")[1]) for p in parts if p.startswith("N") and "=" in p}
    except Exception:
        pass
    return {}


def pinned_state(torch, N, local):
    """A page-locked (4, N) FP64 host buffer, allocated while the thread runs on the CPUs of the
    GPU's NUMA node (first-touch placement), and where its pages ended up."""
    node, cpus = _gpu_numa_node(torch, local)
    old = os.sched_getaffinity(0)
    if cpus:
        try:
            os.sched_setaffinity(0, cpus)
        except OSError:
            cpus = []
    try:
        host = torch.empty((4, N), dtype=torch.float64, pin_memory=True)
        host.zero_()
    finally:
        if cpus:
            os.sched_setaffinity(0, old)
    return host, {"gpu_numa_node": node, "allocated_on_node_cpus": bool(cpus),
                  "pages_per_node": _pages_per_node(host.data_ptr())}


def run_e2e(torch, s, U0, N, T, steps, world, barrier, local):
    """End to end through the C ABI with host buffers, as a caller of the library steps:
    fvgb_set_state from a page-locked host buffer, fvgb_step(1), fvgb_get_state into it, every step.
    Each phase is timed on its own (each call returns after its work), and a raw pinned
    cudaMemcpyAsync of the same bytes each way is timed beside it with CUDA events."""
    host, numa = pinned_state(torch, N, local)
    host.copy_(torch.from_numpy(U0))
    t = 0.0
    s.set_state_ptr(host.data_ptr())
    t = s.step(t, T, 1)
    s.get_state_ptr(host.data_ptr())
    barrier()
    h2d = stp = d2h = 0.0
    t0 = time.perf_counter()
    for _ in range(steps):
        a = time.perf_counter()
        s.set_state_ptr(host.data_ptr())
        b = time.perf_counter()
        t = s.step(t, T, 1)
        c = time.perf_counter()
        s.get_state_ptr(host.data_ptr())
        d = time.perf_counter()
        h2d += b - a
        stp += c - b
        d2h += d - c
    barrier()
    el = max_over_ranks(time.perf_counter() - t0, world)
    # raw copies of the same bytes through the same pinned buffer
    dev = torch.empty((4, N), dtype=torch.float64, device=f"cuda:{local}")
    nbytes = 32 * N
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    dev.copy_(host, non_blocking=True)
    host.copy_(dev, non_blocking=True)
    torch.cuda.synchronize()
    reps = 5
    ev[0].record()
    for _ in range(reps):
        dev.copy_(host, non_blocking=True)
    ev[1].record()
    for _ in range(reps):
        host.copy_(dev, non_blocking=True)
    ev[2].record()
    torch.cuda.synchronize()
    raw_h2d = nbytes * reps / (ev[0].elapsed_time(ev[1]) / 1e3) / 1e9
    raw_d2h = nbytes * reps / (ev[1].elapsed_time(ev[2]) / 1e3) / 1e9
    del dev
    return {"value": job_throughput(N, 3, steps, world, el), "unit": "cell-stage updates/s",
            "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes, "steps": steps,
            "api": "fvgb_set_state + fvgb_step + fvgb_get_state (page-locked host buffers)",
            "ms_per_step": 1e3 * el / steps,
            "split_ms_per_step": {"set_state": 1e3 * h2d / steps, "step": 1e3 * stp / steps,
                                  "get_state": 1e3 * d2h / steps},
            "link_gbs": {"set_state": nbytes / (h2d / steps) / 1e9, "get_state": nbytes / (d2h / steps) / 1e9,
                         "raw_pinned_memcpy_h2d": raw_h2d, "raw_pinned_memcpy_d2h": raw_d2h},
            "host_buffer": numa}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    standalone = {"batch": run_batch, "adjoint": run_adjoint, "output": run_output, "cylinder_ns": run_cylinder}
    if args.workload in standalone:
        if rank == 0:
            standalone[args.workload](args)
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
        s.step_timed(T, args.warmup)  # warm-up

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

        prof, dom, avg_ms, ncu, roof, stage_roof = kernel_roofline(s, T, N, E, V, max(3, min(args.steps, 20)),
                                                                   args.flux, True, local)
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
            fp64["per_kernel_issue_frac"] = {}
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            for grp, f in ncu.items():
                if f.get("fp64_inst_per_launch") and prof.get(grp, (0, 0))[1] and clocks.get("sm_mhz"):
                    ms_l = prof[grp][0] / prof[grp][1]
                    fp64["per_kernel_issue_frac"][grp] = (f["fp64_inst_per_launch"] / (ms_l / 1e3)) / (
                        2 * sms * clocks["sm_mhz"] * 1e6)

        e2e = None
        if not args.no_e2e:
            e2e = run_e2e(torch, s, U0, N, T, args.steps, world, barrier, local)
        s.close()

        cpu = None
        if rank == 0 and not args.no_cpu_baseline:
            cpu = cpu_baseline(tp, su2, N, threads=1, max_steps=3)

    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        line = {"metric": JSON_METRIC, "value": value, "unit": "cell-stage updates/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (generated mesh and initial field of the configuration's shape)",
                "config": config(args, N, E, V), "clocks": clocks, "gpu_launches": launches,
                "roofline": roof, "roofline_stage": stage_roof, "fp64": fp64, "kernel_ms": prof,
                "e2e": e2e, "cpu_baseline": cpu}
        if world == 1 and not args.no_extras:
            # the other configurations, each measured on its own after the headline run
            for key, fn in (("edge_colour", run_colour), ("cylinder_ns", run_cylinder), ("batch", run_batch),
                            ("adjoint", run_adjoint)):
                t0 = time.perf_counter()
                try:
                    rec = fn(args, quiet=True)
                except Exception as exc:  # one record's failure must not hide the headline number
                    rec = {"error": f"{type(exc).__name__}: {exc}"}
                rec["wall_s"] = time.perf_counter() - t0
                if key == "edge_colour" and rec.get("value"):
                    rec["ratio_to_gather"] = rec["value"] / value
                line[key] = rec
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
