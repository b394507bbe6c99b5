#!/usr/bin/env python3
"""Throughput of NairnMPM's explicit time step on GB300, in particle-steps/s.

Workload (default): the 3D elastic-plastic Taylor impact -- von Mises with
linear hardening (E=200 GPa, nu=0.3, yield 300 MPa, Ep 2 GPa, rho 7.8 g/cm^3),
cylinder r=5 mm, L=25 mm at 200 m/s onto a rigid wall (zero normal velocity on
the wall node plane), 0.25 mm cells, 2x2x2 particles per cell (1,004,800
particles), uGIMP, USAVG, 2,000 steps.  Inputs are synthetic (seeded,
deterministic), built exactly as the reference's XML generator builds them.

One "step" = one explicit MPM step over all particles (P2G, grid update with
velocity BCs, strain/constitutive update, internal forces, momentum update,
G2P, second extrapolation and strain update, element reset).

The headline `value` is the plain single-run FP64 path -- the arithmetic of
the reference -- timed over a window in the middle of the 2,000-step run
(the run is advanced untimed to --window-start, default step 1,000, where the
plastic zone has grown; then W warm-up and K timed steps).  The reference arm
(--impl reference: the CPU restatement of the reference step, all host
threads) times the same window of the same run.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

"e2e" is the same FP64 step through the C ABI with the particle state in host
memory: the state stays in page-locked host memory and each step's kernels
read and write its columns in place over the host link (mpmgpu_step_host);
"e2e.copy" is the copying form (upload the state, step, download it).

The line also carries "mixed": the same window in the mixed-precision mode
(FP32 transfers, FP64 constitutive update) with its error against the FP64
path; "batched": 512 independent seeded 2D runs (2k-200k particles each)
advanced by one graph-captured batched step in mixed precision, against the
same runs on the plain single-run FP64 path, with the error of the batched
results against that path; "contact3d": the 3D two-material contact problem
(4.1 M particles, lCPDI) in FP64 and mixed precision; "contact3d_batched": 48
seeded contact runs of 20k-500k particles in one batched mixed step against
each run alone on the plain FP64 path; "served": a seeded request stream
through the continuous-batching server; and "batched_vs_plain", the ratio the
batched/served forms reach over the plain FP64 path at their stated error.

Under torchrun (N>1) every rank runs an independent replica of the workload
(the runs do not exchange data), so scaling is weak.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "nairn-mpm-fea_gb300", "python"))

METRIC = "particle-steps/s"
KERNEL_NAMES = ("p2g", "node_post", "strain_forces", "node_update", "g2p", "node_usl", "strain_last", "sort")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--radius", type=float, default=5.0)
    ap.add_argument("--length", type=float, default=25.0)
    ap.add_argument("--cell", type=float, default=0.25)
    ap.add_argument("--sort-interval", type=int, default=0,
                    help="cell-sort interval of the single-run measurements (0: autotuned over 1, 2, 4, 8)")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision window (and its archive leg)")
    ap.add_argument("--window-start", type=int, default=1000,
                    help="step at which the timed window opens (the run is advanced to it untimed)")
    ap.add_argument("--batch-runs", type=int, default=512,
                    help="runs of the batched measurement (0: skip it)")
    ap.add_argument("--batch-steps", type=int, default=100, help="timed steps of the batched measurement")
    ap.add_argument("--serve-requests", type=int, default=40,
                    help="requests of the served measurement, a prefix of the seeded 200-request stream (0: skip)")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0, help="HBM admission budget of the server")
    ap.add_argument("--contact-runs", type=int, default=48,
                    help="runs of the batched 3D contact instance mix (0: skip)")
    ap.add_argument("--contact-steps", type=int, default=40, help="timed steps of the batched contact measurement")
    ap.add_argument("--contact-normals", type=int, choices=(0, 1, 2, 5, 6), default=2,
                    help="contact normal method of the contact legs (2: average volume gradients; 6: logistic "
                         "regression, the reference's default)")
    ap.add_argument("--contact-serve-requests", type=int, default=32,
                    help="requests of the served 3D contact stream (0: skip)")
    ap.add_argument("--config3-steps", type=int, default=10,
                    help="timed steps of the 3D contact (config 3) measurement (0: skip)")
    ap.add_argument("--archive-steps", type=int, default=60,
                    help="steps of the archiving measurement on the headline workload (0: skip)")
    ap.add_argument("--archive-every", type=int, default=10, help="steps between archives")
    ap.add_argument("--xpic-steps", type=int, default=20,
                    help="timed steps of the XPIC/FMPM measurement on the headline workload (0: skip)")
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-reduction across ranks (torch.distributed when launched by torchrun)."""

    def __init__(self, ws, rank, local, backend):
        self.ws, self.rank = ws, rank
        self.pg = None
        if ws > 1:
            import torch
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            if backend == "nccl":
                torch.cuda.set_device(local)
            dist.init_process_group(backend=backend)
            self.dist = dist
            self.torch = torch
            self.dev = torch.device("cuda", local) if backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if self.ws == 1:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


def workload(args):
    from nairn_gb300 import model
    return model.taylor_3d(radius=args.radius, length=args.length, cell=args.cell, steps=2000)


TUNE_STEPS = 64  # real steps the sort-interval autotuner takes (2 rounds x 4 intervals x 8 steps)


def window_open(args) -> int:
    """Step the run is advanced to, untimed, before the warm-up steps."""
    return max(args.window_start, TUNE_STEPS if args.sort_interval <= 0 else 0)


def window_first(args) -> int:
    """Steps completed when the timed window opens."""
    return window_open(args) + args.warmup


def workload_config(args, m, extra=None):
    cfg = {"workload": "3D elastic-plastic Taylor impact (von Mises, linear hardening), r=%g mm, L=%g mm, "
                       "%g mm cells, 2x2x2 particles/cell, uGIMP, USAVG, 2,000 steps" % (args.radius, args.length,
                                                                                         args.cell),
           "particles": m.n, "grid_nodes": m.grid.nnodes, "material": "IsoPlasticity + LinearHardening",
           "timestep_s": m.options["timestep"],
           "timed_window": "steps %d-%d of the run (advanced untimed to step %d, then %d warm-up steps)" % (
               window_first(args) + 1, window_first(args) + args.steps, window_open(args), args.warmup),
           "l2": ("particle state %.0f MB vs 129 MB L2: inputs larger than L2, no flush needed"
                  if m.n * 39 * 8 > 129e6 else "particle state %.0f MB fits in L2") % (m.n * 39 * 8 / 1e6),
           "parallelism": "replicas" if int(os.environ.get("WORLD_SIZE", "1")) > 1 else "single GPU"}
    if extra:
        cfg.update(extra)
    return cfg


# ---------------------------------------------------------------------------
# roofline byte model: algorithmic bytes per launch of each kernel (each
# particle column touched once, each node column of the active grid once)
# ---------------------------------------------------------------------------
def algorithmic_bytes(m, nodes_active: int) -> dict:
    dim = m.grid.dim
    d = 8
    vec = dim * d
    plastic = any(mm["type"] == 9 for mm in m.materials)
    ten = (6 if dim == 3 else 4) * d
    F = (9 if dim == 3 else 5) * d
    state = F + ten + (d + ten + d + d if plastic else 0) + d  # F, sigma, (P, eps_p, alpha, plastic E), work
    elem, mat = 4, 4
    xi = dim * d
    lp = dim * d
    n = m.n
    per_particle = {
        "p2g": elem + vec + d + vec + lp + xi,                 # read elem,x,m,v,lp; write xi
        "strain_forces": elem + xi + lp + mat + d + 2 * state,  # read geometry + state, write state
        "g2p": elem + xi + lp + 2 * vec + d + 2 * vec,          # read v,x,m; write v,x
        "strain_last": elem + xi + lp + mat + vec + 2 * state + elem,
        "node_post": 0, "node_update": 0, "node_usl": 0, "sort": 0,
    }
    per_node = {
        "p2g": 2 * (d + vec),                 # mass, momentum accumulated (read-modify-write)
        "node_post": 1 + 4 + (d + vec) + 2 * vec,
        "strain_forces": vec + 2 * vec,       # velocity gather, force accumulation
        "node_update": 1 + 4 + d + 2 * vec + 3 * vec,
        "g2p": d + 2 * vec + 2 * vec,         # v, f, m gathered; second momentum accumulated
        "node_usl": 1 + 4 + d + vec + 2 * vec,
        "strain_last": vec,
        "sort": 0,
    }
    return {k: n * per_particle[k] + nodes_active * per_node[k] for k in per_particle}


def host_link_bytes(m) -> tuple[int, int]:
    """Bytes one step on host-resident state (mpmgpu_step_host) moves over the
    host link: the host columns each kernel reads, and those it writes
    (algorithmic, each column once per kernel; the natural coordinates stay
    on the device)."""
    dim = m.grid.dim
    d = 8
    vec = dim * d
    plastic = any(mm["type"] == 9 for mm in m.materials)
    ten = (6 if dim == 3 else 4) * d
    F = (9 if dim == 3 else 5) * d
    state = F + ten + (d + ten + d + d if plastic else 0) + d
    elem, mat, lp = 4, 4, dim * d
    reads = ((elem + vec + d + vec + lp)            # p2g: elem, x, m, v, lp
             + (elem + lp + mat + d + state)        # strain_forces: geometry, state
             + (elem + lp + 2 * vec + d)            # g2p: x, v, m
             + (elem + lp + mat + vec + state))     # strain_last: geometry, x, state
    writes = state + 2 * vec + (state + elem)       # strain_forces; g2p x, v; strain_last state, elem
    return m.n * reads, m.n * writes


def active_nodes(m) -> int:
    """Nodes of the cells that hold particles (the extrapolation support at t=0)."""
    import numpy as np
    g = m.grid
    e = np.unique(m.particles["elem"])
    col = e % g.nx
    row = (e // g.nx) % g.ny
    zr = e // (g.nx * g.ny)
    nodes = set()
    for dz in (0, 1) if g.dim == 3 else (0,):
        for dy in (0, 1):
            for dx in (0, 1):
                nodes.update((((zr + dz) * (g.ny + 1) + row + dy) * (g.nx + 1) + col + dx).tolist())
    return len(nodes)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profiles(kernel: str, n_particles: int, precision: int):
    """Per-launch DRAM bytes of the kernel in the given precision from the
    committed ncu summary, scaled to this size."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        d = json.load(fh)
    k = d.get("fp64_kernels" if precision == 0 else "kernels", {}).get(kernel)
    if not k:
        return None
    return k["dram_bytes_per_launch"] * n_particles / d["particles"]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        with open(self.path) as fh:
            for line in fh:
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax.append(float(f[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_baseline(m, p, first_step: int, seconds: float):
    """The CPU restatement of the reference step (oracle port), all host
    threads, on a bounded sample of the same workload: steps from the particle
    state p, which is the state after `first_step` steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_lib
    from nairn_gb300 import abi
    threads = os.cpu_count() or 1
    dt = m.options["timestep"]
    p = abi.copy_particles(p)
    t0 = time.perf_counter()
    oracle_lib.run(m, p, 1, first_step * dt, nthreads=threads)
    t1 = time.perf_counter() - t0
    steps = max(1, min(200, int(seconds / max(t1, 1e-6))))
    t0 = time.perf_counter()
    oracle_lib.run(m, p, steps, (first_step + 1) * dt, nthreads=threads)
    el = time.perf_counter() - t0
    return {"value": m.n * steps / el, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"steps {first_step + 2}-{first_step + 1 + steps} (after 1 untimed) of the same {m.n}-particle "
                      f"run, from its state after {first_step} steps, {threads} OpenMP threads, FP64"}


def run_reference(args, ws, rank, local):
    """The reference arm: the CPU restatement of the reference's step (the
    reference itself is C++ built for this container's host, not for the GPU
    host), all host threads, FP64, on the same window of the same run as the
    GPU arm: advanced untimed to the window, W warm-up steps, K timed steps."""
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_lib
    from nairn_gb300 import abi
    m = workload(args)
    threads = os.cpu_count() or 1
    dt = m.options["timestep"]
    p = abi.copy_particles(m.particles)
    t_adv = time.perf_counter()
    oracle_lib.run(m, p, window_open(args), 0.0, nthreads=threads)
    oracle_lib.run(m, p, args.warmup, window_open(args) * dt, nthreads=threads)
    t_adv = time.perf_counter() - t_adv
    k = max(1, args.steps)
    t0 = time.perf_counter()
    oracle_lib.run(m, p, k, window_first(args) * dt, nthreads=threads)
    el = time.perf_counter() - t0
    value = m.n * k / el
    b = {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
         "sample": "steps %d-%d of the %d-particle run (advanced untimed to step %d in %.0f s), %d OpenMP "
                   "threads, FP64" % (window_first(args) + 1, window_first(args) + k, m.n, window_first(args), t_adv,
                                      threads)}
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": k,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / k, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference", "config": workload_config(args, m),
            "cpu_baseline": b, "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def window_run(args, m, dist, precision: int, local: int):
    """The run advanced untimed to the window (the sort interval autotuned
    on its last TUNE_STEPS steps), W warm-up steps, then K steps timed with
    CUDA events on the context stream -- nothing else is recorded in that
    region -- and a second pass of K steps with per-kernel event pairs that
    gives the kernel split.  Returns the run (still open), its timings and
    the state at the end."""
    from nairn_gb300 import gpu
    si = args.sort_interval
    run = gpu.GpuRun(m, sort_interval=si if si > 0 else 8, precision=precision)
    run.upload(m.particles)
    if si <= 0:
        run.step(window_open(args) - TUNE_STEPS)
        si, _ = run.autotune_sort(16)
    else:
        run.step(window_open(args))
    run.step(args.warmup)
    launches0 = run.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    dist.barrier()
    ms = run.step_timed(args.steps)
    dist.barrier()
    clk = clocks.stop()
    launches = run.launch_count() - launches0
    run.set_profiling(True)
    ms_prof = run.step_timed(args.steps)
    prof = run.profile()
    run.set_profiling(False)
    final = run.download(m.particles)
    return run, {"ms": ms, "prof": prof, "ms_profiled_pass": ms_prof, "launches": launches, "clocks": clk,
                 "sort_interval": si, "steps_done": window_first(args) + 2 * args.steps}, final


def state_error(a: dict, b: dict, dim: int) -> dict:
    """Relative L2 of positions, velocities and stresses of a against b."""
    import numpy as np

    def rel(keys):
        x = np.concatenate([a[k] for k in keys])
        y = np.concatenate([b[k] for k in keys])
        return float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))

    ax = ("x", "y", "z")[:dim]
    vx = ("vx", "vy", "vz")[:dim]
    sx = ("sxx", "syy", "szz", "sxy") + (("sxz", "syz") if dim == 3 else ())
    return {"pos": rel(ax), "vel": rel(vx), "stress": rel(sx)}


def batched_measurement(args, dist, local):
    """The batched form: `batch_runs` independent seeded 2D plane-strain runs
    (2k-200k particles log-uniform, 50/50 elastic / von Mises, E 0.1-200 GPa,
    velocity fields 0.1-10 m/s, 500 steps each, uGIMP, USAVG) resident together
    and advanced by one graph-captured batched step in mixed precision, block
    size and sort interval picked by the autotuner.  Beside it: the same runs
    on the plain single-run FP64 path (every 16th run, the same steps) and the
    error of each sampled batched result against that path."""
    import numpy as np
    from nairn_gb300 import gpu, model
    ms = model.batch_models(args.batch_runs, seed=2024)
    n = sum(m.n for m in ms)
    b = gpu.GpuBatch.for_models(ms, precision=1)
    ids = [b.add(m) for m in ms]
    b.step(max(3, args.warmup))
    blk, si, _ = b.autotune(8)
    k = args.batch_steps
    l0 = b.info()["launches"]
    clocks = ClockSampler(local)
    clocks.start()
    dist.barrier()
    ms_b = b.step_timed(k)
    dist.barrier()
    clk = clocks.stop()
    info = b.info()
    done = b.state(ids[0])[1]
    value = dist.sum(float(n)) * k / (dist.max(ms_b) / 1e3)
    # the plain single-run FP64 path on a sample of the same runs, same steps
    sample = list(range(0, len(ms), 16))
    plain_ms, plain_ps, errs = 0.0, 0, []
    for j in sample:
        m = ms[j]
        r = gpu.GpuRun(m)
        r.upload(m.particles)
        r.step(done - k)
        plain_ms += r.step_timed(k)
        plain_ps += m.n * k
        alone = r.download(m.particles)
        r.close()
        errs.append(state_error(b.download(ids[j]), alone, 2))
    b.close()
    plain_value = plain_ps / (plain_ms / 1e3)
    # the same batch in FP64 (separates the batching gain from the precision gain)
    b64 = gpu.GpuBatch.for_models(ms, precision=0)
    for m in ms:
        b64.add(m)
    b64.step(max(3, args.warmup))
    k64 = max(1, k // 4)
    ms64 = b64.step_timed(k64)
    b64.close()
    emax = {q: max(e[q] for e in errs) for q in ("pos", "vel", "stress")}
    return {"value": value, "unit": METRIC, "ms_per_step": ms_b / k, "steps": k, "dtype": "mixed",
            "config": {"workload": "%d independent 2D plane-strain runs, 2k-200k particles each (log-uniform, "
                                   "seed 2024), 50/50 elastic / von Mises + linear hardening, uGIMP, USAVG, "
                                   "500 steps each; one graph-captured batched step" % len(ms),
                       "particles": n, "grid_nodes": info["nodes_used"], "runs": len(ms),
                       "autotuned": {"block": blk, "sort_interval": si},
                       "timed_window": "steps %d-%d of each run" % (done - k + 1, done),
                       "l2": "batch state %.1f GB vs 129 MB L2: no flush needed" % (n * 39 * 8 / 1e9)},
            "gpu_launches": info["launches"] - l0, "clocks": clk,
            "plain_fp64_same_runs": {"value": plain_value, "unit": METRIC, "runs": len(sample),
                                     "sample": "every 16th run alone on the single-run FP64 path, "
                                               "same %d steps (small runs fit in L2: favours this path)" % k},
            "speedup_vs_plain_fp64": value / plain_value,
            "fp64_batch": {"value": dist.sum(float(n)) * k64 / (dist.max(ms64) / 1e3), "steps": k64},
            "error_vs_plain_fp64": dict(emax, statistic="max over the %d sampled runs" % len(sample),
                                        target="<= 1e-5 relative L2")}


def served_measurement(args, dist):
    """The served form: a seeded Poisson stream (20 requests/s) of independent
    2D/3D elastic-plastic runs, 10k-2M particles (log-uniform), 200-2,000 steps,
    submitted at their arrival times to the C++ serving loop (continuous
    batching, HBM admission budget, mixed precision).  Reports throughput and
    p50/p99 completion latency, beside every 5th request run alone on the plain
    single-run FP64 path (20 timed steps, scaled to its step count)."""
    import numpy as np
    from nairn_gb300 import gpu, model
    params = model.serve_request_params(200, seed=77)[:args.serve_requests]
    ms = model.serve_models(params)

    def serve(cap, order, slowdown=0.0):
        srv = gpu.GpuServer(model.USAVG, model.SHAPE_UGIMP, 1, hbm_budget_bytes=int(args.serve_budget_gb * 1e9),
                            max_runs=256, steps_per_round=10, frac_3d=0.5, max_resident_particles=cap, order=order,
                            slowdown_target=slowdown)
        dist.barrier()
        t0 = time.perf_counter()
        ids = []
        for (t_arr, _, _), m in zip(params, ms):
            delay = t_arr - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            ids.append(srv.submit(m))
        srv.drain(3600)
        wall = time.perf_counter() - t0
        infos = [srv.poll(r) for r in ids]
        st = srv.stats()
        srv.close()
        return wall, infos, st

    # latency policy: the deadline order (least work first; admitted only while
    # the running requests' predicted latency stays within 4x their time alone)
    wall_l, infos_l, _ = serve(0, "deadline", 4.0)
    lat_l = np.array([i["total_ms"] for i in infos_l])
    # throughput policy: every request admitted on arrival (the headline of this section)
    wall, infos, st = serve(0, "fifo")
    lat = np.array([i["total_ms"] for i in infos])
    qms = np.array([i["queue_ms"] for i in infos])
    work = float(sum(m.n * m.nsteps for m in ms))
    # each sampled request alone on the plain single-run FP64 path
    alone, ratio, ratio_l, alone_ps, alone_s = [], [], [], 0.0, 0.0
    for j in range(0, len(ms), 5):
        m = ms[j]
        t1 = time.perf_counter()
        r = gpu.GpuRun(m)
        r.upload(m.particles)
        r.step(2)
        k = 20
        step_ms = r.step_timed(k) / k
        r.close()
        setup_ms = 1e3 * (time.perf_counter() - t1) - step_ms * (k + 2)
        a = max(setup_ms, 0.0) + step_ms * m.nsteps
        alone.append(a)
        ratio.append(infos[j]["total_ms"] / a)
        ratio_l.append(infos_l[j]["total_ms"] / a)
        alone_ps += m.n * m.nsteps
        alone_s += a / 1e3
    return {"value": work / wall, "unit": METRIC, "requests": len(ms), "completed": st["completed"],
            "failed": st["failed"], "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "queue_p50_ms": float(np.percentile(qms, 50)), "wall_s": wall, "particle_steps": work, "dtype": "mixed",
            "config": {"workload": "seeded Poisson(20/s) stream, 2D/3D elastic-plastic blocks, 10k-2M particles "
                                   "(log-uniform), 200-2000 steps, uGIMP, USAVG; first %d of 200 requests" % len(ms),
                       "policy": "every request admitted on arrival (FIFO, no resident cap)",
                       "hbm_budget_gb": args.serve_budget_gb, "reserved_gb": st["reserved_bytes"] / 1e9,
                       "steps_per_round": 10, "rounds": st["rounds"]},
            "alone_plain_fp64": {"p50_ms": float(np.percentile(alone, 50)), "p99_ms": float(np.percentile(alone, 99)),
                                 "throughput": alone_ps / alone_s, "unit": METRIC, "requests": len(alone),
                                 "served_over_alone_latency_p50": float(np.percentile(ratio, 50)),
                                 "served_over_alone_latency_max": float(np.max(ratio)),
                                 "sample": "every 5th request alone: setup + 20 timed steps scaled to its steps"},
            "speedup_vs_plain_fp64": (work / wall) / (alone_ps / alone_s),
            "latency_policy": {"value": work / wall_l, "p50_ms": float(np.percentile(lat_l, 50)),
                               "p99_ms": float(np.percentile(lat_l, 99)),
                               "p99_over_alone_p99": float(np.percentile(lat_l, 99) / np.percentile(alone, 99)),
                               "served_over_alone_latency_p50": float(np.percentile(ratio_l, 50)),
                               "served_over_alone_latency_max": float(np.max(ratio_l)),
                               "speedup_vs_plain_fp64": (work / wall_l) / (alone_ps / alone_s),
                               "policy": "deadline order: least work first, a request admitted only while its "
                                         "dimension's resident particles stay within the load at which the online "
                                         "step-time model a + b x resident particles reaches 90% of its asymptotic "
                                         "throughput, and every running request's predicted latency within 4x its "
                                         "predicted time alone"}}


def contact_served_measurement(args, dist):
    """The served form on the 3D contact instance mix: a seeded Poisson stream
    (20 requests/s) of two-material contact runs of the contact_3d form
    (20k-500k particles, 200-1,500 steps), submitted at their arrival times to
    the serving loop (3D lCPDI batch, two material fields, mixed precision).
    Beside it: every 4th request alone on the plain single-run FP64 path."""
    import numpy as np
    from nairn_gb300 import gpu, model
    n_req = args.contact_serve_requests
    rng = np.random.default_rng(404)
    arrivals = np.cumsum(rng.exponential(1. / 20., n_req))
    steps = rng.integers(200, 1501, n_req)
    ms = model.contact_models(n_req, seed=404, steps=1500, normals=args.contact_normals)
    for m, k in zip(ms, steps):
        m.nsteps = int(k)
    srv = gpu.GpuServer(model.USAVG, model.SHAPE_LCPDI, 1, hbm_budget_bytes=int(args.serve_budget_gb * 1e9),
                        max_runs=256, steps_per_round=10, frac_3d=1.0, nodes_per_particle=1.5, max_fields=2,
                        lr_links=64 if args.contact_normals >= 5 else 0)
    dist.barrier()
    t0 = time.perf_counter()
    ids = []
    for t_arr, m in zip(arrivals, ms):
        delay = t_arr - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        ids.append(srv.submit(m))
    srv.drain(3600)
    wall = time.perf_counter() - t0
    infos = [srv.poll(r) for r in ids]
    st = srv.stats()
    srv.close()
    lat = np.array([i["total_ms"] for i in infos])
    work = float(sum(m.n * m.nsteps for m in ms))
    alone_ps, alone_s, alone = 0.0, 0.0, []
    for j in range(0, len(ms), 4):
        m = ms[j]
        t1 = time.perf_counter()
        r = gpu.GpuRun(m)
        r.upload(m.particles)
        r.step(2)
        k = 10
        step_ms = r.step_timed(k) / k
        r.close()
        setup_ms = 1e3 * (time.perf_counter() - t1) - step_ms * (k + 2)
        a = max(setup_ms, 0.0) + step_ms * m.nsteps
        alone.append(a)
        alone_ps += m.n * m.nsteps
        alone_s += a / 1e3
    return {"value": work / wall, "unit": METRIC, "requests": n_req, "completed": st["completed"],
            "failed": st["failed"], "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "wall_s": wall, "particle_steps": work, "dtype": "mixed",
            "config": {"workload": "seeded Poisson(20/s) stream of %d 3D two-material contact runs (Neo-Hookean "
                                   "block on elastic plate, Coulomb 0.3, lCPDI, 0.5 mm cells, 8 particles/cell, "
                                   "USAVG), 20k-500k particles, 200-1500 steps (seed 404)" % n_req,
                       "policy": "every request admitted on arrival (FIFO)", "hbm_budget_gb": args.serve_budget_gb,
                       "steps_per_round": 10, "rounds": st["rounds"], "normals": args.contact_normals},
            "alone_plain_fp64": {"throughput": alone_ps / alone_s, "unit": METRIC, "requests": len(alone),
                                 "p50_ms": float(np.percentile(alone, 50)), "p99_ms": float(np.percentile(alone, 99)),
                                 "sample": "every 4th request alone: setup + 10 timed steps scaled to its steps"},
            "speedup_vs_plain_fp64": (work / wall) / (alone_ps / alone_s)}


ARCHIVE_ORDER = "iYYYYYNYNYNNNYNNNN"  # position, velocity, stress, strain, plastic strain, energies, history


def archive_measurement(args, run, m, dist):
    """The headline run taking a NairnMPM archive (the particle records of
    ArchiveData::ArchiveResults) every `archive_every` steps: without
    archives, with mpmgpu_archive_records (pack, copy, wait) and with
    mpmgpu_archive_records_async (the copy to pinned host memory overlaps the
    following steps).  Host wall time around whole step sequences."""
    import numpy as np
    from nairn_gb300 import gpu
    L = gpu.lib()
    rec = int(L.mpmgpu_archive_record_size(m.grid.dim, ARCHIVE_ORDER.encode()))
    buf = np.empty(m.n * rec, dtype=np.uint8)
    held = gpu.pin({"records": buf})
    every, total = max(1, args.archive_every), max(args.archive_every, args.archive_steps)
    total -= total % every

    def timed(mode):
        run.step(1)
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(total // every):
            run.step(every)
            if mode == "sync":
                run.archive_records(ARCHIVE_ORDER)
            elif mode == "async":
                run.archive_records_async(ARCHIVE_ORDER, buf)
        run.archive_wait()
        t = time.perf_counter() - t0
        dist.barrier()
        return dist.max(t) * 1e3 / total

    out = {"every": every, "steps": total, "order": ARCHIVE_ORDER, "record_bytes": rec,
           "archive_bytes": m.n * rec}
    for mode in ("none", "sync", "async"):
        out[mode + "_ms_per_step"] = timed(mode)
    gpu.unpin(held)
    out["sync_overhead"] = out["sync_ms_per_step"] / out["none_ms_per_step"] - 1.
    out["async_overhead"] = out["async_ms_per_step"] / out["none_ms_per_step"] - 1.
    return out


def xpic_measurement(args, dist, sort_interval: int, precision: int):
    """The headline workload with the PeriodicXPIC custom task on every step:
    XPIC(k) and FMPM(k) grid-to-particle updates (each order k > 1 adds k - 1
    particle passes to the particle update, FMPM also to both strain
    updates).  CUDA events around the timed steps, as the headline."""
    from nairn_gb300 import gpu, model
    out = {"workload": "the headline Taylor impact with PeriodicXPIC on every step", "steps": args.xpic_steps,
           "sort_interval": sort_interval, "dtype": "mixed" if precision else "f64"}
    total = dist.sum(1.)
    for order, fmpm in ((1, 0), (2, 0), (4, 0), (2, 1), (4, 1)):
        m = model.taylor_3d(radius=args.radius, length=args.length, cell=args.cell,
                            steps=args.warmup + args.xpic_steps, xpic=(order, fmpm, 1))
        run = gpu.GpuRun(m, sort_interval=sort_interval, precision=precision)
        run.upload(m.particles)
        run.step(args.warmup)
        dist.barrier()
        ms = dist.max(run.step_timed(args.xpic_steps))
        run.close()
        name = ("FMPM(%d)" if fmpm else "XPIC(%d)") % order
        out[name] = {"ms_per_step": ms / args.xpic_steps,
                     "particle_steps_per_s": total * m.n * args.xpic_steps / (ms / 1e3)}
    return out


def config3_measurement(args, dist, local):
    """The 3D two-material contact form: a Neo-Hookean block (G 10 MPa, K 50 MPa,
    rho 1.1) pressed and sliding (4 m/s down, 4 m/s along) on an elastic plate
    (70 GPa, 0.33, 2.7) whose base is held, Coulomb friction 0.3, lCPDI, 0.5 mm
    cells, 2x2x2 particles per cell (4,136,960 particles), USAVG; plain FP64
    and mixed precision on the same steps, with the mixed state's error."""
    from nairn_gb300 import gpu, model
    m = model.contact_3d(plate=(128, 128, 30), block=(40, 40, 16), block_x0=22.0, block_y0=22.0, cell=0.5,
                         v=(4000., 0., -4000.), steps=1500, gimp="lCPDI", friction=0.3, normals=args.contact_normals)
    k = args.config3_steps
    out, finals = {}, {}
    for prec in (0, 1):
        r = gpu.GpuRun(m, precision=prec, sort_interval=max(1, args.sort_interval))
        r.upload(m.particles)
        r.step(3)
        si = args.sort_interval
        if si <= 0:
            si, _ = r.autotune_sort(8)  # 32 real steps
        l0 = r.launch_count()
        clocks = ClockSampler(local)
        clocks.start()
        dist.barrier()
        ms = r.step_timed(k)
        dist.barrier()
        clk = clocks.stop()
        out[prec] = {"value": dist.sum(float(m.n)) * k / (dist.max(ms) / 1e3), "ms_per_step": ms / k,
                     "gpu_launches": r.launch_count() - l0, "clocks": clk, "sort_interval": si}
        finals[prec] = r.download(m.particles)
        r.close()
    err = state_error(finals[1], finals[0], 3)
    return {"value": out[1]["value"], "unit": METRIC, "ms_per_step": out[1]["ms_per_step"], "dtype": "mixed",
            "steps": k, "gpu_launches": out[1]["gpu_launches"], "clocks": out[1]["clocks"],
            "config": {"workload": "3D multimaterial contact: Neo-Hookean block pressed and sliding on an elastic "
                                   "plate, Coulomb friction 0.3, lCPDI, 0.5 mm cells, 2x2x2 particles/cell, USAVG",
                       "particles": m.n, "grid_nodes": m.grid.nnodes, "material_fields": 2, "normals": args.contact_normals,
                       "sort_interval": out[1]["sort_interval"],
                       "l2": "particle state %.2f GB vs 129 MB L2: no flush needed" % (m.n * 42 * 8 / 1e9)},
            "plain_fp64": {"value": out[0]["value"], "ms_per_step": out[0]["ms_per_step"],
                           "sort_interval": out[0]["sort_interval"]},
            "speedup_vs_plain_fp64": out[1]["value"] / out[0]["value"],
            "error_vs_fp64_path": dict(err, steps=3 + (32 if args.sort_interval <= 0 else 0) + k,
                                       target="<= 1e-5 relative L2")}


def contact_batched_measurement(args, dist, local):
    """The batched form on the 3D contact instance mix: `contact_runs` seeded
    two-material contact runs of the contact_3d form (Neo-Hookean block pressed
    and sliding on an elastic plate, Coulomb friction 0.3, lCPDI, 0.5 mm cells,
    8 particles per cell), 20k-500k particles each (log-uniform), resident
    together and advanced by one graph-captured batched step in mixed
    precision, autotuned.  Beside it: every run alone on the plain single-run
    FP64 path (the same steps) and each batched result's error against it."""
    from nairn_gb300 import gpu, model
    ms = model.contact_models(args.contact_runs, seed=303, steps=1500, normals=args.contact_normals)
    n = sum(m.n for m in ms)
    b = gpu.GpuBatch.for_models(ms, precision=1)
    ids = [b.add(m) for m in ms]
    b.step(max(3, args.warmup))
    blk, si, _ = b.autotune(4)
    k = args.contact_steps
    l0 = b.info()["launches"]
    clocks = ClockSampler(local)
    clocks.start()
    dist.barrier()
    ms_b = b.step_timed(k)
    dist.barrier()
    clk = clocks.stop()
    info = b.info()
    done = b.state(ids[0])[1]
    value = dist.sum(float(n)) * k / (dist.max(ms_b) / 1e3)
    plain_ms, plain_ps, errs = 0.0, 0, []
    for j, m in enumerate(ms):
        r = gpu.GpuRun(m)
        r.upload(m.particles)
        r.step(done - k)
        plain_ms += r.step_timed(k)
        plain_ps += m.n * k
        alone = r.download(m.particles)
        r.close()
        errs.append(state_error(b.download(ids[j]), alone, 3))
    b.close()
    plain_value = plain_ps / (plain_ms / 1e3)
    emax = {q: max(e[q] for e in errs) for q in ("pos", "vel", "stress")}
    # the worst run's own sensitivity: its FP64 run with the initial velocities
    # perturbed by 1e-6 (relative, three seeds) against the unperturbed one --
    # a contact run near a threshold (a stick/slip or separation decision on a
    # near-zero quantity) moves by far more than 1e-6 there, in the reference too
    worst = max(range(len(ms)), key=lambda j: errs[j]["stress"])
    sens = sensitivity(ms[worst], done, 1e-6)
    return {"value": value, "unit": METRIC, "ms_per_step": ms_b / k, "steps": k, "dtype": "mixed",
            "config": {"workload": "%d independent 3D two-material contact runs (Neo-Hookean block on elastic "
                                   "plate, Coulomb 0.3, lCPDI, 0.5 mm cells, 8 particles/cell, USAVG), "
                                   "20k-500k particles each (log-uniform, seed 303); one graph-captured "
                                   "batched step" % len(ms),
                       "particles": n, "grid_nodes": info["nodes_used"], "runs": len(ms), "material_fields": 2, "normals": args.contact_normals,
                       "autotuned": {"block": blk, "sort_interval": si},
                       "timed_window": "steps %d-%d of each run" % (done - k + 1, done),
                       "l2": "batch state %.1f GB vs 129 MB L2: no flush needed" % (n * 42 * 8 / 1e9)},
            "gpu_launches": info["launches"] - l0, "clocks": clk,
            "plain_fp64_same_runs": {"value": plain_value, "unit": METRIC, "runs": len(ms),
                                     "sample": "every run alone on the single-run FP64 path, same %d steps" % k},
            "speedup_vs_plain_fp64": value / plain_value,
            "error_vs_plain_fp64": dict(emax, statistic="max over the %d runs" % len(ms),
                                        target="<= 1e-5 relative L2"),
            "worst_run_sensitivity": dict(sens, run=worst, particles=ms[worst].n,
                                          perturbation="initial velocities x (1 + 1e-6 N(0,1)), three seeds, "
                                                       "FP64 path, max relative L2 against the unperturbed run")}


def sensitivity(m, steps: int, eps: float) -> dict:
    """How far the FP64 single-run result of model m after `steps` steps moves
    when its initial velocities are perturbed by eps (relative, seeded normal
    noise): the largest relative L2 over three seeds, per quantity."""
    import numpy as np
    from nairn_gb300 import abi, gpu

    def final(seed):
        p = abi.copy_particles(m.particles)
        if seed:
            rng = np.random.default_rng(seed)
            for k in ("vx", "vy", "vz"):
                p[k] = p[k] * (1. + eps * rng.standard_normal(p[k].shape))
        r = gpu.GpuRun(m)
        r.upload(p)
        r.step(steps)
        out = r.download(m.particles)
        r.close()
        return out
    base = final(0)
    moves = [state_error(final(seed), base, m.grid.dim) for seed in (1, 2, 3)]
    return {q: max(e[q] for e in moves) for q in ("pos", "vel", "stress")}


def fp64_flops_from_profiles(kernel: str, n_particles: int):
    """FP64 flops per launch (2 per DFMA, 1 per DADD/DMUL) from the committed
    ncu instruction counts of the FP64 path, scaled to this particle count."""
    p = os.path.join(ROOT, "profiles", "ncu_fp64_ops.json")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        d = json.load(fh)
    k = d.get("kernels", {}).get(kernel)
    if not k:
        return None
    return k["fp64_flops_per_launch"] * n_particles / d["particles"]


def kernel_table(prof: dict, steps: int, bytes_model: dict, launches_of) -> dict:
    fams = {k: v for k, v in prof.items() if v > 0}
    total = sum(fams.values())
    return {k: {"ms_per_step": v / steps, "share": v / total,
                "algorithmic_GBps": (bytes_model.get(k, 0) / ((v / launches_of(k)) / 1e3) / 1e9)
                if bytes_model.get(k, 0) > 0 else None}
            for k, v in fams.items()}


def roofline_of(prof: dict, steps: int, sort_interval: int, m, nodes: int, fp64_peak_tflops, precision: int = 0):
    """HBM roofline of the dominant kernel (largest share of the profiled
    pass), and for the FP64 path its FP64-pipe roofline against the FP64 FMA
    rate measured on this GPU."""
    fams = {k: v for k, v in prof.items() if v > 0}
    dom = max(fams, key=fams.get)

    def launches_of(k):
        return steps if k != "sort" else max(1, steps // sort_interval)

    avg_ms = fams[dom] / launches_of(dom)
    bytes_model = algorithmic_bytes(m, nodes)
    peak, peak_kind = peaks()
    achieved = bytes_model[dom] / (avg_ms / 1e3) / 1e9
    roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": traffic_from_profiles(dom, m.n, precision), "algorithmic_bytes_per_launch": bytes_model[dom],
            "avg_launch_ms": avg_ms,
            "note": "per-launch time from CUDA events of a separate profiled pass over the same window"}
    fl = fp64_flops_from_profiles(dom, m.n)
    fp64 = None
    if fl is not None and fp64_peak_tflops:
        ach = fl / (avg_ms / 1e3) / 1e12
        fp64 = {"kernel": dom, "bound": "fp64", "achieved": ach, "peak": fp64_peak_tflops, "unit": "TFLOP/s",
                "frac": ach / fp64_peak_tflops, "flops_per_launch": fl,
                "peak_source": "measured in this run (mpmgpu_fp64_fma_rate: independent DFMA chains)",
                "flops_source": "ncu instruction counts (profiles/ncu_fp64_ops.json), scaled to this size"}
    return roof, fp64, kernel_table(prof, steps, bytes_model, launches_of)


def main():
    args = parse()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, ws, rank, local)
    import __graft_entry__
    __graft_entry__.build_library()
    dist = Dist(ws, rank, local, "nccl" if ws > 1 else "gloo")
    from nairn_gb300 import abi, gpu
    m = workload(args)
    n = m.n
    total_particles = dist.sum(float(n))
    fp64_peak = gpu.fma_rate(True)
    fp32_peak = gpu.fma_rate(False)
    nodes = active_nodes(m)

    # the headline: the plain FP64 path over the window
    run, head, final = window_run(args, m, dist, 0, local)
    ms_max = dist.max(head["ms"])
    value = total_particles * args.steps / (ms_max / 1e3)
    roof, roof64, kernels = roofline_of(head["prof"], args.steps, head["sort_interval"], m, nodes, fp64_peak)

    # end to end through the C ABI with host-resident particle state: every
    # step uploads the state from pinned host memory and downloads the result
    # the host keeps its FP64 columns in one block in the library's column
    # order, so each direction moves them in one copy
    # (the block in page-locked memory the driver allocated, mpmgpu_host_alloc)
    hb = gpu.HostBlock((len(abi.DEVICE_COLUMNS), n))
    host, block = abi.contiguous_particles(final, hb.array)
    pinned = gpu.pin({"mat": host["mat"], "elem": host["elem"]})
    pin_error = None if len(pinned) == 2 else gpu.lib().mpmgpu_last_error(None).decode()
    h2d = block.nbytes + host["mat"].nbytes + host["elem"].nbytes
    d2h = h2d
    ke = max(1, args.e2e_steps)
    run.upload(host)
    run.step(1)
    run.download_into(host)
    dist.barrier()
    split = {"upload": 0., "step": 0., "download": 0.}
    t0 = time.perf_counter()
    for _ in range(ke):
        a = time.perf_counter()
        run.upload(host)
        b = time.perf_counter()
        run.step(1)
        c = time.perf_counter()
        run.download_into(host)
        d = time.perf_counter()
        split["upload"] += b - a
        split["step"] += c - b
        split["download"] += d - c
    t_e2e = time.perf_counter() - t0
    dist.barrier()
    gpu.unpin(pinned)
    t_e2e = dist.max(t_e2e)
    e2e_copy_value = total_particles * ke / t_e2e

    # end to end on host-resident state (mpmgpu_step_host): the particle state
    # stays in page-locked host memory and the kernels read and write its
    # columns in place over the host link, so the link traffic overlaps their
    # arithmetic instead of preceding and following it; one call per step,
    # each returning when the step's results are in host memory
    hs = gpu.HostState(host)
    host = block = None
    hb.close()
    run.step_host(hs.particles, 1)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        run.step_host(hs.particles, 1)
    t_host = time.perf_counter() - t0
    dist.barrier()
    hs.close()
    t_host = dist.max(t_host)
    e2e_value = total_particles * ke / t_host
    link_read, link_write = host_link_bytes(m)
    run.close()

    # the mixed-precision mode over the same window, with its error against
    # the FP64 path at the same step
    archived, mixed_line = None, None
    if not args.no_mixed:
        mrun, mixed, mfinal = window_run(args, m, dist, 1, local)
        archived = archive_measurement(args, mrun, m, dist) if args.archive_steps > 0 else None
        mrun.close()
        mroof, _, mkernels = roofline_of(mixed["prof"], args.steps, mixed["sort_interval"], m, nodes, None, 1)
        err = state_error(mfinal, final, m.grid.dim)
        mixed_value = total_particles * args.steps / (dist.max(mixed["ms"]) / 1e3)
        mixed_line = {"value": mixed_value, "unit": METRIC, "ms_per_step": dist.max(mixed["ms"]) / args.steps,
                      "dtype": "mixed: f32 transfers, f64 constitutive", "sort_interval": mixed["sort_interval"],
                      "speedup_vs_fp64": mixed_value / value, "gpu_launches": mixed["launches"],
                      "clocks": mixed["clocks"], "roofline": mroof, "kernels": mkernels,
                      "error_vs_fp64_path": dict(err, steps=head["steps_done"],
                                                 note="relative L2 against the FP64 GPU path after the same "
                                                      "steps; that path matches the reference within 1e-10")}

    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, m, {"sort_interval": head["sort_interval"],
                                                "sort_interval_autotuned": args.sort_interval <= 0,
                                                "active_nodes_t0": nodes, "precision": "fp64"}),
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": link_read * ws,
                    "d2h_bytes_per_step": link_write * ws, "steps": ke, "ms_per_call": 1e3 * t_host / ke,
                    "form": "host-resident state: mpmgpu_step_host, one call per step",
                    "note": "FP64 path; the particle state (%.0f MB) stays in page-locked host memory the driver "
                            "allocated (mpmgpu_host_alloc) and every step's kernels read and write its columns in "
                            "place over the host link; the byte counts are the host columns the kernels read and "
                            "write (algorithmic: each column once per kernel)" % (h2d / 1e6),
                    "copy": {"value": e2e_copy_value, "unit": METRIC, "h2d_bytes_per_step": h2d * ws,
                             "d2h_bytes_per_step": d2h * ws, "steps": ke,
                             "ms_per_call": {k: 1e3 * v / ke for k, v in split.items()},
                             "host_buffers_page_locked": pin_error is None, "page_lock_error": pin_error,
                             "form": "mpmgpu_upload_particles + mpmgpu_step + mpmgpu_download_particles per step",
                             "note": "per step: upload the full particle state from pinned host memory (FP64 "
                                     "columns in one block the driver allocated), one step, download it again"}},
            "gpu_launches": head["launches"], "roofline": roof, "roofline_fp64": roof64, "kernels": kernels,
            "clocks": head["clocks"],
            "measured_peaks": {"fp64_fma_tflops": fp64_peak, "fp32_fma_tflops": fp32_peak,
                               "ratio_fp32_to_fp64": fp32_peak / fp64_peak},
            "mixed": mixed_line}
    if archived:
        line["archived"] = archived
    if args.xpic_steps > 0:
        line["xpic"] = xpic_measurement(args, dist, head["sort_interval"], 1)
    if args.config3_steps > 0:
        line["contact3d"] = config3_measurement(args, dist, local)
    if args.contact_runs > 0:
        line["contact3d_batched"] = contact_batched_measurement(args, dist, local)
    if args.batch_runs > 0:
        line["batched"] = batched_measurement(args, dist, local)
    if args.serve_requests > 0:
        line["served"] = served_measurement(args, dist)
    if args.contact_serve_requests > 0:
        line["contact3d_served"] = contact_served_measurement(args, dist)
    bvp = {}
    for key, what in (("batched", "512 independent 2D runs in one batched mixed step"),
                      ("contact3d_batched", "48 independent 3D contact runs in one batched mixed step"),
                      ("served", "served 2D/3D elastic-plastic stream (mixed)"),
                      ("contact3d_served", "served 3D contact stream (mixed)")):
        if key in line:
            r = line[key]
            bvp[key] = {"form": what, "speedup_vs_plain_fp64": r["speedup_vs_plain_fp64"],
                        "error_vs_plain_fp64": r.get("error_vs_plain_fp64")}
    if bvp:
        line["batched_vs_plain"] = dict(bvp, target=">= 3x the plain single-run FP64 path at <= 1e-5 relative "
                                                    "stress error")
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(m, final, head["steps_done"], args.cpu_seconds)
    dist.close()
    if rank == 0:
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
