"""Run one synthetic workload on the GPU through the C ABI and print its timing.

    python -m nairn_gb300.run taylor --precision mixed --steps 4
    python -m nairn_gb300.run cantilever --nx 100 --ny 20 --steps 200
    python -m nairn_gb300.run batch --runs 64 --steps 20
    python -m nairn_gb300.run contact3d --plate 64 64 16 --block 20 20 8 --precision mixed

Workloads: `cantilever` (2D elastic beam), `taylor` (3D elastic-plastic
Taylor impact), `block2d` / `block3d` (one block of the batched population's
form), `batch` (the first --runs runs of the seeded 512-run 2D population in
one batch), `contact3d` (Neo-Hookean block pressed and sliding on an elastic
plate, lCPDI, multimaterial contact), `contact_batch` (the first --runs runs of
the seeded 3D contact population in one batch).  Used for profiling single kernels and for quick checks; the
measurement of record is bench.py.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m nairn_gb300.run")
    ap.add_argument("workload", choices=("cantilever", "taylor", "block2d", "block3d", "batch", "contact3d",
                                         "contact_batch"))
    ap.add_argument("--precision", choices=("fp64", "mixed"), default="fp64")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--sort-interval", type=int, default=1)
    ap.add_argument("--nx", type=int, default=100)
    ap.add_argument("--ny", type=int, default=20)
    ap.add_argument("--radius", type=float, default=5.0)
    ap.add_argument("--length", type=float, default=25.0)
    ap.add_argument("--cell", type=float, default=0.25)
    ap.add_argument("--cells", type=int, default=64, help="block edge in cells (block2d/block3d)")
    ap.add_argument("--runs", type=int, default=64, help="runs of the batch workloads")
    ap.add_argument("--plate", type=int, nargs=3, default=(64, 64, 16), help="plate cells (contact3d)")
    ap.add_argument("--block", type=int, nargs=3, default=(20, 20, 8), help="block cells (contact3d)")
    ap.add_argument("--normals", type=int, choices=(0, 1, 2, 5, 6), default=2,
                    help="contact normal method (contact3d): 0-2 volume gradients, 5/6 regressions")
    ap.add_argument("--gap", type=float, default=0.0, help="block-to-plate gap in mm (contact3d)")
    ap.add_argument("--xpic", type=int, default=0, help="PeriodicXPIC order (cantilever, taylor; 0: FLIP)")
    ap.add_argument("--fmpm", action="store_true", help="FMPM(k) instead of XPIC(k)")
    ap.add_argument("--xpic-period", type=int, default=1, help="PeriodicXPIC periodicSteps")
    ap.add_argument("--p2g", choices=("atomic", "deterministic", "untiled"), default="atomic",
                    help="node sums: atomic (shared-memory tiles in the mixed mode), deterministic, or untiled "
                         "(every particle-node pair straight to the node columns)")
    ap.add_argument("--profile", action="store_true", help="per-kernel ms of the timed steps (single runs)")
    a = ap.parse_args(argv)
    from nairn_gb300 import gpu, model
    prec = 1 if a.precision == "mixed" else 0
    total = a.steps + a.warmup
    if a.workload in ("batch", "contact_batch"):
        if a.workload == "batch":
            ms = model.batch_models(512, seed=2024)[:a.runs]
        else:
            ms = model.contact_models(a.runs, seed=303, steps=1500, normals=a.normals)
        b = gpu.GpuBatch.for_models(ms, precision=prec, sort_interval=a.sort_interval)
        for m in ms:
            b.add(m)
        b.step(a.warmup)
        t = b.step_timed(a.steps)
        n = sum(m.n for m in ms)
        out = {"workload": a.workload, "runs": len(ms), "particles": n, "ms_per_step": t / a.steps,
               "particle_steps_per_s": n * a.steps / (t / 1e3), "info": b.info()}
        b.close()
    else:
        xp = (a.xpic, 1 if a.fmpm else 0, a.xpic_period) if a.xpic > 0 else None
        if a.workload == "cantilever":
            m = model.cantilever_2d(nx=a.nx, ny=a.ny, steps=total, xpic=xp)
        elif a.workload == "taylor":
            m = model.taylor_3d(radius=a.radius, length=a.length, cell=a.cell, steps=total, xpic=xp)
        elif a.workload == "block2d":
            m = model.block_2d(ncx=a.cells, ncy=a.cells, steps=total)
        elif a.workload == "contact3d":
            bx0 = 0.5 * (a.plate[0] - a.block[0]) * 0.5
            by0 = 0.5 * (a.plate[1] - a.block[1]) * 0.5
            m = model.contact_3d(plate=tuple(a.plate), block=tuple(a.block), block_x0=bx0, block_y0=by0, cell=0.5,
                                 v=(4000., 0., -4000.), steps=total, gimp="lCPDI", friction=0.3, normals=a.normals,
                                 gap=a.gap)
        else:
            m = model.block_3d(ncx=a.cells, ncy=a.cells, ncz=a.cells, steps=total)
        r = gpu.GpuRun(m, precision=prec, sort_interval=a.sort_interval,
                       p2g={"atomic": 0, "deterministic": 1, "untiled": 2}[a.p2g])
        r.upload(m.particles)
        r.step(a.warmup)
        if a.profile:
            r.set_profiling(True)
        t = r.step_timed(a.steps)
        out = {"workload": m.name, "particles": m.n, "ms_per_step": t / a.steps,
               "particle_steps_per_s": m.n * a.steps / (t / 1e3), "launches": r.launch_count()}
        if a.profile:
            out["kernels_ms_per_step"] = {k: round(v / a.steps, 4) for k, v in r.profile().items() if v > 0}
        r.close()
    out["precision"] = a.precision
    out["sort_interval"] = a.sort_interval
    out["p2g"] = a.p2g
    if a.xpic > 0:
        out["xpic"] = {"order": a.xpic, "fmpm": a.fmpm, "period": a.xpic_period}
    if a.workload == "contact3d":
        out["normals"] = a.normals
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
