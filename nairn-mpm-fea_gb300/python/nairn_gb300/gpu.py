"""Python binding of the C ABI in libnairn_mpm_gb300.so (include/nairn_mpm_gpu.h).

The library is the product: CUDA kernels plus the C ABI a NairnMPM host task
calls.  This module loads it in-tree (nairn-mpm-fea_gb300/lib/) and fails
loudly when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi
from .model import Model

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(os.path.dirname(HERE))
LIBPATH = os.path.join(PKG, "lib", "libnairn_mpm_gb300.so")

_lib = None


class GpuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise RuntimeError(f"{LIBPATH} is missing: build it with __graft_entry__.build()")
    L = C.CDLL(LIBPATH)
    P = C.POINTER
    L.mpmgpu_abi_version.restype = C.c_int
    L.mpmgpu_create.argtypes = [P(abi.MpmGpuGrid), P(abi.MpmGpuOptions), P(C.c_void_p)]
    L.mpmgpu_set_materials.argtypes = [C.c_void_p, P(abi.MpmGpuMaterial), C.c_int32]
    L.mpmgpu_set_contact.argtypes = [C.c_void_p, P(abi.MpmGpuContact)]
    L.mpmgpu_set_velocity_bcs.argtypes = [C.c_void_p, P(abi.MpmGpuVelBC), C.c_int32]
    L.mpmgpu_upload_particles.argtypes = [C.c_void_p, P(abi.MpmGpuParticles)]
    L.mpmgpu_step.argtypes = [C.c_void_p, C.c_int32, C.c_double]
    L.mpmgpu_step_host.argtypes = [C.c_void_p, C.POINTER(abi.MpmGpuParticles), C.c_int32, C.c_double]
    L.mpmgpu_download_particles.argtypes = [C.c_void_p, P(abi.MpmGpuParticles)]
    L.mpmgpu_last_error.argtypes = [C.c_void_p]
    L.mpmgpu_last_error.restype = C.c_char_p
    L.mpmgpu_destroy.argtypes = [C.c_void_p]
    L.mpmgpu_destroy.restype = None
    L.mpmgpu_profile.argtypes = [C.c_void_p, P(C.c_char_p), P(C.c_double), C.c_int32]
    L.mpmgpu_set_profiling.argtypes = [C.c_void_p, C.c_int32]
    L.mpmgpu_stream.argtypes = [C.c_void_p]
    L.mpmgpu_stream.restype = C.c_void_p
    L.mpmgpu_step_timed.argtypes = [C.c_void_p, C.c_int32, C.c_double, P(C.c_double)]
    L.mpmgpu_autotune_sort.argtypes = [C.c_void_p, C.c_int32, C.c_double, P(C.c_int32), P(C.c_double),
                                       P(C.c_int32)]
    L.mpmgpu_autotune_sort.restype = C.c_int
    L.mpmgpu_archive_record_size.argtypes = [C.c_int32, C.c_char_p]
    L.mpmgpu_archive_record_size.restype = C.c_int64
    L.mpmgpu_archive_records.argtypes = [C.c_void_p, C.c_char_p, C.c_double, C.c_void_p, C.c_int64]
    L.mpmgpu_archive_records.restype = C.c_int
    L.mpmgpu_archive_records_async.argtypes = [C.c_void_p, C.c_char_p, C.c_double, C.c_void_p, C.c_int64]
    L.mpmgpu_archive_records_async.restype = C.c_int
    L.mpmgpu_archive_wait.argtypes = [C.c_void_p]
    L.mpmgpu_archive_wait.restype = C.c_int
    L.mpmgpu_step_timed.restype = C.c_int
    L.mpmgpu_launch_count.argtypes = [C.c_void_p]
    L.mpmgpu_launch_count.restype = C.c_longlong
    L.mpmgpu_host_register.argtypes = [C.c_void_p, C.c_uint64]
    L.mpmgpu_host_register.restype = C.c_int
    L.mpmgpu_sort_by_cell.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
    L.mpmgpu_sort_by_cell.restype = C.c_int
    L.mpmgpu_sort_by_cell_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
    L.mpmgpu_sort_by_cell_noalloc.restype = C.c_int
    L.mpmgpu_host_unregister.argtypes = [C.c_void_p]
    L.mpmgpu_host_unregister.restype = C.c_int
    for f in ("mpmgpu_fp64_fma_rate", "mpmgpu_fp32_fma_rate"):
        getattr(L, f).argtypes = [C.c_int32, P(C.c_double), P(C.c_double)]
        getattr(L, f).restype = C.c_int
    VP = C.c_void_p
    batch_sigs = {
        "mpmgpu_batch_bytes": ([P(abi.MpmGpuBatchOptions)], C.c_int64),
        "mpmgpu_batch_create": ([P(abi.MpmGpuBatchOptions), P(VP)], C.c_int),
        "mpmgpu_batch_add_run": ([VP, P(abi.MpmGpuGrid), P(abi.MpmGpuMaterial), C.c_int32, P(abi.MpmGpuVelBC),
                                  C.c_int32, P(abi.MpmGpuContact), P(abi.MpmGpuParticles), C.c_double, C.c_int32,
                                  P(C.c_int32)], C.c_int),
        "mpmgpu_batch_step": ([VP, C.c_int32], C.c_int),
        "mpmgpu_batch_step_timed": ([VP, C.c_int32, P(C.c_double)], C.c_int),
        "mpmgpu_batch_run_state": ([VP, C.c_int32, P(C.c_int32), P(C.c_int32)], C.c_int),
        "mpmgpu_batch_download_run": ([VP, C.c_int32, P(abi.MpmGpuParticles)], C.c_int),
        "mpmgpu_batch_remove_run": ([VP, C.c_int32, P(abi.MpmGpuParticles)], C.c_int),
        "mpmgpu_batch_set_tuning": ([VP, C.c_int32, C.c_int32], C.c_int),
        "mpmgpu_batch_autotune": ([VP, C.c_int32, P(C.c_int32), P(C.c_int32), P(C.c_double)], C.c_int),
        "mpmgpu_batch_info": ([VP, P(abi.MpmGpuBatchInfo)], C.c_int),
        "mpmgpu_batch_last_error": ([VP], C.c_char_p),
        "mpmgpu_batch_stream": ([VP], VP),
        "mpmgpu_batch_destroy": ([VP], None),
        "mpmgpu_server_create": ([P(abi.MpmGpuServerOptions), P(VP)], C.c_int),
        "mpmgpu_server_submit": ([VP, P(abi.MpmGpuGrid), P(abi.MpmGpuMaterial), C.c_int32, P(abi.MpmGpuVelBC),
                                  C.c_int32, P(abi.MpmGpuContact), P(abi.MpmGpuParticles), C.c_double, C.c_int32,
                                  P(C.c_int64)], C.c_int),
        "mpmgpu_server_poll": ([VP, C.c_int64, P(abi.MpmGpuRequestInfo)], C.c_int),
        "mpmgpu_server_wait": ([VP, C.c_int64, C.c_double], C.c_int),
        "mpmgpu_server_drain": ([VP, C.c_double], C.c_int),
        "mpmgpu_server_release": ([VP, C.c_int64], C.c_int),
        "mpmgpu_server_stats": ([VP, P(abi.MpmGpuServerStats)], C.c_int),
        "mpmgpu_server_last_error": ([VP], C.c_char_p),
        "mpmgpu_server_destroy": ([VP], None),
        "mpmgpu_server_admits": ([C.c_double, C.c_double, C.c_double, P(abi.MpmGpuRunLoad), C.c_int32, C.c_int64,
                                  C.c_int32, C.c_double], C.c_int),
    }
    for f, (args, res) in batch_sigs.items():
        getattr(L, f).argtypes = args
        getattr(L, f).restype = res
    for f in ("mpmgpu_create", "mpmgpu_set_materials", "mpmgpu_set_contact", "mpmgpu_set_velocity_bcs",
              "mpmgpu_upload_particles", "mpmgpu_step", "mpmgpu_download_particles", "mpmgpu_profile",
              "mpmgpu_set_profiling", "mpmgpu_step_host"):
        getattr(L, f).restype = C.c_int
    _lib = L
    return L


# every symbol the header declares (checked by the CPU tests)
EXPORTED = ("mpmgpu_step_timed", "mpmgpu_autotune_sort", "mpmgpu_archive_record_size", "mpmgpu_archive_records",
            "mpmgpu_archive_records_async", "mpmgpu_archive_wait",
            "mpmgpu_set_profiling", "mpmgpu_stream", "mpmgpu_launch_count",
            "mpmgpu_host_register", "mpmgpu_host_unregister", "mpmgpu_host_alloc", "mpmgpu_host_free",
            "mpmgpu_step_host", "mpmgpu_fp64_fma_rate", "mpmgpu_fp32_fma_rate",
            "mpmgpu_abi_version", "mpmgpu_create", "mpmgpu_set_materials", "mpmgpu_set_contact",
            "mpmgpu_set_velocity_bcs", "mpmgpu_upload_particles", "mpmgpu_step", "mpmgpu_download_particles",
            "mpmgpu_last_error", "mpmgpu_destroy", "mpmgpu_profile")


class GpuRun:
    """One MPM run resident on the current GPU."""

    def __init__(self, model: Model, precision: int = 0, p2g: int = 0, sort_interval: int = 1):
        L = lib()
        self.model = model
        self._b = abi.Bound()
        g = abi.grid_struct(model, self._b)
        o = abi.options_struct(model, precision=precision, p2g=p2g, sort_interval=sort_interval)
        h = C.c_void_p()
        st = L.mpmgpu_create(C.byref(g), C.byref(o), C.byref(h))
        if st != 0:
            raise GpuError(st, L.mpmgpu_last_error(None).decode())
        self.h = h
        self._check(L.mpmgpu_set_materials(self.h, abi.materials_array(model), len(model.materials)))
        ct = abi.contact_struct(model)
        if ct.enabled:
            self._check(L.mpmgpu_set_contact(self.h, C.byref(ct)))
        bcs, nbc = abi.bcs_array(model)
        self._check(L.mpmgpu_set_velocity_bcs(self.h, bcs, nbc))
        self.t = 0.0

    def _check(self, st):
        if st != 0:
            raise GpuError(st, lib().mpmgpu_last_error(self.h).decode())

    def upload(self, particles: dict):
        b = abi.Bound()
        ps = abi.particles_struct(particles, b)
        self._check(lib().mpmgpu_upload_particles(self.h, C.byref(ps)))

    def step(self, nsteps: int):
        self._check(lib().mpmgpu_step(self.h, int(nsteps), float(self.t)))
        self.t += nsteps * self.model.options["timestep"]

    def step_host(self, particles: dict, nsteps: int):
        """Advance nsteps on state kept in host memory (mpmgpu_step_host): the
        kernels read and write the columns of `particles` in place, which must
        lie in blocks of mpmgpu_host_alloc (HostState)."""
        b = abi.Bound()
        ps = abi.particles_struct(particles, b)
        self._check(lib().mpmgpu_step_host(self.h, C.byref(ps), int(nsteps), float(self.t)))
        self.t += nsteps * self.model.options["timestep"]

    def step_timed(self, nsteps: int) -> float:
        """Advance nsteps; return their device time in ms (CUDA events on the context stream)."""
        ms = C.c_double()
        self._check(lib().mpmgpu_step_timed(self.h, int(nsteps), float(self.t), C.byref(ms)))
        self.t += nsteps * self.model.options["timestep"]
        return ms.value

    def autotune_sort(self, trial_steps: int = 16):
        """Keep the fastest cell-sort interval of 1, 2, 4, 8 (about 4 x
        trial_steps real steps are taken); returns (interval, ms per step)."""
        si, ms, taken = C.c_int32(), C.c_double(), C.c_int32()
        st = lib().mpmgpu_autotune_sort(self.h, int(trial_steps), float(self.t), C.byref(si), C.byref(ms),
                                        C.byref(taken))
        self.t += taken.value * self.model.options["timestep"]
        self._check(st)
        return si.value, ms.value

    def archive_records(self, order: str, thickness: float = 1.0) -> bytes:
        """The particle records of a NairnMPM archive for the current state,
        packed on the device (mpmgpu_archive_records)."""
        L = lib()
        rec = int(L.mpmgpu_archive_record_size(int(self.model.grid.dim), order.encode("ascii")))
        if rec < 0:
            raise GpuError(-rec, L.mpmgpu_last_error(None).decode())
        buf = np.empty(self.model.n * rec, dtype=np.uint8)
        self._check(L.mpmgpu_archive_records(self.h, order.encode("ascii"), float(thickness),
                                             buf.ctypes.data_as(C.c_void_p), buf.nbytes))
        return buf.tobytes()

    def archive_records_async(self, order: str, buf: np.ndarray, thickness: float = 1.0):
        """Start packing the records of the current state into `buf` (uint8,
        n * record size bytes, best pinned with pin()); they are complete
        after archive_wait(), while steps may run meanwhile."""
        self._check(lib().mpmgpu_archive_records_async(self.h, order.encode("ascii"), float(thickness),
                                                       buf.ctypes.data_as(C.c_void_p), buf.nbytes))

    def archive_wait(self):
        self._check(lib().mpmgpu_archive_wait(self.h))

    def launch_count(self) -> int:
        return int(lib().mpmgpu_launch_count(self.h))

    def download_into(self, out: dict):
        b = abi.Bound()
        ps = abi.particles_struct(out, b)
        self._check(lib().mpmgpu_download_particles(self.h, C.byref(ps)))

    def download(self, like: dict) -> dict:
        out = abi.empty_like_particles(like)
        b = abi.Bound()
        ps = abi.particles_struct(out, b)
        self._check(lib().mpmgpu_download_particles(self.h, C.byref(ps)))
        return out

    def set_profiling(self, on: bool):
        self._check(lib().mpmgpu_set_profiling(self.h, 1 if on else 0))

    def profile(self) -> dict:
        names = (C.c_char_p * 16)()
        ms = (C.c_double * 16)()
        k = lib().mpmgpu_profile(self.h, names, ms, 16)
        return {names[i].decode(): ms[i] for i in range(k)}

    def stream(self) -> int:
        return lib().mpmgpu_stream(self.h)


    def close(self):
        if getattr(self, "h", None):
            lib().mpmgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def xpic_of(m) -> tuple | None:
    """The PeriodicXPIC settings (order, fmpm, period) of a model, or None."""
    o = m.options
    return (o["xpic_order"], o.get("xpic_fmpm", 0), o.get("xpic_period", 1)) if o.get("xpic_order", 0) > 0 else None


def lr_links_for(models) -> int:
    """Links per particle slot a batch of `models` reserves for regression
    contact normals: every shape-function node of a particle (64 in 3D, 16 in
    2D) when one of them uses methods 5 or 6, else none."""
    if not any(((m.extra or {}).get("contact") or {}).get("normals", 0) >= 5 for m in models):
        return 0
    return 64 if models[0].grid.dim == 3 else 16


class GpuBatch:
    """Many independent runs resident on the current GPU, advanced together by
    one graph-captured batched step (mpmgpu_batch_* in the C ABI).  All runs
    share the analysis options (dimension, method, shape functions,
    precision); grids, materials, velocity conditions, particles, time steps
    and step counts are per run."""

    def __init__(self, np_: int, method: int, shape: int, precision: int = 0, *, max_runs: int,
                 max_particles: int, max_nodes: int, max_materials: int | None = None, sort_interval: int = 1,
                 block: int = 0, fraction_usf: float = 0.5, inc_defgrad_terms: int = 0, max_fields: int = 1,
                 lr_links: int = 0, xpic=None):
        L = lib()
        xo, xf, xp = xpic if xpic else (0, 0, 1)
        self.opts = abi.MpmGpuBatchOptions(np_, method, shape, precision, sort_interval, block, max_runs,
                                           max_materials or max_runs, max_particles, max_nodes, fraction_usf,
                                           inc_defgrad_terms, max_fields, lr_links, xo, xf, xp)
        self.bytes = int(L.mpmgpu_batch_bytes(C.byref(self.opts)))
        h = C.c_void_p()
        st = L.mpmgpu_batch_create(C.byref(self.opts), C.byref(h))
        if st != 0:
            raise GpuError(st, L.mpmgpu_batch_last_error(None).decode())
        self.h = h
        self.models = {}

    @classmethod
    def for_models(cls, models, precision: int = 0, slack: float = 1.0, **kw) -> "GpuBatch":
        """A batch sized to hold all `models` at once (times `slack`).  The
        runs of a batch share its analysis options, PeriodicXPIC included."""
        o = models[0].options
        if "xpic" not in kw and len({xpic_of(m) for m in models}) > 1:
            raise ValueError("the runs of a batch share one PeriodicXPIC setting")
        for key in ("np", "method", "shape"):
            if len({m.options[key] for m in models}) > 1:
                raise ValueError(f"the runs of a batch share one analysis option {key!r}")
        return cls(o["np"], o["method"], o["shape"], precision, max_runs=kw.pop("max_runs", len(models)),
                   max_particles=int(slack * sum(m.n for m in models)),
                   max_nodes=int(slack * sum(m.grid.nnodes for m in models)),
                   max_materials=int(slack * sum(len(m.materials) for m in models)) + 1,
                   fraction_usf=o.get("fraction_usf", 0.5), inc_defgrad_terms=o.get("inc_defgrad_terms", 0),
                   max_fields=kw.pop("max_fields", max(m.options.get("nfields", 1) for m in models)),
                   lr_links=kw.pop("lr_links", lr_links_for(models)), xpic=kw.pop("xpic", xpic_of(models[0])),
                   **kw)

    @staticmethod
    def bytes_for(models, precision: int = 0) -> int:
        o = models[0].options
        opts = abi.MpmGpuBatchOptions(o["np"], o["method"], o["shape"], precision, 1, 0, len(models),
                                      sum(len(m.materials) for m in models) + 1, sum(m.n for m in models),
                                      sum(m.grid.nnodes for m in models), 0.5, o.get("inc_defgrad_terms", 0),
                                      max(m.options.get("nfields", 1) for m in models), lr_links_for(models),
                                      *(xpic_of(models[0]) or (0, 0, 1)))
        return int(lib().mpmgpu_batch_bytes(C.byref(opts)))

    def _check(self, st):
        if st != 0:
            raise GpuError(st, lib().mpmgpu_batch_last_error(self.h).decode())

    def add(self, model: Model, nsteps: int | None = None, particles: dict | None = None) -> int:
        """Admit a run; returns its run id (GpuError BUSY when it does not fit now)."""
        b = abi.Bound()
        g = abi.grid_struct(model, b)
        bcs, nbc = abi.bcs_array(model)
        ps = abi.particles_struct(particles if particles is not None else model.particles, b)
        rid = C.c_int32(-1)
        ct = abi.contact_struct(model)
        self._check(lib().mpmgpu_batch_add_run(self.h, C.byref(g), abi.materials_array(model), len(model.materials),
                                               bcs, nbc, C.byref(ct), C.byref(ps), float(model.options["timestep"]),
                                               int(nsteps if nsteps is not None else model.nsteps), C.byref(rid)))
        self.models[rid.value] = model
        return rid.value

    def step(self, nsteps: int = 1):
        self._check(lib().mpmgpu_batch_step(self.h, int(nsteps)))

    def step_host(self, particles: dict, nsteps: int):
        """Advance nsteps on state kept in host memory (mpmgpu_step_host): the
        kernels read and write the columns of `particles` in place, which must
        lie in blocks of mpmgpu_host_alloc (HostState)."""
        b = abi.Bound()
        ps = abi.particles_struct(particles, b)
        self._check(lib().mpmgpu_step_host(self.h, C.byref(ps), int(nsteps), float(self.t)))
        self.t += nsteps * self.model.options["timestep"]

    def step_timed(self, nsteps: int) -> float:
        ms = C.c_double()
        self._check(lib().mpmgpu_batch_step_timed(self.h, int(nsteps), C.byref(ms)))
        return ms.value

    def state(self, rid: int):
        s, d = C.c_int32(), C.c_int32()
        self._check(lib().mpmgpu_batch_run_state(self.h, rid, C.byref(s), C.byref(d)))
        return s.value, d.value

    def download(self, rid: int, like: dict | None = None) -> dict:
        out = abi.empty_like_particles(like if like is not None else self.models[rid].particles)
        b = abi.Bound()
        ps = abi.particles_struct(out, b)
        self._check(lib().mpmgpu_batch_download_run(self.h, rid, C.byref(ps)))
        return out

    def remove(self, rid: int, download: bool = True):
        out = None
        if download:
            out = abi.empty_like_particles(self.models[rid].particles)
            b = abi.Bound()
            ps = abi.particles_struct(out, b)
            self._check(lib().mpmgpu_batch_remove_run(self.h, rid, C.byref(ps)))
        else:
            self._check(lib().mpmgpu_batch_remove_run(self.h, rid, None))
        self.models.pop(rid, None)
        return out

    def set_tuning(self, block: int, sort_interval: int):
        self._check(lib().mpmgpu_batch_set_tuning(self.h, block, sort_interval))

    def autotune(self, trial_steps: int = 8):
        blk, si, ms = C.c_int32(), C.c_int32(), C.c_double()
        self._check(lib().mpmgpu_batch_autotune(self.h, trial_steps, C.byref(blk), C.byref(si), C.byref(ms)))
        return blk.value, si.value, ms.value

    def info(self) -> dict:
        i = abi.MpmGpuBatchInfo()
        self._check(lib().mpmgpu_batch_info(self.h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in abi.MpmGpuBatchInfo._fields_}

    def close(self):
        if getattr(self, "h", None):
            lib().mpmgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


SERVER_ORDERS = {"fifo": 0, "least_work": 1, "deadline": 2}


def server_admits(a_ms: float, b_ms: float, k: float, running, cand_n: int, cand_steps: int,
                  cand_waited_ms: float) -> int:
    """The deadline order's admission rule (mpmgpu_server_admits): running is
    a list of (n, steps_left, steps_total, elapsed_ms)."""
    arr = (abi.MpmGpuRunLoad * max(1, len(running)))(*[abi.MpmGpuRunLoad(*r) for r in running])
    return lib().mpmgpu_server_admits(a_ms, b_ms, k, arr, len(running), cand_n, cand_steps, cand_waited_ms)


class GpuServer:
    """Continuous-batching request loop on the current GPU (mpmgpu_server_*):
    a C++ thread admits submitted runs against the HBM budget, advances all
    admitted runs together and retires them as they finish.  Each request's
    particle state is a private copy that receives the result."""

    def __init__(self, method: int, shape: int, precision: int = 1, *, hbm_budget_bytes: int,
                 max_runs: int = 256, steps_per_round: int = 10, backfill: bool = True, sort_interval: int = 1,
                 block: int = 0, frac_3d: float = 0.5, nodes_per_particle: float = 0.5, fraction_usf: float = 0.5,
                 max_resident_particles: int = 0, order: str = "fifo", max_fields: int = 1, lr_links: int = 0,
                 xpic=None, slowdown_target: float = 0.0):
        L = lib()
        xo, xf, xp = xpic if xpic else (0, 0, 1)
        o = abi.MpmGpuServerOptions(method, shape, precision, max_runs, steps_per_round, 1 if backfill else 0,
                                    sort_interval, block, int(hbm_budget_bytes), frac_3d, nodes_per_particle,
                                    fraction_usf, int(max_resident_particles),
                                    SERVER_ORDERS[order], int(max_fields), int(lr_links),
                                    int(xo), int(xf), int(xp), float(slowdown_target))
        h = C.c_void_p()
        st = L.mpmgpu_server_create(C.byref(o), C.byref(h))
        if st != 0:
            raise GpuError(st, L.mpmgpu_server_last_error(None).decode())
        self.h = h
        self._held = {}

    def _check(self, st):
        if st != 0:
            raise GpuError(st, lib().mpmgpu_server_last_error(self.h).decode())

    def submit(self, model: Model, particles: dict | None = None, nsteps: int | None = None) -> int:
        b = abi.Bound()
        g = abi.grid_struct(model, b)
        bcs, nbc = abi.bcs_array(model)
        state = abi.copy_particles(particles if particles is not None else model.particles)
        ps = abi.particles_struct(state, b)
        rid = C.c_int64(-1)
        ct = abi.contact_struct(model)
        self._check(lib().mpmgpu_server_submit(self.h, C.byref(g), abi.materials_array(model), len(model.materials),
                                               bcs, nbc, C.byref(ct), C.byref(ps), float(model.options["timestep"]),
                                               int(nsteps if nsteps is not None else model.nsteps), C.byref(rid)))
        self._held[rid.value] = (state, b, ps)
        return rid.value

    def poll(self, rid: int) -> dict:
        i = abi.MpmGpuRequestInfo()
        self._check(lib().mpmgpu_server_poll(self.h, rid, C.byref(i)))
        return {f: getattr(i, f) for f, _ in abi.MpmGpuRequestInfo._fields_ if f != "pad"}

    def wait(self, rid: int, timeout: float = 600.0) -> int:
        """Status of the request once done or failed (TIMEOUT after `timeout` s)."""
        return lib().mpmgpu_server_wait(self.h, rid, float(timeout))

    def drain(self, timeout: float = 3600.0):
        self._check(lib().mpmgpu_server_drain(self.h, float(timeout)))

    def result(self, rid: int) -> dict:
        return self._held[rid][0]

    def release(self, rid: int):
        self._check(lib().mpmgpu_server_release(self.h, rid))
        self._held.pop(rid, None)

    def stats(self) -> dict:
        s = abi.MpmGpuServerStats()
        self._check(lib().mpmgpu_server_stats(self.h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in abi.MpmGpuServerStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            lib().mpmgpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fma_rate(fp64: bool = True, iters: int = 20000) -> float:
    """Measured FMA throughput of the current GPU in TFLOP/s (FP64 or FP32)."""
    tf, ms = C.c_double(), C.c_double()
    f = lib().mpmgpu_fp64_fma_rate if fp64 else lib().mpmgpu_fp32_fma_rate
    st = f(int(iters), C.byref(tf), C.byref(ms))
    if st != 0:
        raise GpuError(st, lib().mpmgpu_last_error(None).decode())
    return tf.value


class HostBlock:
    """Page-locked host memory allocated by the driver (mpmgpu_host_alloc),
    seen as a numpy array of the given shape and dtype; close() frees it."""

    def __init__(self, shape, dtype=np.float64):
        L = lib()
        L.mpmgpu_host_alloc.argtypes = [C.c_uint64, C.POINTER(C.c_void_p)]
        L.mpmgpu_host_alloc.restype = C.c_int
        L.mpmgpu_host_free.argtypes = [C.c_void_p]
        L.mpmgpu_host_free.restype = None
        dt = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dt.itemsize
        self.ptr = C.c_void_p()
        st = L.mpmgpu_host_alloc(nbytes, C.byref(self.ptr))
        if st != 0:
            raise GpuError(st, L.mpmgpu_last_error(None).decode())
        buf = (C.c_char * nbytes).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=dt).reshape(shape)

    def close(self):
        if self.ptr:
            self.array = None
            lib().mpmgpu_host_free(self.ptr)
            self.ptr = None


class HostState:
    """A particle state in page-locked blocks the driver allocated: the FP64
    columns as rows of one block in the library's column order, mat and elem
    as the rows of a second; `particles` maps the column names to views of
    them (the form mpmgpu_step_host steps in place).  close() frees both."""

    def __init__(self, p: dict):
        n = len(p["x"])
        self._d = HostBlock((len(abi.DEVICE_COLUMNS), n))
        self._i = HostBlock((2, n), np.int32)
        out, _ = abi.contiguous_particles(p, self._d.array)
        self._i.array[0] = p["mat"]
        self._i.array[1] = p["elem"]
        out["mat"], out["elem"] = self._i.array[0], self._i.array[1]
        self.particles = out
        self.nbytes = self._d.array.nbytes + self._i.array.nbytes

    def close(self):
        self.particles = None
        self._d.close()
        self._i.close()


def pin(arrays: dict) -> list:
    """Page-lock numpy arrays for DMA transfers; returns the registered list."""
    done = []
    for a in arrays.values():
        if a.nbytes and lib().mpmgpu_host_register(a.ctypes.data, a.nbytes) == 0:
            done.append(a)
    return done


def unpin(done: list):
    for a in done:
        lib().mpmgpu_host_unregister(a.ctypes.data)
