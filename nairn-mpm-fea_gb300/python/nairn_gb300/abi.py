"""ctypes mirror of include/nairn_mpm_gpu.h and helpers to fill it from a Model.

This is the same binding a NairnMPM maintainer would write to drive the C ABI
from Python; the product's C++ host code uses the header directly.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .model import Model, PARTICLE_FIELDS

c_double_p = C.POINTER(C.c_double)
c_int32_p = C.POINTER(C.c_int32)

MPMGPU_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "UNSUPPORTED", 3: "CUDA", 4: "OOM", 5: "NAN",
                6: "LEFT_GRID", 7: "CPDI_NODES", 8: "TIMEOUT", 9: "BUSY", 10: "RANGE"}


class MpmGpuGrid(C.Structure):
    _fields_ = [("dim", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("xmin", C.c_double), ("ymin", C.c_double), ("zmin", C.c_double),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("thickness", C.c_double),
                ("xnodes", c_double_p), ("ynodes", c_double_p), ("znodes", c_double_p)]


class MpmGpuMaterial(C.Structure):
    _fields_ = [("type", C.c_int32), ("field", C.c_int32), ("rho", C.c_double),
                ("E", C.c_double), ("nu", C.c_double), ("yield_", C.c_double), ("Ep", C.c_double),
                ("G", C.c_double), ("K", C.c_double), ("UJOption", C.c_int32), ("pad", C.c_int32)]


class MpmGpuContact(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("normals", C.c_int32), ("friction", C.c_double),
                ("contact_cutoff", C.c_double), ("rigid_gradient_bias", C.c_double)]


class MpmGpuVelBC(C.Structure):
    _fields_ = [("node", C.c_int32), ("dir", C.c_int32), ("value", C.c_double), ("ftime", C.c_double)]


class MpmGpuOptions(C.Structure):
    _fields_ = [("np", C.c_int32), ("method", C.c_int32), ("shape", C.c_int32), ("precision", C.c_int32),
                ("p2g", C.c_int32), ("inc_defgrad_terms", C.c_int32), ("nfields", C.c_int32),
                ("sort_interval", C.c_int32), ("timestep", C.c_double), ("fraction_usf", C.c_double),
                ("xpic_order", C.c_int32), ("xpic_fmpm", C.c_int32), ("xpic_period", C.c_int32),
                ("xpic_reserved", C.c_int32)]


_PFIELDS = ["x", "y", "z", "vx", "vy", "vz", "x0", "y0", "z0", "mass", "mat", "elem", "lpx", "lpy", "lpz",
            "exx", "eyy", "ezz", "exy", "exz", "eyz", "wxy", "wxz", "wyz",
            "sxx", "syy", "szz", "sxy", "sxz", "syz", "pressure",
            "pxx", "pyy", "pzz", "pxy", "pxz", "pyz", "hist0", "hist1", "work", "plast"]


class MpmGpuParticles(C.Structure):
    _fields_ = [("n", C.c_int64)] + [(f, c_int32_p if f in ("mat", "elem") else c_double_p) for f in _PFIELDS]


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(c_double_p)


class Bound:
    """Keeps numpy arrays alive while their pointers sit in ctypes structs."""

    def __init__(self):
        self.keep = []

    def hold(self, a):
        self.keep.append(a)
        return a


def grid_struct(m: Model, b: Bound) -> MpmGpuGrid:
    g = m.grid
    xs = b.hold(np.ascontiguousarray(g.xnodes, dtype=np.float64))
    ys = b.hold(np.ascontiguousarray(g.ynodes, dtype=np.float64))
    zs = b.hold(np.ascontiguousarray(g.znodes, dtype=np.float64)) if g.znodes is not None else None
    return MpmGpuGrid(g.dim, g.nx, g.ny, g.nz, g.xmin, g.ymin, g.zmin, g.dx, g.dy, g.dz, g.thickness,
                      _dptr(xs), _dptr(ys), _dptr(zs) if zs is not None else None)


def options_struct(m: Model, precision: int = 0, p2g: int = 0, sort_interval: int = 1) -> MpmGpuOptions:
    o = m.options
    return MpmGpuOptions(o["np"], o["method"], o["shape"], precision, p2g, o.get("inc_defgrad_terms", 1),
                         o.get("nfields", 1), sort_interval, o["timestep"], o.get("fraction_usf", 0.5),
                         o.get("xpic_order", 0), o.get("xpic_fmpm", 0), o.get("xpic_period", 1), 0)


def materials_array(m: Model):
    arr = (MpmGpuMaterial * len(m.materials))()
    for i, d in enumerate(m.materials):
        arr[i] = MpmGpuMaterial(d["type"], d.get("field", 0), d["rho"], d.get("E", 0.), d.get("nu", 0.),
                                d.get("yield_", 0.), d.get("Ep", 0.), d.get("G", 0.), d.get("K", 0.),
                                d.get("UJOption", 0), 0)
    return arr


def contact_struct(m: Model) -> MpmGpuContact:
    """Multimaterial contact settings of a model (disabled when it has none)."""
    c = m.extra.get("contact") if m.extra else None
    if not c:
        return MpmGpuContact()
    return MpmGpuContact(int(c["enabled"]), int(c["normals"]), float(c["friction"]), float(c["contact_cutoff"]),
                         float(c["rigid_gradient_bias"]))


def bcs_array(m: Model):
    n = len(m.bcs)
    arr = (MpmGpuVelBC * max(n, 1))()
    for i in range(n):
        r = m.bcs[i]
        arr[i] = MpmGpuVelBC(int(r["node"]), int(r["dir"]), float(r["value"]), float(r["ftime"]))
    return arr, n


def particles_struct(p: dict, b: Bound) -> MpmGpuParticles:
    """Struct whose pointers alias the arrays of p (which must be contiguous
    float64 / int32 arrays of equal length)."""
    s = MpmGpuParticles()
    s.n = int(p["x"].shape[0])
    for f in _PFIELDS:
        a = p[f]
        if f in ("mat", "elem"):
            assert a.dtype == np.int32 and a.flags.c_contiguous
            setattr(s, f, a.ctypes.data_as(c_int32_p))
        else:
            assert a.dtype == np.float64 and a.flags.c_contiguous, f
            setattr(s, f, _dptr(a))
        b.hold(a)
    return s


def copy_particles(p: dict) -> dict:
    return {k: np.array(v, copy=True) for k, v in p.items()}


# the library's device column order of the FP64 particle columns (nmg::hcols)
DEVICE_COLUMNS = ["x", "y", "z", "vx", "vy", "vz", "mass", "lpx", "lpy", "lpz",
                  "exx", "eyy", "ezz", "exy", "exz", "eyz", "wxy", "wxz", "wyz",
                  "sxx", "syy", "szz", "sxy", "sxz", "syz", "pressure",
                  "pxx", "pyy", "pzz", "pxy", "pxz", "pyz", "hist0", "hist1", "work", "plast", "x0", "y0", "z0"]


def contiguous_particles(p: dict, block: np.ndarray | None = None) -> tuple[dict, np.ndarray]:
    """A copy of p whose FP64 columns are rows of one block in the library's
    device column order, so uploads and downloads move them with one copy
    each; returns (columns, block).  `block` (len(DEVICE_COLUMNS) x n FP64),
    when given, receives the columns -- e.g. page-locked memory."""
    n = len(p["x"])
    if block is None:
        block = np.empty((len(DEVICE_COLUMNS), n), dtype=np.float64)
    assert block.shape == (len(DEVICE_COLUMNS), n) and block.dtype == np.float64
    out = {}
    for i, k in enumerate(DEVICE_COLUMNS):
        block[i] = p[k]
        out[k] = block[i]
    for k, v in p.items():
        if k not in out:
            out[k] = np.array(v, copy=True)
    return out, block


def empty_like_particles(p: dict) -> dict:
    return {k: np.zeros_like(v) for k, v in p.items()}


class MpmGpuBatchOptions(C.Structure):
    _fields_ = [("np", C.c_int32), ("method", C.c_int32), ("shape", C.c_int32), ("precision", C.c_int32),
                ("sort_interval", C.c_int32), ("block", C.c_int32), ("max_runs", C.c_int32),
                ("max_materials", C.c_int32), ("max_particles", C.c_int64), ("max_nodes", C.c_int64),
                ("fraction_usf", C.c_double), ("inc_defgrad_terms", C.c_int32), ("max_fields", C.c_int32),
                ("lr_links", C.c_int32), ("xpic_order", C.c_int32), ("xpic_fmpm", C.c_int32),
                ("xpic_period", C.c_int32)]


class MpmGpuRunLoad(C.Structure):
    _fields_ = [("n", C.c_int64), ("steps_left", C.c_int32), ("steps_total", C.c_int32), ("elapsed_ms", C.c_double)]


class MpmGpuBatchInfo(C.Structure):
    _fields_ = [("runs", C.c_int32), ("running", C.c_int32), ("block", C.c_int32), ("sort_interval", C.c_int32),
                ("particles_used", C.c_int64), ("particles_dead", C.c_int64), ("nodes_used", C.c_int64),
                ("steps", C.c_int64), ("launches", C.c_int64)]


RUN_EMPTY, RUN_RUNNING, RUN_FINISHED = 0, 1, 2


class MpmGpuServerOptions(C.Structure):
    _fields_ = [("method", C.c_int32), ("shape", C.c_int32), ("precision", C.c_int32), ("max_runs", C.c_int32),
                ("steps_per_round", C.c_int32), ("backfill", C.c_int32), ("sort_interval", C.c_int32),
                ("block", C.c_int32), ("hbm_budget_bytes", C.c_int64), ("frac_3d", C.c_double),
                ("nodes_per_particle", C.c_double), ("fraction_usf", C.c_double),
                ("max_resident_particles", C.c_int64), ("order", C.c_int32), ("max_fields", C.c_int32),
                ("lr_links", C.c_int32), ("xpic_order", C.c_int32), ("xpic_fmpm", C.c_int32),
                ("xpic_period", C.c_int32), ("slowdown_target", C.c_double)]


class MpmGpuRequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("steps_done", C.c_int32), ("pad", C.c_int32),
                ("queue_ms", C.c_double), ("run_ms", C.c_double), ("total_ms", C.c_double)]


class MpmGpuServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64), ("queued", C.c_int64),
                ("running", C.c_int64), ("particle_steps", C.c_int64), ("rounds", C.c_int64),
                ("reserved_bytes", C.c_int64), ("busy_ms", C.c_double)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 1, 2, 3, 4
