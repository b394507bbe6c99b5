"""Loader for the CPU oracle (mpm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the bench's
CPU-baseline leg, never by the product.  build() compiles the C restatement
with gcc (FP contraction off, so results do not depend on the host's FMA
defaults) into oracle/_build/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmpm_oracle.so")
SRC = os.path.join(HERE, "mpm_oracle.c")

sys.path.insert(0, os.path.join(ROOT, "nairn-mpm-fea_gb300", "python"))
from nairn_gb300 import abi  # noqa: E402

_lib = None


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "mpm_oracle.h"))):
        cmd = ["gcc", "-O2", "-std=c99", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               "-I", os.path.join(ROOT, "include"), SRC, "-o", LIB + ".tmp", "-lm"]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.mpm_oracle_run.restype = C.c_int
        _lib.mpm_oracle_run.argtypes = [C.POINTER(abi.MpmGpuGrid), C.POINTER(abi.MpmGpuOptions),
                                        C.POINTER(abi.MpmGpuMaterial), C.c_int,
                                        C.POINTER(abi.MpmGpuVelBC), C.c_int, C.POINTER(abi.MpmGpuContact),
                                        C.POINTER(abi.MpmGpuParticles), C.c_int, C.c_double, C.c_int]
        _lib.mpm_oracle_last_error.restype = C.c_char_p
    return _lib


def run(model, particles: dict, nsteps: int, t0: float = 0.0, nthreads: int = 1, contact=None) -> int:
    """Advance particles (dict of numpy arrays, modified in place) nsteps."""
    L = lib()
    b = abi.Bound()
    g = abi.grid_struct(model, b)
    o = abi.options_struct(model)
    mats = abi.materials_array(model)
    bcs, nbc = abi.bcs_array(model)
    ps = abi.particles_struct(particles, b)
    if contact is None:
        contact = abi.contact_struct(model)
    ct = contact
    st = L.mpm_oracle_run(C.byref(g), C.byref(o), mats, len(model.materials), bcs, nbc, C.byref(ct),
                          C.byref(ps), int(nsteps), float(t0), int(nthreads))
    if st != 0:
        raise RuntimeError(f"oracle status {abi.STATUS_NAMES.get(st, st)}: {L.mpm_oracle_last_error().decode()}")
    return st
