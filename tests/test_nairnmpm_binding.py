"""The NairnMPM-side binding (nairn-mpm-fea_gb300/nairnmpm: GPUStepTask and
NairnMPMGPU) compiled into the reference itself and driven by the reference's
XML input.

oracle/ref/Makefile's `gpu` target links NairnMPM-gpu: the reference's
objects with the binding's main and task, and the C ABI library -- here the
CPU test double of the ABI (oracle/mpmgpu_cpu_double.c, over the oracle), as
this machine has no GPU.  Every case is run by NairnMPM and by NairnMPM-gpu
from the same XML file with archives every few steps; the binding reads the
grid, materials, contact law, velocity conditions and particles from
NairnMPM's objects, steps through the ABI and writes the state back before
each archive, so the archives must be identical byte for byte.  Runs only
where the reference was built from source (oracle/_ref/NairnMPM).
"""
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "NairnMPM")
GPU_BIN = os.path.join(ROOT, "oracle", "_ref", "NairnMPM-gpu")

CASES = {
    "cantilever_ugimp_usavg": ("cantilever_2d", dict(nx=10, ny=4, steps=60)),
    "cantilever_lcpdi_usl": ("cantilever_2d", dict(nx=10, ny=4, steps=40, gimp="lCPDI", method=3)),
    "cantilever_qcpdi_usavg": ("cantilever_2d", dict(nx=10, ny=4, steps=40, gimp="qCPDI")),
    "taylor_plastic": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30)),
    "taylor_neohookean_usf": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30, mat_type=28, G=10., K=50.,
                                                rho=1.1, v0=-30000., method=0)),
    "contact2d_friction": ("contact_2d", dict(steps=60, friction=0.3, normals=2)),
    "rigid_indenter": ("rigid_contact_2d", dict(steps=60, friction=0.3, normals=2, v=(1500., -2000.),
                                               indenter_x0=5.0)),
}


@pytest.fixture(scope="module")
def gpu_binary():
    if not os.path.exists(REF_BIN):
        pytest.skip("the reference is not built here (oracle/ref recipe needs its source tree)")
    out = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "gpu", "-j8"],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    return GPU_BIN


@pytest.mark.parametrize("case", sorted(CASES))
def test_binding_reproduces_reference_archives(case, gpu_binary, tmp_path):
    sys.path.insert(0, os.path.join(ROOT, "nairn-mpm-fea_gb300", "python"))
    from nairn_gb300 import inputs
    gen, kw = CASES[case]
    xml, info = getattr(inputs, gen)(archive_root="Results/out.", **kw)
    every = max(1, kw["steps"] // 3)
    t_ms = every * info["dt"] * 1e3 * (1. - 1e-9)
    xml = re.sub(r'<ArchiveTime units="ms">[^<]*</ArchiveTime>', f'<ArchiveTime units="ms">{t_ms!r}</ArchiveTime>', xml)
    runs = {}
    for name, binary in (("reference", REF_BIN), ("binding", gpu_binary)):
        d = tmp_path / name
        (d / "Results").mkdir(parents=True)
        (d / "in.xml").write_text(xml)
        out = subprocess.run([binary, "-np", "1", "in.xml"], cwd=d, capture_output=True, text=True)
        assert out.returncode == 0 and "RUN COMPLETED" in out.stdout, (name, out.stdout[-1500:], out.stderr[-1500:])
        runs[name] = d / "Results"
    archives = sorted(f for f in os.listdir(runs["reference"]) if re.fullmatch(r"out\.\d+", f))
    assert len(archives) >= 3
    assert archives == sorted(f for f in os.listdir(runs["binding"]) if re.fullmatch(r"out\.\d+", f))
    for f in archives:
        a = (runs["reference"] / f).read_bytes()
        b = (runs["binding"] / f).read_bytes()
        assert a == b, (case, f)
