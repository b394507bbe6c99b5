"""Generate the golden fixtures from the reference NairnMPM built from source.

Run in a container that has the reference tree and the oracle build:

    make -C oracle/ref -j8            # builds oracle/_ref/NairnMPM
    python tests/golden/make_golden.py                 # the small cases
    python tests/golden/make_golden.py --full [name]   # the benchmark configurations at full size

For every case it writes the synthetic XML (nairn_gb300.inputs), runs
``NairnMPM -np 1`` (single patch, the reference's deterministic order), reads
the t=0 and final binary archives, and stores both plus the generator
arguments in tests/golden/<case>.npz.  The GPU parity tests and the oracle pin
tests replay these files; nothing at test time runs the reference.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "nairn-mpm-fea_gb300", "python"))
from nairn_gb300 import inputs  # noqa: E402
from nairn_gb300.archive import read_archive  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "NairnMPM")

# name -> (generator, kwargs); kwargs are shared with nairn_gb300.model
CASES = {
    "cant2d_ugimp_usavg": ("cantilever_2d", dict(nx=10, ny=4, steps=60)),
    "cant2d_ugimp_usavg_long": ("cantilever_2d", dict(nx=24, ny=6, steps=400)),
    "cant2d_linear_usavg": ("cantilever_2d", dict(nx=10, ny=4, steps=60, gimp="Classic")),
    "cant2d_ugimp_usf": ("cantilever_2d", dict(nx=10, ny=4, steps=60, method=0)),
    "cant2d_ugimp_usl": ("cantilever_2d", dict(nx=10, ny=4, steps=60, method=3)),
    "cant2d_ugimp_ppc3": ("cantilever_2d", dict(nx=8, ny=3, steps=40, ppc_side=3)),
    "taylor3d_ugimp_usavg": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30)),
    "taylor3d_ugimp_long": ("taylor_3d", dict(radius=1.5, length=3.0, cell=0.5, steps=120)),
    "taylor3d_linear_usavg": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30, gimp="Classic")),
    "taylor3d_ugimp_usl": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30, method=3)),
    # Neohookean (type 28): soft rubber, large deformation
    "cant2d_neo_usavg": ("cantilever_2d", dict(nx=10, ny=4, steps=150, mat_type=28, G=3., K=30., rho=1.1,
                                               v0=20000., margin_cells=8)),
    "cant2d_neo_uj1_usl": ("cantilever_2d", dict(nx=10, ny=4, steps=100, mat_type=28, G=3., K=30., rho=1.1,
                                                 v0=20000., uj=1, method=3, margin_cells=8)),
    "cant2d_neo_uj2_terms3": ("cantilever_2d", dict(nx=10, ny=4, steps=100, mat_type=28, G=3., K=30.,
                                                    rho=1.1, v0=20000., uj=2, inc_terms=3, margin_cells=8)),
    "taylor3d_neo_usavg": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=80, mat_type=28, G=10.,
                                             K=50., rho=1.1, v0=-30000.)),
    "taylor3d_neo_terms2_usl": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=60, mat_type=28,
                                                  G=10., K=50., rho=1.1, v0=-30000., inc_terms=2, method=3)),
    # linear CPDI shape functions (lCPDI)
    "cant2d_cpdi_usavg": ("cantilever_2d", dict(nx=10, ny=4, steps=60, gimp="lCPDI")),
    "cant2d_cpdi_usl_ppc3": ("cantilever_2d", dict(nx=8, ny=3, steps=40, ppc_side=3, gimp="lCPDI", method=3)),
    "cant2d_cpdi_neo": ("cantilever_2d", dict(nx=10, ny=4, steps=150, mat_type=28, G=3., K=30., rho=1.1,
                                              v0=20000., margin_cells=8, gimp="lCPDI")),
    "taylor3d_cpdi_usavg": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30, gimp="lCPDI")),
    "taylor3d_cpdi_neo_usf": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=80, mat_type=28, G=10.,
                                                K=50., rho=1.1, v0=-30000., gimp="lCPDI", method=0)),
    # multimaterial contact: Neo-Hookean block onto an elastic plate whose base is held
    "contact2d_fric_avgg": ("contact_2d", dict(steps=200, friction=0.3, normals=2)),
    "contact2d_frictionless_maxg": ("contact_2d", dict(steps=150, friction=0.0, normals=0)),
    "contact2d_stick_maxv_usl": ("contact_2d", dict(steps=150, friction=-1.0, normals=1, method=3)),
    "contact2d_fric_cpdi_usf": ("contact_2d", dict(steps=150, friction=0.3, normals=2, gimp="lCPDI", method=0)),
    "contact3d_fric_cpdi": ("contact_3d", dict(steps=60, friction=0.3, normals=2)),
    "contact3d_fric_ugimp_maxg": ("contact_3d", dict(steps=60, friction=0.5, normals=0, gimp="uGIMP")),
    "contact2d_fric_logreg": ("contact_2d", dict(steps=150, friction=0.3, normals=6)),
    "contact2d_stick_linreg_usl": ("contact_2d", dict(steps=120, friction=-1.0, normals=5, method=3)),
    "contact2d_fric_logreg_cpdi": ("contact_2d", dict(steps=120, friction=0.3, normals=6, gimp="lCPDI")),
    # a one-cell gap closed by a fast block: point clouds that start touching
    # face to face have a regression separation of exactly zero, whose sign
    # is then a matter of rounding
    "contact3d_fric_logreg_cpdi": ("contact_3d", dict(steps=70, friction=0.3, normals=6, gap=0.5,
                                                      v=(50000., 0., -200000.))),
    "contact3d_fric_logreg_ugimp_usf": ("contact_3d", dict(steps=70, friction=0.3, normals=6, gimp="uGIMP",
                                                           method=0, gap=0.5, v=(50000., 0., -200000.))),
    # PeriodicXPIC: XPIC(k) and FMPM(k) grid-to-particle updates, every step or
    # every few steps (xpic = (order, fmpm, period))
    "cant2d_xpic2": ("cantilever_2d", dict(nx=10, ny=4, steps=60, xpic=(2, 0, 1))),
    "cant2d_pic_every3": ("cantilever_2d", dict(nx=10, ny=4, steps=60, xpic=(1, 0, 3))),
    "cant2d_fmpm3": ("cantilever_2d", dict(nx=10, ny=4, steps=60, xpic=(3, 1, 1))),
    "cant2d_fmpm1_usl": ("cantilever_2d", dict(nx=10, ny=4, steps=60, method=3, xpic=(1, 1, 1))),
    "cant2d_fmpm2_usl_every2": ("cantilever_2d", dict(nx=10, ny=4, steps=60, method=3, xpic=(2, 1, 2))),
    "cant2d_xpic2_cpdi_every2": ("cantilever_2d", dict(nx=10, ny=4, steps=60, gimp="lCPDI", xpic=(2, 0, 2))),
    "taylor3d_xpic3": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30, xpic=(3, 0, 1))),
    "taylor3d_fmpm2_cpdi_usf": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30, gimp="lCPDI",
                                                  method=0, xpic=(2, 1, 1))),
    "taylor3d_neo_fmpm4_usl": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=40, mat_type=28, G=10.,
                                                 K=50., rho=1.1, v0=-30000., method=3, xpic=(4, 1, 1))),
    # quadratic B-spline shape functions (B2SPLINE)
    "cant2d_b2spline": ("cantilever_2d", dict(nx=10, ny=4, steps=60, gimp="B2SPLINE")),
    "cant2d_b2spline_usl_neo": ("cantilever_2d", dict(nx=10, ny=4, steps=100, gimp="B2SPLINE", method=3, mat_type=28,
                                                      G=3., K=30., rho=1.1, v0=20000., margin_cells=8)),
    "taylor3d_b2spline": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30, gimp="B2SPLINE")),
    "taylor3d_b2spline_usf_xpic2": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30, gimp="B2SPLINE",
                                                      method=0, xpic=(2, 0, 1))),
    "contact2d_b2spline_fric": ("contact_2d", dict(steps=150, friction=0.3, normals=2, gimp="B2SPLINE")),
    "contact3d_b2spline_logreg": ("contact_3d", dict(steps=70, friction=0.3, normals=6, gimp="B2SPLINE", gap=0.5,
                                                     v=(50000., 0., -200000.))),
    # B-spline GIMP shape functions (B2GIMP)
    "cant2d_b2gimp": ("cantilever_2d", dict(nx=10, ny=4, steps=60, gimp="B2GIMP")),
    "cant2d_b2gimp_ppc3_usl": ("cantilever_2d", dict(nx=8, ny=3, steps=40, ppc_side=3, gimp="B2GIMP", method=3)),
    "taylor3d_b2gimp": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=30, gimp="B2GIMP")),
    "taylor3d_b2gimp_neo_usf": ("taylor_3d", dict(radius=1.0, length=2.0, cell=0.5, steps=60, gimp="B2GIMP", method=0,
                                                  mat_type=28, G=10., K=50., rho=1.1, v0=-30000.)),
    "contact2d_b2gimp_fric": ("contact_2d", dict(steps=150, friction=0.3, normals=2, gimp="B2GIMP")),
    # rigid contact materials (type 35): a rigid indenter moving at constant
    # velocity into an elastic plate, and the Taylor bar onto a rigid slab
    # (an off-centre indenter sliding as it presses, and an oblique impact:
    # with a symmetric normal approach the stick/slip decision sits on a
    # near-zero tangential momentum and the reference's run is chaotic)
    "rigid2d_indent_fric": ("rigid_contact_2d", dict(steps=150, friction=0.3, normals=2, v=(1500., -2000.),
                                                     indenter_x0=5.0)),
    "rigid2d_indent_maxg_usl": ("rigid_contact_2d", dict(steps=120, friction=0.0, normals=0, method=3)),
    "rigid2d_indent_maxv_stick": ("rigid_contact_2d", dict(steps=120, friction=-1.0, normals=1, v=(1000., -1500.))),
    "rigid2d_indent_cpdi_usf": ("rigid_contact_2d", dict(steps=120, friction=0.3, normals=2, gimp="lCPDI", method=0)),
    "rigid3d_taylor_wall": ("rigid_taylor_3d", dict(steps=40, friction=0.0, normals=2)),
    "rigid3d_taylor_wall_fric_usl": ("rigid_taylor_3d", dict(steps=40, friction=0.3, normals=0, method=3,
                                                             vx0=40000.)),
    # quadratic CPDI (qCPDI, 2D only): nine domain points per particle
    "cant2d_qcpdi_usavg": ("cantilever_2d", dict(nx=10, ny=4, steps=60, gimp="qCPDI")),
    "cant2d_qcpdi_ppc3_usl": ("cantilever_2d", dict(nx=8, ny=3, steps=40, ppc_side=3, gimp="qCPDI", method=3)),
    "cant2d_qcpdi_neo_usf": ("cantilever_2d", dict(nx=10, ny=4, steps=150, mat_type=28, G=3., K=30., rho=1.1,
                                                   v0=20000., margin_cells=8, gimp="qCPDI", method=0)),
    "cant2d_qcpdi_xpic2": ("cantilever_2d", dict(nx=10, ny=4, steps=60, gimp="qCPDI", xpic=(2, 0, 1))),
    "contact2d_fric_qcpdi": ("contact_2d", dict(steps=120, friction=0.3, normals=2, gimp="qCPDI")),
    # PeriodicXPIC with multimaterial contact: the contact law re-applied to
    # every expansion pass's increment from the last contact call's state
    "contact2d_xpic2_fric": ("contact_2d", dict(steps=120, friction=0.3, normals=2, xpic=(2, 0, 1))),
    "contact2d_fmpm2_fric_usl": ("contact_2d", dict(steps=120, friction=0.3, normals=2, method=3, xpic=(2, 1, 1))),
    "contact2d_fmpm3_frictionless": ("contact_2d", dict(steps=120, friction=0.0, normals=0, xpic=(3, 1, 1))),
    "contact2d_xpic3_stick_every2": ("contact_2d", dict(steps=120, friction=-1.0, normals=1, xpic=(3, 0, 2))),
    "contact2d_xpic2_logreg": ("contact_2d", dict(steps=100, friction=0.3, normals=6, xpic=(2, 0, 1))),
    "contact3d_xpic2_fric_cpdi": ("contact_3d", dict(steps=50, friction=0.3, normals=2, xpic=(2, 0, 1))),
    "contact3d_fmpm2_fric_ugimp_usf": ("contact_3d", dict(steps=50, friction=0.3, normals=2, gimp="uGIMP",
                                                          method=0, xpic=(2, 1, 1))),
}

KEEP = ("pos", "vel", "stress", "strain", "plastic", "work", "plastE", "hist1", "elem", "mass", "mat", "origpos")

# The benchmark configurations at their full sizes and lengths, each run once
# by the reference (-np 1) and written to tests/golden/full/<name>.npz.
# name -> (generator, kwargs, archive interval in steps or None for the final
# step only, sample size or 0 to keep every particle).  For a sampled case the
# file holds the records of a seeded sample of particles at every archived
# step, and for every particle the sum of squares of each quantity and a CRC32
# of the element column, so a test checks the sample element by element and
# the whole state through its norms and the element checksum.
FULL_CASES = {
    # 100x20 cells of 1 mm, 2x2 particles per cell (8,000), uGIMP, USAVG, 1,000 steps
    "full_c1_cantilever": ("cantilever_2d", dict(nx=100, ny=20, steps=1000), None, 0),
    # the 1,004,800-particle Taylor bar: the first 20 steps, and the whole
    # 2,000-step run archived every 500 steps
    "full_c2_taylor_20": ("taylor_3d", dict(steps=20), None, 4096),
    "full_c2_taylor": ("taylor_3d", dict(steps=2000), 500, 4096),
    # the 4,136,960-particle contact problem (lCPDI, Coulomb 0.3, volume-gradient normals)
    "full_c3_contact": ("contact_3d", dict(plate=(128, 128, 30), block=(40, 40, 16), block_x0=22.0, block_y0=22.0,
                                           cell=0.5, v=(4000., 0., -4000.), steps=10, gimp="lCPDI", friction=0.3,
                                           normals=2), None, 4096),
}
FULL_DIR = os.path.join(HERE, "full")


def run_case(name, gen, kw, workdir):
    xml, info = getattr(inputs, gen)(archive_root="Results/out.", **kw)
    d = os.path.join(workdir, name)
    os.makedirs(os.path.join(d, "Results"), exist_ok=True)
    with open(os.path.join(d, "in.xml"), "w") as fh:
        fh.write(xml)
    out = subprocess.run([REF, "-np", "1", "in.xml"], cwd=d, capture_output=True, text=True)
    if out.returncode != 0 or "RUN COMPLETED" not in out.stdout:
        raise RuntimeError(f"{name}: reference failed\n{out.stdout[-2000:]}\n{out.stderr[-2000:]}")
    steps = int(out.stdout.split("Calculation Steps:")[1].split()[0])
    assert steps == kw["steps"], (name, steps)
    a0 = read_archive(os.path.join(d, "Results", "out.0"))
    a1 = read_archive(os.path.join(d, "Results", f"out.{steps}"))
    arrays = {}
    for k in KEEP:
        if k in a0:
            arrays["init_" + k] = a0[k]
        if k in a1:
            arrays["final_" + k] = a1[k]
    meta = dict(generator=gen, kwargs=kw, steps=steps, three_d=bool(a0["three_d"]), order=a0["order"],
                time_ms=a1["time_ms"])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
    return steps, len(a0["mass"])


def run_full_case(name, gen, kw, every, sample, workdir):
    """One benchmark configuration at full size (see FULL_CASES)."""
    import re
    import zlib
    xml, info = getattr(inputs, gen)(archive_root="Results/out.", **kw)
    if every:
        # archive every `every` steps: ArchiveData::ArchiveResults writes when
        # the time reaches the next multiple of the archive time, which sits a
        # hair below every-th step times so rounding cannot skip one
        t_ms = every * info["dt"] * 1e3 * (1. - 1e-9)
        xml = re.sub(r'<ArchiveTime units="ms">[^<]*</ArchiveTime>',
                     f'<ArchiveTime units="ms">{t_ms!r}</ArchiveTime>', xml)
    d = os.path.join(workdir, name)
    os.makedirs(os.path.join(d, "Results"), exist_ok=True)
    with open(os.path.join(d, "in.xml"), "w") as fh:
        fh.write(xml)
    out = subprocess.run([REF, "-np", "1", "in.xml"], cwd=d, capture_output=True, text=True)
    if out.returncode != 0 or "RUN COMPLETED" not in out.stdout:
        raise RuntimeError(f"{name}: reference failed\n{out.stdout[-2000:]}\n{out.stderr[-2000:]}")
    steps = int(out.stdout.split("Calculation Steps:")[1].split()[0])
    assert steps == kw["steps"], (name, steps)
    per_step_ms = float(out.stdout.split("Elapsed Time per Step:")[1].split()[0])
    archived = sorted(int(f.split(".")[-1]) for f in os.listdir(os.path.join(d, "Results"))
                      if re.fullmatch(r"out\.\d+", f))
    a0 = read_archive(os.path.join(d, "Results", "out.0"))
    n = len(a0["mass"])
    idx = np.sort(np.random.default_rng(2025).choice(n, sample, replace=False)) if sample else np.arange(n)
    arrays = {"sample": idx.astype(np.int64)}
    for k in KEEP:
        if k in a0:
            arrays["init_" + k] = a0[k][idx]
    for s in archived[1:]:
        a = read_archive(os.path.join(d, "Results", f"out.{s}"))
        for k in KEEP:
            if k not in a:
                continue
            arrays[f"s{s}_{k}"] = a[k][idx]
            if k != "elem" and a[k].dtype.kind == "f":
                arrays[f"s{s}_sumsq_{k}"] = np.array(np.sum(a[k].astype(np.float64) ** 2))
        arrays[f"s{s}_elem_crc32"] = np.array(zlib.crc32(np.ascontiguousarray(a["elem"], dtype="<i4").tobytes()))
    meta = dict(generator=gen, kwargs=kw, steps=steps, archived=archived[1:], particles=n,
                sampled=bool(sample), three_d=bool(a0["three_d"]), order=a0["order"],
                reference_ms_per_step=per_step_ms, reference_threads=1)
    os.makedirs(FULL_DIR, exist_ok=True)
    np.savez_compressed(os.path.join(FULL_DIR, name + ".npz"), meta=json.dumps(meta), **arrays)
    return steps, n, per_step_ms


def main():
    if not os.path.exists(REF):
        sys.exit(f"{REF} not built: make -C oracle/ref -j8")
    work = tempfile.mkdtemp(prefix="nairn_golden_")
    try:
        only = sys.argv[1:]
        full = bool(only) and only[0] == "--full"
        if full:
            only = only[1:]
            for name, (gen, kw, every, sample) in FULL_CASES.items():
                if only and name not in only:
                    continue
                steps, n, ms = run_full_case(name, gen, kw, every, sample, work)
                print(f"{name}: {n} particles, {steps} steps, reference {ms:.1f} ms/step")
                shutil.rmtree(os.path.join(work, name), ignore_errors=True)
            return
        for name, (gen, kw) in CASES.items():
            if only and name not in only:
                continue
            steps, n = run_case(name, gen, kw, work)
            print(f"{name}: {n} particles, {steps} steps")
    finally:
        shutil.rmtree(work)


if __name__ == "__main__":
    main()
