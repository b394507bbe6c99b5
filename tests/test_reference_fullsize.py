"""The benchmark configurations at their full sizes and lengths, against the
reference's own runs of them (tests/golden/full, written by
``make_golden.py --full`` from ``NairnMPM -np 1``):

- the 2D cantilever: 100x20 cells, 8,000 particles, 1,000 steps, every particle;
- the Taylor bar: 1,004,800 particles, the first 20 steps, and the whole
  2,000-step run archived every 500 steps;
- the two-material contact problem: 4,136,960 particles (lCPDI, Coulomb 0.3,
  volume-gradient normals), 10 steps.

The large cases keep a seeded sample of 4,096 particles (all their archived
quantities) plus, over every particle, the sum of squares of each quantity and
a CRC32 of the element column; the tests compare the sample element by element,
the whole state through its norms, and every particle's element exactly.
"""
import json
import os
import zlib

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2, view_for

FULL = os.path.join(GOLDEN, "full")
TOL = {0: 1e-10, 1: 1e-5}  # relative L2: all-FP64 mode, mixed mode (FP32 transfers)
QUANTITIES = ("pos", "vel", "stress", "strain")


def full_cases():
    return sorted(f[:-4] for f in os.listdir(FULL) if f.endswith(".npz")) if os.path.isdir(FULL) else []


def load_full(name):
    d = np.load(os.path.join(FULL, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    return meta, {k: d[k] for k in d.files if k != "meta"}


def build_model(meta):
    from nairn_gb300 import model
    return getattr(model, meta["generator"])(**meta["kwargs"])


def check_state(v, g, step, tol, what):
    """Sample quantities within tol (relative L2), global norms within tol,
    elements of the sample equal and the CRC32 of every element equal."""
    idx = g["sample"]
    for k in QUANTITIES:
        got, want = v[k][idx], g[f"s{step}_{k}"]
        e = rel_l2(got, want)
        assert e <= tol, (what, step, k, "sample", e)
        norm = float(np.sqrt(np.sum(np.asarray(v[k], dtype=np.float64) ** 2)))
        ref = float(np.sqrt(g[f"s{step}_sumsq_{k}"]))
        assert abs(norm - ref) <= tol * ref, (what, step, k, "norm", norm, ref)
    assert np.array_equal(v["elem"][idx], g[f"s{step}_elem"]), (what, step, "elem sample")
    crc = zlib.crc32(np.ascontiguousarray(v["elem"], dtype="<i4").tobytes())
    assert crc == int(g[f"s{step}_elem_crc32"]), (what, step, "elem crc32")


def test_full_goldens_present():
    assert {"full_c1_cantilever", "full_c2_taylor_20", "full_c2_taylor", "full_c3_contact"} <= set(full_cases())


def test_cantilever_builder_and_oracle_match_reference_full_length():
    """The model builder reproduces the reference's t=0 state of the 8,000-particle
    cantilever, and the single-threaded oracle (the reference's summation
    order) matches the reference bit for bit after all 1,000 steps."""
    import oracle_lib
    from nairn_gb300 import abi
    meta, g = load_full("full_c1_cantilever")
    m = build_model(meta)
    v0 = view_for(m.particles, m)
    for k in ("pos", "vel", "stress"):
        assert rel_l2(v0[k], g["init_" + k]) == 0.0, k
    assert np.array_equal(v0["elem"], g["init_elem"])
    p = abi.copy_particles(m.particles)
    oracle_lib.run(m, p, meta["steps"], nthreads=1)
    check_state(view_for(p, m), g, meta["steps"], 0.0, "oracle")


def test_taylor_builder_matches_reference_sample():
    """The 1,004,800-particle Taylor bar as the model builder makes it equals the
    reference's t=0 state on the sampled particles."""
    meta, g = load_full("full_c2_taylor_20")
    m = build_model(meta)
    assert m.n == meta["particles"]
    idx = g["sample"]
    v0 = view_for(m.particles, m)
    for k in ("pos", "vel", "stress"):
        assert rel_l2(v0[k][idx], g["init_" + k]) == 0.0, k
    assert np.array_equal(v0["elem"][idx], g["init_elem"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("case", full_cases())
def test_gpu_full_size_matches_reference(case, precision, gpu_lib):
    from nairn_gb300.gpu import GpuRun
    meta, g = load_full(case)
    m = build_model(meta)
    assert m.n == meta["particles"]
    idx = g["sample"]
    v0 = view_for(m.particles, m)
    assert rel_l2(v0["pos"][idx], g["init_pos"]) == 0.0
    r = GpuRun(m, precision=precision, sort_interval=8)
    r.upload(m.particles)
    done = 0
    for s in meta["archived"]:
        r.step(s - done)
        done = s
        check_state(view_for(r.download(m.particles), m), g, s, TOL[precision],
                    ("fp64", "mixed")[precision])
    r.close()
