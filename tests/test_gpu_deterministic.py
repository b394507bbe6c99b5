"""Deterministic node sums (MPMGPU_P2G_DETERMINISTIC): the same bits in every
run, whatever the particle order or sort interval, and the reference's
results within the FP64 tolerance (the mixed tolerance in the mixed mode)."""
import numpy as np
import pytest

from conftest import contact_tolerance, golden_cases, load_golden, model_for, rel_l2, view_for

pytestmark = pytest.mark.gpu

TOL = 1e-10
TOL_MIXED = 1e-5
DET = 1


def run(m, steps, particles=None, **kw):
    from nairn_gb300.gpu import GpuRun
    r = GpuRun(m, **kw)
    p = particles if particles is not None else m.particles
    r.upload(p)
    r.step(steps)
    out = r.download(p)
    r.close()
    return out


def same_bits(a, b, what=""):
    for k, v in a.items():
        assert np.array_equal(np.asarray(v).view(np.uint8), np.asarray(b[k]).view(np.uint8)), (what, k)


@pytest.mark.parametrize("case", golden_cases())
def test_deterministic_mode_matches_reference(case, gpu_lib):
    meta, g = load_golden(case)
    m = model_for(meta)
    if m.options.get("xpic_order", 0) > 1:
        pytest.skip("XPIC/FMPM of order > 1 runs with atomic node sums only (refused with UNSUPPORTED)")
    v = view_for(run(m, meta["steps"], p2g=DET), m)
    tol = contact_tolerance(case, m, TOL)
    for k in ("pos", "vel", "stress", "strain"):
        assert rel_l2(v[k], g["final_" + k]) <= tol[k], (k, rel_l2(v[k], g["final_" + k]), tol[k])
    if tol["vel"] == TOL:
        assert np.array_equal(v["elem"], g["final_elem"])


MODELS = {
    "taylor3d_ugimp": lambda model: model.taylor_3d(radius=1.5, length=3.0, cell=0.5, steps=30),
    "cantilever_linear_usl": lambda model: model.cantilever_2d(nx=30, ny=6, steps=40, gimp="Classic",
                                                               method=model.USL),
    "contact3d_cpdi": lambda model: model.contact_3d(plate=(8, 8, 3), block=(3, 3, 2), block_x0=1.0, block_y0=1.0,
                                                     steps=20),
    "contact2d_usf": lambda model: model.contact_2d(plate=(16, 4), block=(5, 3), steps=30, method=model.USF),
}


@pytest.mark.parametrize("name", sorted(MODELS))
@pytest.mark.parametrize("precision", [0, 1])
def test_same_bits_for_any_particle_order_and_sort_interval(name, precision, gpu_lib):
    """Two runs, the particles of the second in a shuffled order and sorted
    on another schedule: every particle ends with the same bits."""
    from nairn_gb300 import model, abi
    m = MODELS[name](model)
    steps = m.nsteps
    a = run(m, steps, p2g=DET, precision=precision, sort_interval=1)
    again = run(m, steps, p2g=DET, precision=precision, sort_interval=1)
    same_bits(a, again, "rerun")
    perm = np.random.default_rng(7).permutation(m.n)
    shuffled = {k: np.ascontiguousarray(v[perm]) for k, v in abi.copy_particles(m.particles).items()}
    b = run(m, steps, particles=shuffled, p2g=DET, precision=precision, sort_interval=3)
    same_bits({k: v[perm] for k, v in a.items()}, b, "shuffled")


@pytest.mark.parametrize("precision,tol", [(0, TOL), (1, TOL_MIXED)])
def test_deterministic_contact_cpdi_against_oracle(precision, tol, gpu_lib):
    import oracle_lib
    from nairn_gb300 import model, abi
    m = model.contact_3d(plate=(8, 8, 3), block=(3, 3, 2), block_x0=1.0, block_y0=1.5, steps=25, friction=0.3)
    ref = abi.copy_particles(m.particles)
    oracle_lib.run(m, ref, m.nsteps, nthreads=4)
    out = run(m, m.nsteps, p2g=DET, precision=precision)
    for k in ("x", "y", "z", "vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "syz", "sxz", "pressure"):
        assert rel_l2(out[k], ref[k]) <= tol, (k, rel_l2(out[k], ref[k]))


def test_nan_velocity_reports_range(gpu_lib):
    """A NaN reaching a deterministic node sum stops the step with RANGE (or
    NaN) instead of a silent wrong sum."""
    from nairn_gb300 import model, abi
    from nairn_gb300.gpu import GpuRun, GpuError
    m = model.cantilever_2d(nx=20, ny=4, steps=5)
    p = abi.copy_particles(m.particles)
    p["vx"][3] = np.nan
    r = GpuRun(m, p2g=DET)
    r.upload(p)
    with pytest.raises(GpuError, match="RANGE|NAN"):
        r.step(5)
    r.close()


@pytest.mark.parametrize("name", ["contact3d_cpdi", "taylor3d_ugimp", "contact2d_usf"])
@pytest.mark.parametrize("precision", [0, 1])
def test_resume_from_a_snapshot_is_exact(name, precision, gpu_lib):
    """Checkpoint and resume: a run stopped after k steps, downloaded to the
    host (the complete particle state), uploaded into a fresh context and
    continued from time k dt ends with the same bits as the run taken in one
    go.  The device keeps no particle state the snapshot lacks."""
    from nairn_gb300 import model
    from nairn_gb300.gpu import GpuRun
    m = MODELS[name](model)
    steps, k = m.nsteps, m.nsteps // 2 + 1
    whole = run(m, steps, p2g=DET, precision=precision)
    r = GpuRun(m, p2g=DET, precision=precision)
    r.upload(m.particles)
    r.step(k)
    snap = r.download(m.particles)
    r.close()
    r = GpuRun(m, p2g=DET, precision=precision)
    r.upload(snap)
    r.t = k * m.options["timestep"]
    r.step(steps - k)
    same_bits(whole, r.download(m.particles), "resumed")
    r.close()


def test_contiguous_host_columns_move_the_same_state(gpu_lib):
    """Host columns kept in one block in the library's column order (moved
    with one copy per direction) give the same bits as separate arrays."""
    from nairn_gb300 import model, abi
    from nairn_gb300.gpu import GpuRun
    m = MODELS["contact3d_cpdi"](model)
    a = run(m, 8, p2g=DET)
    host, block = abi.contiguous_particles(m.particles)
    r = GpuRun(m, p2g=DET)
    r.upload(host)
    r.step(8)
    out, _ = abi.contiguous_particles(m.particles)
    r.download_into(out)
    r.close()
    same_bits(a, out, "contiguous")
