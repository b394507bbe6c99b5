"""Batched runs (mpmgpu_batch_*): every run of a batch gives the result it
gives alone -- against the CPU oracle at the FP64 tolerance, and in the mixed
mode at the mixed tolerance -- whatever else shares the batch, including runs
that finish early, leave, fail or arrive later."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-10
TOL_MIXED = 1e-5
FIELDS = ("x", "y", "vx", "vy", "sxx", "syy", "sxy", "szz", "exx", "exy", "hist0", "work")


def small_models(count=6, seed=11, steps=40, nmin=300, nmax=3000):
    from nairn_gb300 import model
    return model.batch_models(count, seed=seed, nmin=nmin, nmax=nmax, steps=steps)


def oracle(m, steps):
    import oracle_lib
    from nairn_gb300 import abi
    ref = abi.copy_particles(m.particles)
    oracle_lib.run(m, ref, steps, nthreads=4)
    return ref


def assert_close(out, ref, tol, what=""):
    for k in FIELDS:
        if np.abs(ref[k]).max() == 0. and np.abs(out[k]).max() == 0.:
            continue
        e = rel_l2(out[k], ref[k])
        assert e <= tol, (what, k, e)
    assert np.array_equal(out["elem"], ref["elem"]), what


@pytest.mark.parametrize("precision,tol", [(0, TOL), (1, TOL_MIXED)])
def test_batch_runs_match_oracle(precision, tol, gpu_lib):
    from nairn_gb300.gpu import GpuBatch
    from nairn_gb300 import abi
    ms = small_models()
    b = GpuBatch.for_models(ms, precision=precision)
    ids = [b.add(m) for m in ms]
    b.step(ms[0].nsteps)
    for rid, m in zip(ids, ms):
        st, done = b.state(rid)
        assert (st, done) == (abi.RUN_FINISHED, m.nsteps)
        assert_close(b.download(rid), oracle(m, m.nsteps), tol, m.name)
    info = b.info()
    assert info["runs"] == len(ms) and info["running"] == 0
    b.close()


def test_batch_matches_single_run_path(gpu_lib):
    """The batch and the single-run context compute the same step."""
    from nairn_gb300.gpu import GpuBatch, GpuRun
    ms = small_models(count=3, seed=5, steps=25)
    b = GpuBatch.for_models(ms)
    ids = [b.add(m) for m in ms]
    b.step(25)
    for rid, m in zip(ids, ms):
        r = GpuRun(m)
        r.upload(m.particles)
        r.step(25)
        alone = r.download(m.particles)
        r.close()
        assert_close(b.download(rid), alone, TOL, m.name)
    b.close()


def test_runs_stop_at_their_own_step_counts(gpu_lib):
    from nairn_gb300.gpu import GpuBatch
    from nairn_gb300 import abi
    ms = small_models(count=4, seed=3, steps=30)
    counts = [7, 30, 18, 1]
    b = GpuBatch.for_models(ms)
    ids = [b.add(m, nsteps=c) for m, c in zip(ms, counts)]
    b.step(10)
    assert [b.state(r) for r in ids] == [(abi.RUN_FINISHED, 7), (abi.RUN_RUNNING, 10), (abi.RUN_RUNNING, 10),
                                         (abi.RUN_FINISHED, 1)]
    b.step(25)
    for rid, m, c in zip(ids, ms, counts):
        assert b.state(rid) == (abi.RUN_FINISHED, c)
        assert_close(b.download(rid), oracle(m, c), TOL, m.name)
    b.close()


def test_removal_compaction_and_late_admission(gpu_lib):
    """A run removed mid-way leaves the others untouched; its slots are
    compacted away and a run admitted later starts from its own t = 0."""
    from nairn_gb300.gpu import GpuBatch
    ms = small_models(count=5, seed=9, steps=30)
    first, late = ms[:4], ms[4]
    b = GpuBatch.for_models(ms)
    ids = [b.add(m) for m in first]
    b.step(12)
    mid = b.remove(ids[1])
    assert_close(mid, oracle(first[1], 12), TOL, "removed run")
    rid_late = b.add(late)
    b.step(30)
    info = b.info()
    assert info["particles_dead"] == 0
    assert info["particles_used"] == sum(m.n for m in ms) - first[1].n
    for k in (0, 2, 3):
        assert_close(b.download(ids[k]), oracle(first[k], 30), TOL, first[k].name)
    assert_close(b.download(rid_late), oracle(late, 30), TOL, "late run")
    b.close()


def test_a_failing_run_is_confined(gpu_lib):
    """A run whose particle leaves its grid reports LEFT_GRID and stops; the
    other runs of the batch are unaffected."""
    from nairn_gb300.gpu import GpuBatch
    from nairn_gb300 import abi
    ms = small_models(count=3, seed=21, steps=20)
    bad = {k: np.array(v, copy=True) for k, v in ms[1].particles.items()}
    bad["vx"][0] = -1.e9
    b = GpuBatch.for_models(ms)
    ids = [b.add(ms[0]), b.add(ms[1], particles=bad), b.add(ms[2])]
    b.step(20)
    st, done = b.state(ids[1])
    assert st == -6 and done < 20  # -MPMGPU_ERR_LEFT_GRID
    for k in (0, 2):
        assert b.state(ids[k]) == (abi.RUN_FINISHED, 20)
        assert_close(b.download(ids[k]), oracle(ms[k], 20), TOL, ms[k].name)
    b.close()


def test_admission_rejects_bad_indices_and_full_batch(gpu_lib):
    from nairn_gb300.gpu import GpuBatch, GpuError
    ms = small_models(count=2, seed=4, steps=5)
    b = GpuBatch.for_models(ms[:1])
    bad = {k: np.array(v, copy=True) for k, v in ms[0].particles.items()}
    bad["elem"][3] = ms[0].grid.nelems
    with pytest.raises(GpuError, match="INVALID"):
        b.add(ms[0], particles=bad)
    rid = b.add(ms[0])  # the rejected run's slots are reused
    with pytest.raises(GpuError, match="BUSY"):
        b.add(ms[1])
    b.step(5)
    assert_close(b.download(rid), oracle(ms[0], 5), TOL, "after rejection")
    b.close()


@pytest.mark.parametrize("sort_interval", [0, 3])
def test_sort_interval_and_block_do_not_change_results(sort_interval, gpu_lib):
    from nairn_gb300.gpu import GpuBatch
    ms = small_models(count=3, seed=13, steps=20)
    b = GpuBatch.for_models(ms, sort_interval=sort_interval, block=128)
    ids = [b.add(m) for m in ms]
    b.step(20)
    for rid, m in zip(ids, ms):
        assert_close(b.download(rid), oracle(m, 20), TOL, m.name)
    b.close()


def test_autotune_steps_count_and_results_hold(gpu_lib):
    from nairn_gb300.gpu import GpuBatch
    ms = small_models(count=4, seed=17, steps=200)
    b = GpuBatch.for_models(ms, precision=1)
    ids = [b.add(m) for m in ms]
    blk, si, ms_step = b.autotune(trial_steps=8)
    assert blk in (128, 256) and si in (1, 2, 4, 8) and ms_step > 0.
    done = b.state(ids[0])[1]
    assert done == 8 * (8 + 1)  # 8 candidates x (1 capture step + 8 timed steps)
    b.step(200 - done)
    for rid, m in zip(ids, ms):
        assert_close(b.download(rid), oracle(m, 200), TOL_MIXED, m.name)
    b.close()


FIELDS_3D = ("x", "y", "z", "vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "syz", "sxz", "pressure", "hist0")


def assert_close_3d(out, ref, tol, what=""):
    for k in FIELDS_3D:
        if np.abs(ref[k]).max() == 0. and np.abs(out[k]).max() == 0.:
            continue
        e = rel_l2(out[k], ref[k])
        assert e <= tol, (what, k, e)
    assert np.array_equal(out["elem"], ref["elem"]), what


@pytest.mark.parametrize("precision,tol", [(0, TOL), (1, TOL_MIXED)])
def test_batched_contact_cpdi_runs_match_oracle(precision, tol, gpu_lib):
    """3D two-material contact runs (lCPDI, Neo-Hookean on elastic, Coulomb
    friction) of uneven sizes in one batch, each against the oracle."""
    from nairn_gb300.gpu import GpuBatch
    from nairn_gb300 import model, abi
    ms = model.contact_models(4, seed=5, nmin=1500, nmax=8000, steps=25)
    b = GpuBatch.for_models(ms, precision=precision)
    assert b.opts.max_fields == 2
    ids = [b.add(m) for m in ms]
    b.step(25)
    for rid, m in zip(ids, ms):
        assert b.state(rid) == (abi.RUN_FINISHED, 25)
        assert_close_3d(b.download(rid), oracle(m, 25), tol, m.name)
    b.close()


def test_contact_and_single_field_runs_share_a_batch(gpu_lib):
    """A single-field run (no contact) in a two-field batch computes what it
    computes alone; contact runs beside it are unaffected, including ones
    with other normals and friction laws."""
    from nairn_gb300.gpu import GpuBatch
    from nairn_gb300 import model
    plain = model.block_3d(ncx=6, ncy=5, ncz=4, steps=20, gimp="lCPDI")
    c1 = model.contact_3d(plate=(8, 8, 3), block=(3, 3, 2), block_x0=1.0, block_y0=1.0, steps=20, normals=0,
                          friction=0.)
    c2 = model.contact_3d(plate=(7, 9, 3), block=(3, 3, 2), block_x0=1.5, block_y0=0.5, steps=20, normals=1,
                          friction=-1.)
    ms = [c1, plain, c2]
    b = GpuBatch.for_models(ms)
    ids = [b.add(m) for m in ms]
    b.step(20)
    for rid, m in zip(ids, ms):
        assert_close_3d(b.download(rid), oracle(m, 20), TOL, m.name)
    b.close()


def test_batched_contact_2d_ugimp(gpu_lib):
    from nairn_gb300.gpu import GpuBatch
    from nairn_gb300 import model
    ms = [model.contact_2d(plate=(16, 4), block=(5, 3), block_x0=3.0 + k, friction=0.3 * k, normals=k % 3,
                           steps=30) for k in range(3)]
    b = GpuBatch.for_models(ms, precision=1)
    ids = [b.add(m) for m in ms]
    b.step(30)
    for rid, m in zip(ids, ms):
        assert_close(b.download(rid), oracle(m, 30), TOL_MIXED, m.name)
    b.close()


def test_contact_run_needs_a_multifield_batch(gpu_lib):
    from nairn_gb300.gpu import GpuBatch, GpuError
    from nairn_gb300 import model
    c = model.contact_3d(plate=(6, 6, 3), block=(2, 2, 2), steps=5)
    plain = model.block_3d(ncx=4, ncy=4, ncz=4, steps=5, gimp="lCPDI")
    b = GpuBatch.for_models([c, plain], max_fields=1)
    with pytest.raises(GpuError, match="INVALID"):
        b.add(c)
    b.close()


REGRESSION_CASES = ("contact2d_fric_logreg", "contact2d_fric_logreg_cpdi", "contact2d_stick_linreg_usl",
                    "contact3d_fric_logreg_cpdi", "contact3d_fric_logreg_ugimp_usf")


def with_normals(m, normals):
    """The same problem with another contact normal method."""
    import copy
    o = copy.deepcopy(m)
    o.extra["contact"]["normals"] = normals
    o.name = f"{m.name}_normals{normals}"
    return o


@pytest.mark.parametrize("case", REGRESSION_CASES)
def test_batched_regression_normals_match_reference(case, gpu_lib):
    """A regression-normal run (linear 5, logistic 6) shares a batch with the
    same problem under maximum-volume-gradient normals: the first matches the
    reference's golden result within the FP64 tolerance, the second the
    oracle."""
    from conftest import load_golden, model_for, view_for
    from nairn_gb300.gpu import GpuBatch
    from nairn_gb300 import abi
    meta, g = load_golden(case)
    m = model_for(meta)
    other = with_normals(m, 0)
    steps = meta["steps"]
    b = GpuBatch.for_models([other, m])
    assert b.opts.lr_links == (64 if m.grid.dim == 3 else 16)
    ids = [b.add(other), b.add(m)]
    b.step(steps)
    assert b.state(ids[1]) == (abi.RUN_FINISHED, steps)
    v = view_for(b.download(ids[1]), m)
    for k in ("pos", "vel", "stress", "strain"):
        assert rel_l2(v[k], g["final_" + k]) <= TOL, (k, rel_l2(v[k], g["final_" + k]))
    assert np.array_equal(v["elem"], g["final_elem"])
    out, ref = b.download(ids[0]), oracle(other, steps)
    (assert_close_3d if m.grid.dim == 3 else assert_close)(out, ref, TOL, other.name)
    b.close()


def test_batched_logistic_normals_mixed(gpu_lib):
    """Mixed precision with logistic normals in a batch: within twice the
    reference's own sensitivity to a 1e-9 perturbation (these runs are
    chaotic), as the single-run mixed path."""
    from conftest import load_golden, model_for, regression_sensitivity, view_for
    from nairn_gb300.gpu import GpuBatch
    meta, g = load_golden("contact3d_fric_logreg_cpdi")
    m = model_for(meta)
    b = GpuBatch.for_models([m], precision=1)
    rid = b.add(m)
    b.step(meta["steps"])
    v = view_for(b.download(rid), m)
    sens = regression_sensitivity(m, meta["steps"])
    for k in ("pos", "vel", "stress", "strain"):
        tol = max(TOL_MIXED, 2. * sens[k])
        assert rel_l2(v[k], g["final_" + k]) <= tol, (k, rel_l2(v[k], g["final_" + k]), tol)
    b.close()


def test_regression_links_overflow_fails_only_that_run(gpu_lib):
    """Links beyond the batch's lr_links reserve fail the run that made them
    with RANGE; a run beside it is unaffected.  The overflowing run has its
    two materials interleaved particle by particle, so nearly every node is a
    contact node and the links far outnumber the particle slots."""
    from nairn_gb300.gpu import GpuBatch
    from nairn_gb300 import model, abi
    plain = model.block_2d(ncx=8, ncy=5, vel=(0., 1500., 0.3, 0., -700., 1.1), steps=10)  # deforming
    c = model.contact_2d(plate=(16, 4), block=(5, 3), normals=6, steps=10)
    p = abi.copy_particles(c.particles)
    p["mat"][::2] = 1 - p["mat"][::2]
    b = GpuBatch.for_models([plain, c], lr_links=1)
    ids = [b.add(plain), b.add(c, particles=p)]
    b.step(10)
    assert b.state(ids[1])[0] == -10  # -MPMGPU_ERR_RANGE
    assert b.state(ids[0]) == (abi.RUN_FINISHED, 10)
    assert_close(b.download(ids[0]), oracle(plain, 10), TOL, plain.name)
    b.close()


def test_regression_normals_need_a_link_reserve(gpu_lib):
    from nairn_gb300.gpu import GpuBatch, GpuError
    from nairn_gb300 import model
    c = model.contact_2d(plate=(16, 4), block=(5, 3), normals=5, steps=5)
    b = GpuBatch.for_models([c], lr_links=0)
    with pytest.raises(GpuError, match="INVALID"):
        b.add(c)
    b.close()


@pytest.mark.parametrize("case,precision,tol", [("cant2d_xpic2", 0, TOL), ("cant2d_fmpm2_usl_every2", 0, TOL),
                                                ("cant2d_xpic2_cpdi_every2", 0, TOL), ("cant2d_fmpm3", 1, TOL_MIXED)])
def test_batched_xpic_runs_match_reference(case, precision, tol, gpu_lib):
    """PeriodicXPIC in a batch (XPIC(k) and FMPM(k), every step or every
    second step): the golden run matches the reference; a larger run of the
    same settings admitted five steps later counts its own steps (its
    schedule starts at its admission) and matches the oracle."""
    from conftest import load_golden, model_for, view_for
    from nairn_gb300.gpu import GpuBatch
    from nairn_gb300 import model, abi
    meta, g = load_golden(case)
    m = model_for(meta)
    kw = dict(meta["kwargs"], nx=14, ny=5, steps=meta["steps"] - 5)
    late = model_for(dict(meta, kwargs=kw))
    b = GpuBatch.for_models([m, late], precision=precision)
    assert b.opts.xpic_order == m.options["xpic_order"]
    r0 = b.add(m)
    b.step(5)
    r1 = b.add(late)
    b.step(meta["steps"])
    assert b.state(r0) == (abi.RUN_FINISHED, meta["steps"])
    assert b.state(r1) == (abi.RUN_FINISHED, late.nsteps)
    v = view_for(b.download(r0), m)
    for k in ("pos", "vel", "stress", "strain"):
        assert rel_l2(v[k], g["final_" + k]) <= tol, (k, rel_l2(v[k], g["final_" + k]))
    assert_close(b.download(r1), oracle(late, late.nsteps), tol, "late")
    b.close()


@pytest.mark.parametrize("case,precision,tol", [("contact2d_xpic2_fric", 0, TOL), ("contact2d_fmpm2_fric_usl", 1, TOL_MIXED),
                                                ("contact3d_xpic2_fric_cpdi", 0, TOL)])
def test_batched_xpic_contact_runs_match_reference(case, precision, tol, gpu_lib):
    """PeriodicXPIC with multimaterial contact in a batch: the golden run
    matches the reference, and a run of another plate and block size admitted
    five steps later (its own XPIC schedule) matches the oracle."""
    from conftest import contact_tolerance, load_golden, model_for, view_for
    from nairn_gb300.gpu import GpuBatch
    from nairn_gb300 import abi
    meta, g = load_golden(case)
    m = model_for(meta)
    bigger = dict(plate=(24, 5), block=(7, 4)) if m.grid.dim == 2 else dict(plate=(14, 12, 3), block=(5, 4, 3))
    late = model_for(dict(meta, kwargs=dict(meta["kwargs"], steps=meta["steps"] - 5, **bigger)))
    b = GpuBatch.for_models([m, late], precision=precision)
    assert b.opts.xpic_order == m.options["xpic_order"]
    r0 = b.add(m)
    b.step(5)
    r1 = b.add(late)
    b.step(meta["steps"])
    assert b.state(r0) == (abi.RUN_FINISHED, meta["steps"])
    assert b.state(r1) == (abi.RUN_FINISHED, late.nsteps)
    v = view_for(b.download(r0), m)
    ctol = contact_tolerance(case, m, tol)
    for k in ("pos", "vel", "stress", "strain"):
        assert rel_l2(v[k], g["final_" + k]) <= ctol[k], (k, rel_l2(v[k], g["final_" + k]), ctol[k])
    (assert_close if m.grid.dim == 2 else assert_close_3d)(b.download(r1), oracle(late, late.nsteps), tol, "late")
    b.close()


def test_batched_xpic_refused_with_rigid_materials(gpu_lib):
    from nairn_gb300.gpu import GpuBatch, GpuError
    from nairn_gb300 import model
    c = model.rigid_contact_2d(steps=5)
    c.options.update(xpic_order=2, xpic_fmpm=0, xpic_period=1)
    b = GpuBatch.for_models([c])
    with pytest.raises(GpuError, match="UNSUPPORTED"):
        b.add(c)
    b.close()


@pytest.mark.parametrize("precision,tol", [(0, TOL), (1, TOL_MIXED)])
@pytest.mark.parametrize("case", ["rigid2d_indent_fric", "rigid3d_taylor_wall"])
def test_batched_rigid_contact_matches_reference(case, precision, tol, gpu_lib):
    """A run with a rigid contact material shares a batch with a contact run
    of deformable materials only: the first matches the reference's golden
    result, the second the oracle."""
    from conftest import contact_tolerance, load_golden, model_for, view_for
    from nairn_gb300 import abi, model
    from nairn_gb300.gpu import GpuBatch
    meta, g = load_golden(case)
    m = model_for(meta)
    steps = meta["steps"]
    if m.grid.dim == 2:
        other = model.contact_2d(steps=steps, friction=0.3, normals=2)
    else:
        other = model.contact_3d(steps=steps, friction=0.3, normals=2, gimp="uGIMP")
    b = GpuBatch.for_models([other, m], precision=precision)
    ids = [b.add(other), b.add(m)]
    b.step(steps)
    assert b.state(ids[1]) == (abi.RUN_FINISHED, steps)
    v = view_for(b.download(ids[1]), m)
    ctol = contact_tolerance(case, m, tol)
    for k in ("pos", "vel", "stress", "strain"):
        assert rel_l2(v[k], g["final_" + k]) <= ctol[k], (k, rel_l2(v[k], g["final_" + k]), ctol[k])
    out, ref = b.download(ids[0]), oracle(other, steps)
    for k in ("x", "y", "vx", "vy", "sxx", "syy", "sxy"):
        assert rel_l2(out[k], ref[k]) <= tol, (k, rel_l2(out[k], ref[k]))
    b.close()


@pytest.mark.parametrize("precision,tol", [(0, TOL), (1, TOL_MIXED)])
@pytest.mark.parametrize("case", ["contact2d_fric_qcpdi", "cant2d_qcpdi_neo_usf"])
def test_batched_qcpdi_runs_match_reference(case, precision, tol, gpu_lib):
    """qCPDI (2D, nine domain points per particle) in a batch: the golden run
    matches the reference's result, and a larger qCPDI cantilever admitted
    five steps later matches the oracle."""
    from conftest import contact_tolerance, load_golden, model_for, view_for
    from nairn_gb300 import abi, model
    from nairn_gb300.gpu import GpuBatch
    meta, g = load_golden(case)
    m = model_for(meta)
    steps = meta["steps"]
    # the batch's runs share its MPM method: the late run takes the golden run's
    late = model.cantilever_2d(nx=14, ny=5, steps=steps - 5, gimp="qCPDI", method=meta["kwargs"].get("method", 2))
    b = GpuBatch.for_models([m, late], precision=precision)
    r0 = b.add(m)
    b.step(5)
    r1 = b.add(late)
    b.step(steps)
    assert b.state(r0) == (abi.RUN_FINISHED, steps)
    assert b.state(r1) == (abi.RUN_FINISHED, late.nsteps)
    v = view_for(b.download(r0), m)
    ctol = contact_tolerance(case, m, tol)
    for k in ("pos", "vel", "stress", "strain"):
        assert rel_l2(v[k], g["final_" + k]) <= ctol[k], (k, rel_l2(v[k], g["final_" + k]), ctol[k])
    assert_close(b.download(r1), oracle(late, late.nsteps), tol, "late")
    b.close()


def test_qcpdi_refused_in_3d(gpu_lib):
    """qCPDI exists in 2D only (the reference refuses it in 3D): a 3D batch
    of that shape option is refused before any device work."""
    from nairn_gb300 import model
    from nairn_gb300.gpu import GpuBatch
    with pytest.raises(RuntimeError, match="qCPDI"):
        GpuBatch(model.THREED, model.USAVG, model.SHAPE_QCPDI, 0, max_runs=1, max_particles=1000, max_nodes=1000)
