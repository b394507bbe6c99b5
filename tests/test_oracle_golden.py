"""The CPU oracle against golden vectors produced by the reference NairnMPM."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, model_for, rel_l2, view_for


@pytest.mark.parametrize("case", golden_cases())
def test_model_builder_matches_reference_setup(case):
    """Grid, particle generation and mass reproduce the reference's t=0 archive exactly."""
    meta, g = load_golden(case)
    m = model_for(meta)
    dim = 3 if meta["three_d"] else 2
    pos = np.stack([m.particles[k] for k in ("x", "y", "z")[:dim]], 1)
    vel = np.stack([m.particles[k] for k in ("vx", "vy", "vz")[:dim]], 1)
    assert pos.shape == g["init_pos"].shape
    assert np.array_equal(pos, g["init_pos"])
    assert np.array_equal(vel, g["init_vel"])
    assert np.array_equal(m.particles["mass"], g["init_mass"])
    assert np.array_equal(m.particles["elem"] + 1, g["init_elem"])


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_matches_reference(case):
    """The FP64 restatement reproduces the reference's final state (bit-exact in
    practice; within 1e-12 with XPIC/FMPM of order > 1, whose double loop over
    each particle's nodes may add in another order, and with regression
    normals, whose exponentials and sums may round differently)."""
    import oracle_lib
    meta, g = load_golden(case)
    m = model_for(meta)
    p = {k: np.array(v, copy=True) for k, v in m.particles.items()}
    oracle_lib.run(m, p, meta["steps"], nthreads=1)
    v = view_for(p, m)
    lr = m.extra and m.extra.get("contact") and m.extra["contact"]["normals"] >= 5
    tol = 1e-12 if m.options.get("xpic_order", 0) > 1 or lr else 1e-13
    for k in ("pos", "vel", "stress", "strain"):
        assert rel_l2(v[k], g["final_" + k]) <= tol, (k, rel_l2(v[k], g["final_" + k]))
    if g["final_hist1"].any():
        assert rel_l2(v["hist1"], g["final_hist1"]) <= tol
        assert rel_l2(v["plastic"], g["final_plastic"]) <= tol
    assert np.array_equal(v["elem"], g["final_elem"])


def test_oracle_threads_agree():
    """OpenMP particle loops change only the summation order."""
    import oracle_lib
    meta, g = load_golden("taylor3d_ugimp_usavg")
    m = model_for(meta)
    a = {k: np.array(v, copy=True) for k, v in m.particles.items()}
    b = {k: np.array(v, copy=True) for k, v in m.particles.items()}
    oracle_lib.run(m, a, 10, nthreads=1)
    oracle_lib.run(m, b, 10, nthreads=4)
    for k in ("x", "y", "z", "vz", "szz"):
        assert rel_l2(b[k], a[k]) <= 1e-12


def test_oracle_reports_left_grid():
    """A particle pushed outside the grid is reported, as ResetElementsTask does."""
    import oracle_lib
    from nairn_gb300 import model
    m = model.cantilever_2d(nx=6, ny=3, steps=5)
    p = {k: np.array(v, copy=True) for k, v in m.particles.items()}
    p["vx"][0] = -1.e9
    with pytest.raises(RuntimeError, match="LEFT_GRID"):
        oracle_lib.run(m, p, 2)


def test_oracle_cpdi_node_limit():
    """A CPDI domain touching more than 49 nodes (3D) stops the run, as
    GetCPDIFunctions throws 'Too many CPDI nodes found' (in 2D four corner
    elements touch at most 16 nodes, the 2D limit)."""
    import oracle_lib
    from nairn_gb300 import model
    m = model.taylor_3d(radius=1.0, length=2.0, cell=0.5, steps=3, gimp="lCPDI")
    p = {k: np.array(v, copy=True) for k, v in m.particles.items()}
    # F = 6 I: the eight corners fall in eight separate cells, 64 nodes > 49
    p["exx"][5] = p["eyy"][5] = p["ezz"][5] = 5.0
    with pytest.raises(RuntimeError, match="CPDI_NODES"):
        oracle_lib.run(m, p, 1)


def test_regression_contact_is_chaotic_and_gradient_contact_is_not():
    """With regression normals the contact decision comes from point-cloud
    supports near zero separation: a 1e-9 perturbation of the initial
    velocities moves the reference's result by far more than 1e-9 (which is
    why the mixed mode is held there to the reference's own sensitivity),
    while with volume-gradient normals the response stays linear."""
    import oracle_lib
    from nairn_gb300 import abi

    def moved(case):
        meta, g = load_golden(case)
        m = model_for(meta)
        outs = []
        for eps in (0., 1e-9):
            p = abi.copy_particles(m.particles)
            rng = np.random.default_rng(1)
            for k in ("vx", "vy"):
                p[k] = p[k] * (1. + eps * rng.standard_normal(p[k].shape))
            oracle_lib.run(m, p, meta["steps"], nthreads=4)
            outs.append(view_for(p, m)["vel"])
        return rel_l2(outs[1], outs[0])

    assert moved("contact2d_fric_logreg") > 1e-4
    assert moved("contact2d_fric_avgg") < 1e-7


def test_xpic_and_fmpm_change_the_result():
    """The PeriodicXPIC goldens are not FLIP runs: the same problem with FLIP
    on every step ends far from them (so their parity tests test XPIC/FMPM)."""
    import oracle_lib
    for case in [c for c in golden_cases() if load_golden(c)[0]["kwargs"].get("xpic")]:
        meta, g = load_golden(case)
        kw = {k: v for k, v in meta["kwargs"].items() if k != "xpic"}
        m = model_for(dict(meta, kwargs=kw))
        p = {k: np.array(v, copy=True) for k, v in m.particles.items()}
        oracle_lib.run(m, p, meta["steps"], nthreads=1)
        assert rel_l2(view_for(p, m)["vel"], g["final_vel"]) > 0.1, case


def test_b2spline_goldens_are_not_ugimp_runs():
    """The B2SPLINE goldens are quadratic B-spline runs: the same problems
    with uGIMP end far from them (so their parity tests test B-splines)."""
    import oracle_lib
    for case in [c for c in golden_cases() if load_golden(c)[0]["kwargs"].get("gimp") == "B2SPLINE"]:
        meta, g = load_golden(case)
        m = model_for(dict(meta, kwargs=dict(meta["kwargs"], gimp="uGIMP")))
        p = {k: np.array(v, copy=True) for k, v in m.particles.items()}
        oracle_lib.run(m, p, meta["steps"], nthreads=1)
        assert rel_l2(view_for(p, m)["stress"], g["final_stress"]) > 1e-3, case


def test_oracle_rigid_material_options():
    """Rigid contact materials need multimaterial contact and are refused with
    regression normals, as on the device; the rigid particles keep their
    velocity and move by it, and the golden cases exercise the contact (the
    plate under the indenter moves)."""
    import oracle_lib
    from nairn_gb300 import abi, model
    m = model.rigid_contact_2d(steps=5)
    rigid = m.particles["mat"] == 1
    p = abi.copy_particles(m.particles)
    oracle_lib.run(m, p, 60, nthreads=1)
    dt = m.options["timestep"]
    assert np.array_equal(p["vy"][rigid], m.particles["vy"][rigid])
    assert np.allclose(p["y"][rigid], m.particles["y"][rigid] + 60 * dt * m.particles["vy"][rigid], rtol=0, atol=1e-12)
    assert np.abs(p["vy"][~rigid]).max() > 100.
    bad = abi.copy_particles(m.particles)
    ct = abi.contact_struct(m)
    ct.normals = 6
    with pytest.raises(RuntimeError, match="rigid"):
        oracle_lib.run(m, bad, 1, nthreads=1, contact=ct)
    ct.enabled = 0
    with pytest.raises(RuntimeError):
        oracle_lib.run(m, bad, 1, nthreads=1, contact=ct)
