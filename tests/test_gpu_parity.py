"""GPU path against the reference's golden vectors and the CPU oracle (FP64 mode)."""
import numpy as np
import pytest

from conftest import (contact_tolerance, golden_cases, load_golden, model_for, regression_sensitivity, rel_l2,
                      view_for)

pytestmark = pytest.mark.gpu

TOL = 1e-10  # relative L2, all-FP64 GPU mode vs the reference's FP64 path


def gpu_run(m, steps, **kw):
    from nairn_gb300.gpu import GpuRun
    r = GpuRun(m, **kw)
    r.upload(m.particles)
    r.step(steps)
    out = r.download(m.particles)
    r.close()
    return out


@pytest.mark.parametrize("case", golden_cases())
def test_gpu_matches_reference(case, gpu_lib):
    meta, g = load_golden(case)
    m = model_for(meta)
    out = gpu_run(m, meta["steps"])
    v = view_for(out, m)
    tol = contact_tolerance(case, m, TOL)
    for k in ("pos", "vel", "stress", "strain"):
        assert rel_l2(v[k], g["final_" + k]) <= tol[k], (k, rel_l2(v[k], g["final_" + k]), tol[k])
    if g["final_hist1"].any():
        assert rel_l2(v["hist1"], g["final_hist1"]) <= tol["hist1"]
    # cell indexing is bit-exact
    assert np.array_equal(v["elem"], g["final_elem"])


@pytest.mark.parametrize("sort_interval", [0, 1, 7])
def test_sort_interval_does_not_change_results(sort_interval, gpu_lib):
    import oracle_lib
    from nairn_gb300 import model, abi
    m = model.taylor_3d(radius=1.5, length=3.0, cell=0.5, steps=40)
    ref = abi.copy_particles(m.particles)
    oracle_lib.run(m, ref, m.nsteps)
    out = gpu_run(m, m.nsteps, sort_interval=sort_interval)
    for k in ("x", "y", "z", "vx", "vz", "szz", "sxy", "hist0"):
        assert rel_l2(out[k], ref[k]) <= TOL, k
    assert np.array_equal(out["elem"], ref["elem"])


def test_larger_2d_against_oracle(gpu_lib):
    import oracle_lib
    from nairn_gb300 import model, abi
    m = model.cantilever_2d(nx=100, ny=20, steps=200)
    ref = abi.copy_particles(m.particles)
    oracle_lib.run(m, ref, m.nsteps, nthreads=4)
    out = gpu_run(m, m.nsteps)
    for k in ("x", "y", "vx", "vy", "sxx", "syy", "sxy", "szz"):
        assert rel_l2(out[k], ref[k]) <= TOL, k


def test_left_grid_is_reported(gpu_lib):
    from nairn_gb300 import model
    from nairn_gb300.gpu import GpuRun, GpuError
    m = model.cantilever_2d(nx=6, ny=3, steps=5)
    p = {k: np.array(v, copy=True) for k, v in m.particles.items()}
    p["vx"][0] = -1.e9
    r = GpuRun(m)
    r.upload(p)
    with pytest.raises(GpuError, match="LEFT_GRID"):
        r.step(2)
    r.close()


@pytest.mark.parametrize("n,nelems", [(1, 1), (1000, 37), (70000, 570000), (300001, 1 << 20)])
def test_cell_sort_is_a_stable_argsort(n, nelems, gpu_lib):
    """mpmgpu_sort_by_cell is bit-for-bit numpy's stable argsort."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n)
    # many repeated keys, as particles share cells
    keys = rng.integers(0, nelems, size=n, dtype=np.int32)
    if n > 10:
        keys[: n // 3] = keys[n // 3]
    d_keys = torch.from_numpy(keys).cuda()
    d_perm = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = gpu_lib.mpmgpu_sort_by_cell(C.c_void_p(d_keys.data_ptr()), n, nelems, C.c_void_p(d_perm.data_ptr()), None)
    assert st == 0
    assert np.array_equal(d_perm.cpu().numpy(), np.argsort(keys, kind="stable").astype(np.int32))


TOL_MIXED = 1e-5  # relative L2, FP32 transfers + FP64 constitutive vs the reference's FP64 path


@pytest.mark.parametrize("case", golden_cases())
def test_mixed_precision_matches_reference(case, gpu_lib):
    """Every golden case within 1e-5 -- except with regression normals, whose
    runs are chaotic (see regression_sensitivity): there the mixed result may
    differ from the reference by at most twice what a 1e-9 perturbation of the
    input moves the reference itself."""
    meta, g = load_golden(case)
    m = model_for(meta)
    out = gpu_run(m, meta["steps"], precision=1)
    v = view_for(out, m)
    chaotic = m.extra and m.extra.get("contact") and m.extra["contact"]["normals"] >= 5
    sens = regression_sensitivity(m, meta["steps"]) if chaotic else {}
    ctol = contact_tolerance(case, m, TOL_MIXED)
    chaotic = chaotic or ctol["vel"] > TOL_MIXED
    for k in ("pos", "vel", "stress", "strain"):
        tol = max(TOL_MIXED, 2. * sens[k]) if k in sens else ctol[k]
        assert rel_l2(v[k], g["final_" + k]) <= tol, (k, rel_l2(v[k], g["final_" + k]), tol)
    if not chaotic:
        assert np.array_equal(v["elem"], g["final_elem"])


def test_mixed_precision_taylor_against_oracle(gpu_lib):
    """A longer 3D plastic run: stresses stay within 1e-5 of the FP64 path."""
    import oracle_lib
    from nairn_gb300 import model, abi
    m = model.taylor_3d(radius=2.0, length=5.0, cell=0.25, steps=300)
    ref = abi.copy_particles(m.particles)
    oracle_lib.run(m, ref, m.nsteps, nthreads=8)
    out = gpu_run(m, m.nsteps, precision=1)
    for k in ("x", "y", "z", "vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "syz", "sxz", "hist0"):
        assert rel_l2(out[k], ref[k]) <= TOL_MIXED, (k, rel_l2(out[k], ref[k]))


@pytest.mark.parametrize("precision,tol", [(0, TOL), (1, TOL_MIXED)])
def test_neohookean_3d_against_oracle(precision, tol, gpu_lib):
    """Neo-Hookean rubber bar impact (large strains), FP64 and mixed modes."""
    import oracle_lib
    from nairn_gb300 import model, abi
    m = model.taylor_3d(radius=2.0, length=5.0, cell=0.25, steps=200, mat_type=28, G=10., K=50., rho=1.1,
                        v0=-30000.)
    ref = abi.copy_particles(m.particles)
    oracle_lib.run(m, ref, m.nsteps, nthreads=8)
    out = gpu_run(m, m.nsteps, precision=precision)
    for k in ("x", "y", "z", "vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "syz", "sxz", "pressure", "pxx", "pzz",
              "hist0"):
        assert rel_l2(out[k], ref[k]) <= tol, (k, rel_l2(out[k], ref[k]))


@pytest.mark.parametrize("precision,tol", [(0, TOL), (1, TOL_MIXED)])
def test_cpdi_3d_neohookean_against_oracle(precision, tol, gpu_lib):
    """lCPDI shape functions on a larger 3D Neo-Hookean impact, FP64 and mixed."""
    import oracle_lib
    from nairn_gb300 import model, abi
    m = model.taylor_3d(radius=2.0, length=4.0, cell=0.25, steps=120, mat_type=28, G=10., K=50., rho=1.1,
                        v0=-30000., gimp="lCPDI")
    ref = abi.copy_particles(m.particles)
    oracle_lib.run(m, ref, m.nsteps, nthreads=8)
    out = gpu_run(m, m.nsteps, precision=precision)
    for k in ("x", "y", "z", "vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "syz", "sxz", "pressure", "hist0"):
        assert rel_l2(out[k], ref[k]) <= tol, (k, rel_l2(out[k], ref[k]))
    assert np.array_equal(out["elem"], ref["elem"])


def test_cpdi_node_limit_is_reported(gpu_lib):
    from nairn_gb300 import model
    from nairn_gb300.gpu import GpuRun, GpuError
    m = model.taylor_3d(radius=1.0, length=2.0, cell=0.5, steps=3, gimp="lCPDI")
    p = {k: np.array(v, copy=True) for k, v in m.particles.items()}
    p["exx"][5] = p["eyy"][5] = p["ezz"][5] = 5.0  # eight corner cells apart: 64 nodes > 49
    r = GpuRun(m)
    r.upload(p)
    with pytest.raises(GpuError, match="CPDI_NODES"):
        r.step(1)
    r.close()


def test_sort_autotune_keeps_results(gpu_lib):
    """The single-run sort autotuner takes real steps (a multiple of 32) and
    leaves the results those of the oracle over the same step count."""
    import oracle_lib
    from nairn_gb300 import model, abi
    from nairn_gb300.gpu import GpuRun
    m = model.taylor_3d(radius=1.5, length=3.0, cell=0.5, steps=40)
    r = GpuRun(m, precision=0)
    r.upload(m.particles)
    r.step(4)
    si, ms = r.autotune_sort(16)
    assert si in (1, 2, 4, 8) and ms > 0.
    r.step(4)
    out = r.download(m.particles)
    r.close()
    ref = abi.copy_particles(m.particles)
    oracle_lib.run(m, ref, 4 + 64 + 4)
    for k in ("x", "y", "z", "vx", "vz", "szz", "sxy", "hist0"):
        assert rel_l2(out[k], ref[k]) <= TOL, k


def test_xpic_schedule_follows_the_step_time(gpu_lib):
    """The PeriodicXPIC schedule counts steps from the time each call starts
    at: a run split into calls of odd lengths meets the reference's golden
    (FMPM(2) on every second step, USL)."""
    from nairn_gb300.gpu import GpuRun
    meta, g = load_golden("cant2d_fmpm2_usl_every2")
    m = model_for(meta)
    r = GpuRun(m)
    r.upload(m.particles)
    for n in (7, 12, meta["steps"] - 19):
        r.step(n)
    v = view_for(r.download(m.particles), m)
    r.close()
    for k in ("pos", "vel", "stress", "strain"):
        assert rel_l2(v[k], g["final_" + k]) <= TOL, (k, rel_l2(v[k], g["final_" + k]))


def test_xpic_refusals(gpu_lib):
    """XPIC/FMPM of order > 1 is refused with rigid contact materials and with
    deterministic node sums; a bad period is invalid.  (With multimaterial
    contact it runs: the XPIC contact goldens.)"""
    from nairn_gb300 import model
    from nairn_gb300.gpu import GpuRun, GpuError
    c = model.rigid_contact_2d(steps=5)
    c.options.update(xpic_order=2, xpic_fmpm=0, xpic_period=1)
    r = GpuRun(c)
    r.upload(c.particles)
    with pytest.raises(GpuError, match="UNSUPPORTED"):
        r.step(1)
    r.close()
    m = model.cantilever_2d(nx=10, ny=4, steps=5, xpic=(2, 1, 1))
    with pytest.raises(GpuError, match="UNSUPPORTED"):
        GpuRun(m, p2g=1)
    m.options["xpic_period"] = 0
    with pytest.raises(GpuError, match="INVALID"):
        GpuRun(m)


@pytest.mark.gpu
def test_driver_allocated_host_block_round_trip(gpu_lib):
    """Particle columns kept in page-locked memory the driver allocated
    (mpmgpu_host_alloc) upload and download like any host columns: with
    deterministic node sums the run gives the same bits as one from ordinary
    numpy arrays."""
    from nairn_gb300 import abi, model
    from nairn_gb300.gpu import GpuRun, HostBlock
    m = model.taylor_3d(radius=1.0, length=2.0, cell=0.5, steps=3)
    hb = HostBlock((len(abi.DEVICE_COLUMNS), m.n))
    host, _ = abi.contiguous_particles(m.particles, hb.array)
    r = GpuRun(m, p2g=1)
    r.upload(host)
    r.step(3)
    r.download_into(host)
    r.close()
    s = GpuRun(m, p2g=1)
    s.upload(m.particles)
    s.step(3)
    ref = s.download(m.particles)
    s.close()
    for k in abi.DEVICE_COLUMNS:
        assert np.array_equal(host[k], ref[k]), k
    host = None
    hb.close()
