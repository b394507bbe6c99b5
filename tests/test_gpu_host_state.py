"""Steps on particle state kept in host memory (mpmgpu_step_host): the kernels
read and write the caller's page-locked columns in place."""
import numpy as np
import pytest

from conftest import contact_tolerance, golden_cases, load_golden, model_for, rel_l2, view_for

pytestmark = pytest.mark.gpu

TOL = 1e-10  # relative L2 against the reference's FP64 path, as the device-resident path


def host_run(m, steps, chunks=1, **kw):
    """Upload (sizes the work arrays), then step the host-resident copy."""
    from nairn_gb300 import abi
    from nairn_gb300.gpu import GpuRun, HostState
    r = GpuRun(m, **kw)
    r.upload(m.particles)
    hs = HostState(m.particles)
    left = steps
    for k in range(chunks):
        s = left // (chunks - k)
        r.step_host(hs.particles, s)
        left -= s
    out = abi.copy_particles(hs.particles)
    hs.close()
    r.close()
    return out


def test_host_state_is_bit_identical_with_deterministic_sums(gpu_lib):
    """With deterministic node sums the result is independent of the particle
    order, so the host-resident step (host order, no sort) and the
    device-resident step (cell-sorted) give the same bits."""
    from nairn_gb300 import abi, model
    from nairn_gb300.gpu import GpuRun
    m = model.taylor_3d(radius=1.5, length=3.0, cell=0.5, steps=30)
    out = host_run(m, 30, chunks=3, p2g=1)
    r = GpuRun(m, p2g=1)
    r.upload(m.particles)
    r.step(30)
    ref = r.download(m.particles)
    r.close()
    for k in abi.DEVICE_COLUMNS + ["elem"]:
        assert np.array_equal(out[k], ref[k]), k


HOST_CASES = ["cant2d_ugimp_usavg", "cant2d_cpdi_neo", "cant2d_xpic2", "contact2d_fric_logreg",
              "contact2d_xpic2_fric", "contact3d_fric_cpdi", "rigid2d_indent_fric", "taylor3d_ugimp_usavg",
              "taylor3d_ugimp_usl", "taylor3d_b2spline"]


def test_host_cases_exist():
    assert set(HOST_CASES) <= set(golden_cases())


@pytest.mark.parametrize("case", HOST_CASES)
def test_host_state_matches_reference(case, gpu_lib):
    meta, g = load_golden(case)
    m = model_for(meta)
    out = host_run(m, meta["steps"], chunks=2)
    v = view_for(out, m)
    tol = contact_tolerance(case, m, TOL)
    for k in ("pos", "vel", "stress", "strain"):
        assert rel_l2(v[k], g["final_" + k]) <= tol[k], (k, rel_l2(v[k], g["final_" + k]), tol[k])
    assert np.array_equal(v["elem"], g["final_elem"])


def test_host_state_mixed_mode_matches_fp64(gpu_lib):
    from nairn_gb300 import model
    m = model.taylor_3d(radius=1.5, length=3.0, cell=0.5, steps=40)
    ref = host_run(m, 40)
    out = host_run(m, 40, precision=1)
    for k in ("x", "vz", "szz", "sxy", "hist0"):
        assert rel_l2(out[k], ref[k]) <= 1e-5, k
    assert np.array_equal(out["elem"], ref["elem"])


def test_host_state_refusals(gpu_lib):
    """Columns outside the driver's blocks, a count other than the uploaded
    one and out-of-range indices are refused before any step runs."""
    from nairn_gb300 import abi, model
    from nairn_gb300.gpu import GpuError, GpuRun, HostState
    m = model.taylor_3d(radius=1.0, length=2.0, cell=0.5, steps=3)
    r = GpuRun(m)
    with pytest.raises(GpuError, match="INVALID"):
        r.step_host(abi.copy_particles(m.particles), 1)  # nothing uploaded yet
    r.upload(m.particles)
    with pytest.raises(GpuError, match="INVALID"):
        r.step_host(abi.copy_particles(m.particles), 1)  # ordinary numpy memory
    hs = HostState(m.particles)
    before = abi.copy_particles(hs.particles)
    hs.particles["mat"][5] = 99
    with pytest.raises(GpuError, match="INVALID"):
        r.step_host(hs.particles, 1)
    hs.particles["mat"][5] = before["mat"][5]
    for k in abi.DEVICE_COLUMNS:
        assert np.array_equal(hs.particles[k], before[k]), k
    r.step_host(hs.particles, 2)
    assert not np.array_equal(hs.particles["z"], before["z"])
    hs.close()
    small = model.taylor_3d(radius=0.5, length=1.0, cell=0.5, steps=1)
    hs = HostState(small.particles)
    with pytest.raises(GpuError, match="INVALID"):
        r.step_host(hs.particles, 1)  # another particle count
    hs.close()
    r.close()
